"""The drop-in `eob` package (eob.seobnrv4phm, eob.new_Dormand_horiz, ...) on
the GPU against the reference's golden configuration-1 outputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_waveform_call_modes(torch_cuda, golden):
    from eob.seobnrv4phm import SEOBNRv4PHM
    c = golden["config1"]
    P = c["params"]
    gen = SEOBNRv4PHM(use_gpu=True, max_step=4096, imr=False)
    out = gen(P[:, 0], P[:, 1], P[:, 2], P[:, 3], np.ones(len(P)), np.zeros(len(P)), modes=[(2, 2)], fs=20.0,
              sampling_frequency=1.0 / float(c["dt"]))
    out = out.cpu().numpy()
    assert out.shape[:2] == (len(P), 1)
    assert out.shape[2] == int(c["npts"].max())
    np.testing.assert_array_equal(gen.lengths.cpu().numpy(), c["nsteps"])
    for b in range(2):
        n = int(c["npts"][b])
        hr = c[f"h_{b}"][:n]
        assert np.max(np.abs(out[b, 0, :n] - hr)) < 1e-8 * np.abs(hr).max()
        # past a binary's own end the batched call holds the value at its last knot (reference semantics:
        # sample times are clamped to the end of each trajectory, eob/seobnrv4phm.py:2339-2340)
        if n < out.shape[2]:
            tail = out[b, 0, n:]
            assert np.all(tail == tail[0])


def test_step_by_step_initial_conditions_and_trajectory(torch_cuda, golden):
    torch = torch_cuda
    from eob.seobnrv4phm import SEOBNRv4PHM, MTSUN_SI
    c = golden["config1"]
    P = c["params"][:3]
    gen = SEOBNRv4PHM(use_gpu=True, max_step=4096, imr=False)
    mt = P[:, 0] + P[:, 1]
    omega0 = 20.0 * (mt * MTSUN_SI * np.pi)
    gen.setup_class(P[:, 0] / mt, P[:, 1] / mt, P[:, 2], P[:, 3], omega0)
    r0, pphi0, pr0 = gen.get_initial_conditions(P[:, 0], P[:, 1], P[:, 2], P[:, 3], fs=20.0)
    np.testing.assert_allclose(r0.cpu().numpy(), c["ic"][:3, 0], rtol=1e-11)
    np.testing.assert_allclose(pphi0.cpu().numpy(), c["ic"][:3, 1], rtol=1e-11)
    assert np.all(np.abs(pr0.cpu().numpy()) < 2e-12)
    t, traj, num_steps = gen.run_trajectory(r0, pphi0, pr0, P[:, 0], P[:, 1], P[:, 2], P[:, 3], fs=20.0)
    np.testing.assert_array_equal(num_steps.cpu().numpy(), c["nsteps"][:3])


def test_bbh_td_strain_and_likelihood(torch_cuda, golden):
    from eob.seobnrv4phm import BBHWaveformTD
    c = golden["config1"]
    P = c["params"]
    fs_hz = 1.0 / float(c["dt"])
    N = int(c["N"])
    bbh = BBHWaveformTD(None, amp_phase_kwargs={"max_step": 4096, "imr": False})
    h = bbh(P[:2, 0], P[:2, 1], P[:2, 2], P[:2, 3], np.ones(2), np.zeros(2), sampling_frequency=fs_hz,
            Tobs=N / fs_hz, modes=[(2, 2)], return_type="geocenter_td").cpu().numpy()
    for b in range(2):
        hr = c[f"h_{b}"]
        n = int(c["npts"][b])
        assert np.max(np.abs(h[b, :n] - hr[:n])) < 1e-8 * np.abs(hr).max()
        assert np.all(h[b, n:] == 0)
    lnl = bbh.get_ll_td(P[:, :4], c["data"], float(c["amp"]), sampling_frequency=fs_hz, modes=[(2, 2)]).cpu().numpy()
    assert np.all(np.abs(lnl / c["lnl"] - 1) < 1e-9)
