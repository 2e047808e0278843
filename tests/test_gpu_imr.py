"""The merger-ringdown completion on the GPU (eob_options.imr = 1: NQC
correction and ringdown attachment, eob/seobnrv4phm.py:2374-2557) against
the oracle's restatement (oracle/imr_oracle.py, whose fits are pinned to the
reference's own functions by tests/golden/imr.npz) on the GPU's own
trajectory knots: the eight configuration-1 binaries, one and five modes,
FP64.  Checked: the attachment sample and the IMR length, every mode and the
summed strain on every sample (within 1e-8 of the peak), the phase at the
peak, and the likelihood (relative 1e-9)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODES5 = [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)]


@pytest.fixture(scope="module")
def runs(golden):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    c = golden["config1"]
    P = torch.tensor(c["params"], dtype=torch.float64, device="cuda")
    D = torch.tensor(c["data"], dtype=torch.float64, device="cuda")
    N, dt, amp = int(c["N"]), float(c["dt"]), float(c["amp"])
    out = {}
    for modes in ([(2, 2)], MODES5):
        o = _lib.default_options()
        o.imr = 1
        wl = WaveformLikelihood(len(P), 4000, modes, N, options=o)
        lnl, st = wl.run(P, D, dt, amp)
        lnl, st = lnl.cpu().numpy(), st.cpu().numpy()
        npts = wl.npts()
        _, _, _, trajs = wl.trajectories()
        wl.prepare(P, dt)
        hm, _ = wl.synth_strain(len(P), dt, N, per_mode=True)
        hs, _ = wl.synth_strain(len(P), dt, N)
        out[len(modes)] = (lnl, st, npts, trajs, hm.cpu().numpy(), hs.cpu().numpy())
    return c, out


@pytest.mark.parametrize("K", [1, 5])
def test_imr_vs_oracle_on_gpu_knots(runs, oracle, K):
    from oracle import imr_oracle as imr
    c, out = runs
    lnl, st, npts, trajs, hm, hs = out[K]
    modes = [(2, 2)] if K == 1 else MODES5
    N, dt, amp = int(c["N"]), float(c["dt"]), float(c["amp"])
    assert np.all(st == 0), st
    worst = [0.0, 0.0, 0.0]
    for b in range(len(lnl)):
        p = c["params"][b]
        h, ll, info = imr.strain_and_lnl(oracle, p, dt, modes, c["data"], amp, replay_t=trajs[b][0])
        md, _ = imr.waveform(oracle, p, dt, modes, replay_t=trajs[b][0])
        n = int(info["npts_imr"])
        assert npts[b] == n, (b, npts[b], n)
        pk = np.max(np.abs(h))
        k = int(np.argmax(np.abs(h)))
        e_sum = np.max(np.abs(hs[b, :n] - h[:n])) / pk
        e_mode = max(np.max(np.abs(hm[b, q, :n] - md[q, :n])) / np.max(np.abs(md[q])) for q in range(K))
        assert np.all(hs[b, n:] == 0) and np.all(hm[b, :, n:] == 0)
        dphi = abs(np.angle(hs[b, k] / h[k]))
        rel = abs(lnl[b] / ll - 1)
        worst = [max(worst[0], e_sum), max(worst[1], e_mode), max(worst[2], rel)]
        assert e_sum < 1e-8 and e_mode < 1e-8, (b, e_sum, e_mode)
        assert dphi < 1e-5, (b, dphi)
        assert rel < 1e-9, (b, lnl[b], ll)
    print(f"\nIMR K={K}: summed strain {worst[0]:.2e}, worst mode {worst[1]:.2e} of peak, lnL {worst[2]:.2e}")


def test_mirror_waveform_class_attaches_the_ringdown(golden, oracle):
    """The drop-in SEOBNRv4PHM (imr on by default, as the reference's
    __call__) returns per-mode IMR waveforms: against the oracle's IMR on the
    generator's own knots, every mode within 1e-8 of its peak, divided by the
    distance."""
    from eobgpu_gb300.eob.seobnrv4phm import SEOBNRv4PHM
    from oracle import imr_oracle as imr
    c = golden["config1"]
    P = c["params"][:3]
    dist = np.array([1.0, 2.0, 4.0])
    gen = SEOBNRv4PHM(max_step=4096)
    fs = 1.0 / float(c["dt"])
    out = gen(P[:, 0], P[:, 1], P[:, 2], P[:, 3], dist, np.zeros(3), fs=20.0, sampling_frequency=fs).cpu().numpy()
    _, _, _, trajs = gen._wl.trajectories()
    for b in range(3):
        md, info = imr.waveform(oracle, P[b], float(c["dt"]), MODES5, replay_t=trajs[b][0])
        n = int(info["npts_imr"])
        for q in range(5):
            ref = md[q] / dist[b]
            assert np.max(np.abs(out[b, q, :n] - ref)) < 1e-8 * np.max(np.abs(ref)), (b, q)
            assert np.all(out[b, q, n:] == 0)


def test_imr_ragged_batch_sample_vs_oracle(oracle):
    """The completion on the ragged-batching population (M 20-200 Msun,
    q 1-8, chi up to 0.9, f0 10-20 Hz, dt = 1/2048 s, N = 2^17): 16 binaries
    spread over the 1024 of the benchmark's seeded draw, run as one batch,
    against the oracle's restatement on the GPU's own knots, with the same IMR
    length.  Bounds: the FP64 tolerances of configuration 1 (summed strain
    within 1e-8 of its peak, phase at the peak within 1e-5 rad, lnL within 1e-9
    relative), or twenty times the oracle's own one-ulp spread where that is
    larger (tests/golden/imr_spread.npz: an ill-conditioned NQC system, with
    coefficients up to ~1e7 that cancel, moves the corrected waveform by up to
    ~1e-3 of its peak when its inputs move by one ulp)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import os
    from eobgpu_gb300 import _lib, workload
    from eobgpu_gb300.pipeline import WaveformLikelihood
    from oracle import imr_oracle as imr
    spread = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "imr_spread.npz"))
    cfg = workload.CONFIGS[2]
    params = workload.draw_params(cfg, stream=0)[::int(spread["stride"])]
    np.testing.assert_array_equal(params, spread["params"])
    N, dt = cfg.n_samples, cfg.dt
    data = np.zeros(N)
    o = _lib.default_options()
    o.imr = 1
    wl = WaveformLikelihood(len(params), 6000, [(2, 2)], N, options=o)
    P = torch.tensor(params, device="cuda")
    lnl, st = wl.run(P, torch.tensor(data, device="cuda"), dt, 1.0)
    lnl, st = lnl.cpu().numpy(), st.cpu().numpy()
    npts = wl.npts()
    trajs = wl.trajectories()[3]
    wl.prepare(P, dt)
    hs, _ = wl.synth_strain(len(params), dt, N)
    hs = hs.cpu().numpy()
    assert np.all(st == 0), st
    rows = []
    for b in range(len(params)):
        h, ll, info = imr.strain_and_lnl(oracle, params[b], dt, [(2, 2)], data, 1.0, replay_t=trajs[b][0])
        n = int(info["npts_imr"])
        assert npts[b] == n, (b, npts[b], n)
        pk = np.max(np.abs(h))
        k = int(np.argmax(np.abs(h)))
        e = np.max(np.abs(hs[b, :n] - h[:n])) / pk
        dphi = abs(np.angle(hs[b, k] / h[k]))
        rel = abs(lnl[b] / ll - 1)
        bs = max(1e-8, 20 * spread["strain"][b])
        rows.append((b, e, dphi, rel, spread["strain"][b]))
        assert e < bs, (b, params[b], e, bs)
        assert dphi < max(1e-5, 20 * spread["strain"][b]), (b, dphi)
        assert rel < max(1e-9, 20 * spread["lnl"][b]), (b, lnl[b], ll)
    print("\nIMR ragged-batch sample, binary: strain of peak, dphi, rel lnL (oracle one-ulp strain spread)")
    for b, e, dphi, rel, sp in rows:
        print(f"  {b:2d}: {e:.2e} {dphi:.1e} {rel:.1e} ({sp:.1e})")
    # the FP64 tolerances themselves hold for most of the sample
    assert sum(1 for r in rows if r[1] < 1e-8 and r[3] < 1e-9) >= 12


def test_imr_window_too_long_keeps_the_inspiral():
    """A binary whose ringdown fit window (the 20 M before the attachment)
    spans more than 256 samples of its grid -- 200 Msun at dt = 1/16384 s,
    dT = 0.062 M, 323 samples -- keeps its inspiral and reports EOB_ST_IMR
    (128), as the inspiral-only run of the same binary: same length, same
    strain, same lnL.  In the same batch the completion still attaches for a
    60 Msun binary (dT = 0.21 M), whose status, length and lnL are bitwise
    those of a batch without the first binary."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    dt, N = 1.0 / 16384.0, 1 << 14
    bad = [100.0, 100.0, 0.2, -0.1, 20.0]
    good = [36.0, 24.0, 0.1, 0.3, 20.0]
    rng = np.random.default_rng(7)
    D = torch.tensor(rng.standard_normal(N), device="cuda")

    def run(rows, imr):
        o = _lib.default_options()
        o.imr = imr
        o.lanes_per_binary = 64
        wl = WaveformLikelihood(len(rows), 20000, [(2, 2)], N, options=o)
        P = torch.tensor(rows, dtype=torch.float64, device="cuda")
        lnl, st = wl.run(P, D, dt, 1.0)
        lnl, st = lnl.cpu().numpy(), st.cpu().numpy()
        npts = wl.npts()
        wl.prepare(P, dt)
        hs, _ = wl.synth_strain(len(rows), dt, N)
        return lnl, st, npts, hs.cpu().numpy()

    lnl_a, st_a, n_a, h_a = run([bad, good], 1)
    lnl_b, st_b, n_b, h_b = run([good], 1)
    lnl_c, st_c, n_c, h_c = run([bad], 0)
    assert st_a[0] == 128, st_a
    assert st_c[0] == 0 and st_a[1] == 0 and st_b[0] == 0, (st_a, st_b, st_c)
    # the first binary: its inspiral, as without the completion
    assert n_a[0] == n_c[0]
    assert np.array_equal(h_a[0], h_c[0])
    assert lnl_a[0] == lnl_c[0], (lnl_a[0], lnl_c[0])
    # the second: completed, and unaffected by its neighbour
    assert n_a[1] == n_b[0] and np.array_equal(h_a[1], h_b[0])
    assert lnl_a[1] == lnl_b[0], (lnl_a[1], lnl_b[0])
