"""The frequency-domain likelihood path on the GPU (BBHWaveformTD.get_ll,
eob/seobnrv4phm.py:772-823) against the numpy restatement of the reference's
flow (oracle/td_oracle.py):

* eob_detector_response (sidereal time, antenna patterns, delays) per
  (detector, binary);
* eob_fd_lnl_from_fft (h~_+ and h~_x split from one complex FFT, projection,
  PSD-weighted residual) on random strains, with bins below a start index
  zeroed;
* the drop-in BBHWaveformTD: geocenter_fd against two real FFTs of its own
  geocenter_td strain, and get_ll end to end against the restated flow on
  (a) the GPU's strain and (b) the oracle's strain replayed on the GPU's
  knots (FP64: relative lnL within 1e-9)."""
import numpy as np
import pytest

from oracle import td_oracle as t

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _detectors(rng, nch):
    D, V = [], []
    for _ in range(nch):
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        D.append(0.5 * (np.outer(q[:, 0], q[:, 0]) - np.outer(q[:, 1], q[:, 1])))
        V.append(6.37e6 * q[:, 2])
    return np.array(D), np.array(V)


def test_detector_response_vs_restatement(torch_cuda):
    from eobgpu_gb300 import fd
    rng = np.random.default_rng(11)
    B, nch = 300, 3
    D, V = _detectors(rng, nch)
    ra, dec = rng.uniform(0, 2 * np.pi, B), rng.uniform(-1.5, 1.5, B)
    psi, tm = rng.uniform(0, np.pi, B), rng.uniform(4e7, 1.4e9, B)  # across many leap seconds
    Fp, Fx, tau = (x.cpu().numpy() for x in fd.detector_response(ra, dec, psi, tm, D, V))
    Rp, Rx, Rt = t.detector_information(ra, dec, tm, psi, D, V)
    np.testing.assert_allclose(Fp, Rp, atol=1e-12)
    np.testing.assert_allclose(Fx, Rx, atol=1e-12)
    np.testing.assert_allclose(tau, Rt, atol=1e-16)


@pytest.mark.parametrize("start_ind", [0, 37])
def test_fd_lnl_from_fft_vs_restatement(torch_cuda, start_ind):
    torch = torch_cuda
    from eobgpu_gb300 import fd
    rng = np.random.default_rng(12 + start_ind)
    B, N, nch, fs = 7, 4100, 3, 512.0
    h = rng.standard_normal((B, N)) + 1j * rng.standard_normal((B, N))
    Nf = N // 2 + 1
    data = rng.standard_normal((nch, Nf)) + 1j * rng.standard_normal((nch, Nf))
    psd = rng.uniform(0.5, 3.0, (nch, Nf))
    D, V = _detectors(rng, nch)
    ra, dec, psi, tm = (rng.uniform(0, 2 * np.pi, B), rng.uniform(-1.5, 1.5, B), rng.uniform(0, np.pi, B),
                        rng.uniform(1e9, 1.3e9, B))
    ref = t.fd_get_ll(h, data, psd, ra, dec, psi, tm, D, V, fs, start_ind=start_ind)
    H = torch.fft.fft(torch.tensor(h, device="cuda"), dim=-1)
    Fp, Fx, tau = fd.detector_response(ra, dec, psi, tm, D, V)
    got = fd.fd_lnl_from_fft(torch.view_as_real(H).contiguous(), torch.tensor(data, device="cuda"),
                             torch.tensor(psd, device="cuda"), Fp, Fx, tau, fs / N, start_ind).cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-12)


@pytest.fixture(scope="module")
def bbh(torch_cuda):
    """Three detectors with synthetic geometry and data (an injection through
    the restated response plus Gaussian noise), 8 configuration-1 binaries."""
    torch = torch_cuda
    from eobgpu_gb300.fd import Interferometer
    from eobgpu_gb300.eob.seobnrv4phm import BBHWaveformTD
    from eobgpu_gb300 import workload
    rng = np.random.default_rng(21)
    fs, Tobs = 1024.0, 8.0
    N = int(fs * Tobs)
    Nf = N // 2 + 1
    D, V = _detectors(rng, 3)
    asd = np.full(Nf, 1.0)
    asd[:10] = np.inf
    ifos = [Interferometer(D[c], V[c], asd, np.zeros(Nf, complex)) for c in range(3)]
    # inspiral-only templates: the oracle comparison below replays the inspiral
    gen = BBHWaveformTD(ifos, amp_phase_kwargs={"imr": False})
    cfg = workload.CONFIGS[1]
    P = workload.draw_params(cfg)
    B = len(P)
    ext = {"distance": np.full(B, 1.0), "phiRef": np.zeros(B), "inc": np.zeros(B),
           "ra": rng.uniform(0, 2 * np.pi, B), "dec": rng.uniform(-1.2, 1.2, B), "psi": rng.uniform(0, np.pi, B),
           "geocent_time": rng.uniform(1.1e9, 1.2e9, B)}
    params = [P[:, 0], P[:, 1], P[:, 2], P[:, 3], ext["distance"], ext["phiRef"], ext["inc"], ext["ra"],
              ext["dec"], ext["psi"], ext["geocent_time"]]
    # data: binary 0 through the restated flow, plus noise
    h0 = gen(*params[:4], params[4], params[5], sampling_frequency=fs, Tobs=Tobs, return_type="geocenter_td")
    h0 = h0.cpu().numpy()
    Fp, Fx, tau = t.detector_information(ext["ra"], ext["dec"], ext["geocent_time"], ext["psi"], D, V)
    f = np.fft.rfftfreq(N, 1.0 / fs)
    hp, hc = np.fft.rfft(h0[0].real), np.fft.rfft(h0[0].imag)
    data = (Fp[:, 0, None] * hp + Fx[:, 0, None] * hc) * np.exp(-2j * np.pi * f * tau[:, 0, None])
    data += 0.3 * (rng.standard_normal((3, Nf)) + 1j * rng.standard_normal((3, Nf)))
    ifos = [Interferometer(D[c], V[c], asd, data[c]) for c in range(3)]
    gen = BBHWaveformTD(ifos, amp_phase_kwargs={"imr": False})
    return gen, params, fs, Tobs, D, V, data, asd


def test_geocenter_fd_is_two_real_ffts(bbh):
    gen, params, fs, Tobs, *_ = bbh
    h = gen(*params, sampling_frequency=fs, Tobs=Tobs, return_type="geocenter_td").cpu().numpy()
    hp, hc = gen(*params, sampling_frequency=fs, Tobs=Tobs, return_type="geocenter_fd", bilby_start_ind=5)
    rp, rc = np.fft.rfft(h.real, axis=-1), np.fft.rfft(h.imag, axis=-1)
    rp[:, :5] = 0
    rc[:, :5] = 0
    sc = np.abs(rp).max()
    assert np.max(np.abs(hp.cpu().numpy() - rp)) < 1e-12 * sc
    assert np.max(np.abs(hc.cpu().numpy() - rc)) < 1e-12 * sc


def test_get_ll_vs_restated_flow(bbh):
    gen, params, fs, Tobs, D, V, data, asd = bbh
    ll = gen.get_ll(params, sampling_frequency=fs, Tobs=Tobs)
    h = gen(*params, sampling_frequency=fs, Tobs=Tobs, return_type="geocenter_td").cpu().numpy()
    psd = np.tile(asd ** 2, (3, 1))
    psd[np.isinf(psd)] = 1e300
    ref = t.fd_get_ll(h, data, psd, params[7], params[8], params[9], params[10], D, V, fs)
    np.testing.assert_allclose(ll, ref, rtol=1e-11)
    assert np.argmax(ll) == 0  # the injected binary fits its data best


def test_get_ll_vs_oracle_strain_on_the_same_knots(bbh, oracle):
    """The waveform under get_ll against the oracle's (replayed on the GPU's
    knots), both through the restated frequency-domain flow."""
    gen, params, fs, Tobs, D, V, data, asd = bbh
    ll = gen.get_ll(params, sampling_frequency=fs, Tobs=Tobs)
    _, _, _, trajs = gen._wl.trajectories()
    N = int(fs * Tobs)
    hs = []
    for b in range(len(ll)):
        p = np.array([params[0][b], params[1][b], params[2][b], params[3][b], 20.0])
        # the default modes of the waveform class: (2,2), (2,1), (3,3), (4,4), (5,5)
        r = oracle.lnl_one(p, 1.0 / fs, N, [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)], np.zeros(N), 1.0,
                           want_detail=True, replay_t=trajs[b][0])
        hs.append(r["h"])
    psd = np.tile(asd ** 2, (3, 1))
    psd[np.isinf(psd)] = 1e300
    ref = t.fd_get_ll(np.array(hs), data, psd, params[7], params[8], params[9], params[10], D, V, fs)
    np.testing.assert_allclose(ll, ref, rtol=1e-9)
