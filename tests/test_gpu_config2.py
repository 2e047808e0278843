"""Configuration 2 (ragged batching: M 20-200, q 1-8, chi up to 0.9, f0 10-20 Hz,
N = 2^17) on the GPU against the oracle on a 64-binary sample, and the
size-independent checks of the full batch (every binary finishes, lnL finite
and bounded by the data)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cfg2(oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import workload
    from eobgpu_gb300.pipeline import WaveformLikelihood
    cfg = workload.CONFIGS[2]
    params = workload.draw_params(cfg)
    inj = workload.injection_params(cfg)
    wl1 = WaveformLikelihood(1, 6000, [(2, 2)], cfg.n_samples)
    h, _ = wl1.strain(torch.tensor(inj[None, :], device="cuda"), cfg.dt, cfg.n_samples)
    data, amp = workload.make_data(h[0].real.cpu().numpy(), cfg.n_samples, cfg.index)
    wl = WaveformLikelihood(len(params), 6000, [(2, 2)], cfg.n_samples)
    lnl, st = wl.run(torch.tensor(params, device="cuda"), torch.tensor(data, device="cuda"), cfg.dt, amp)
    npts = wl.npts()
    nsteps = wl.trajectories()[0]
    idx = np.arange(0, len(params), 16)
    hs, _ = wl.synth_strain(len(params), cfg.dt, cfg.n_samples)
    h_sample = hs[torch.tensor(idx, device="cuda")].cpu().numpy()
    del hs
    return cfg, params, data, amp, lnl.cpu().numpy(), st.cpu().numpy(), npts, nsteps, (idx, h_sample)


def test_config2_full_batch(cfg2):
    cfg, params, data, amp, lnl, st, npts, nsteps, _ = cfg2
    assert np.all(st == 0)
    assert np.all(np.isfinite(lnl))
    # a template can only lower the likelihood below the pure-noise value by its own energy
    assert np.all(lnl < 0)
    assert np.all(npts > 0)


def _peak_phase_amp(h):
    a = np.abs(h)
    k = int(np.argmax(a))
    return k, np.angle(h[k]), a[k]


def test_config2_sample_vs_oracle(cfg2, oracle):
    """Every 16th binary against the oracle.  The adaptive controller's error
    estimate is a difference of slopes that cancels to ~1e-12 of the state, so
    rounding-level differences between two FP64 evaluations of the same RHS
    move it by ~1e-4 relative; a decision with err that close to 1 flips, and
    the two runs then sample the same trajectory on different steps.  Runs on
    the same step sequence agree to the FP64 tolerance (relative lnL 1e-9);
    flipped runs are held to the waveform tolerance (phase at the amplitude
    peak within 1e-5 rad, peak amplitude within 1e-5 relative, lnL within
    1e-6 relative)."""
    cfg, params, data, amp, lnl, st, npts, nsteps, (idx, hg) = cfg2
    flips = 0
    for j, b in enumerate(idx):
        r = oracle.lnl_one(params[b], cfg.dt, cfg.n_samples, list(cfg.modes), data, amp, max_step=6000,
                           want_detail=True)
        assert r["status"] == 0
        ko, po, ao = _peak_phase_amp(r["h"])
        kg, pg, ag = _peak_phase_amp(hg[j])
        dphi = abs((pg - po + np.pi) % (2 * np.pi) - np.pi)
        if r["npts"] != npts[b] or r["nsteps"] != nsteps[b]:
            flips += 1
            assert abs(r["npts"] - npts[b]) <= 1
            assert ko == kg, (b, ko, kg)
            assert dphi < 1e-5, (b, dphi)
            # a different step sequence near the stop moves the fine-pass knots:
            # the spline then samples the peak differently at the 1e-6 level
            assert abs(ag / ao - 1) < 1e-5, (b, ag, ao)
            assert abs(lnl[b] / r["lnl"] - 1) < 1e-6, (b, lnl[b], r["lnl"])
            continue
        # FP64 tolerance: phase at the amplitude peak within 1e-5 rad (the late
        # plunge amplifies rounding-level differences to ~1e-7 rad)
        assert ko == kg and dphi < 1e-5, (b, dphi)
        assert abs(lnl[b] / r["lnl"] - 1) < 1e-9, (b, lnl[b], r["lnl"], nsteps[b])
    # flips are rounding-level events, not a systematic difference
    assert flips <= len(idx) // 2, flips
