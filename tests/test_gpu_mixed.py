"""Mixed-precision synthesis + lnL (eob_options.precision = 1) against the FP64
path on the same trajectories: multi-mode (K = 5) binaries of the
configuration-3 population (M 40-80, q 1-3, chi +-0.3, 20 Hz, dt = 1/2048).
Tolerances: mismatch <= 1e-6 between the mixed and FP64 strains, and
|lnL_mixed - lnL_fp64| <= 1e-3 at SNR 30."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODES = [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)]


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import workload
    from eobgpu_gb300.pipeline import WaveformLikelihood
    cfg = workload.CONFIGS[3]
    params = workload.draw_params(cfg)[:64]
    inj = workload.injection_params(cfg)
    N = 1 << 15
    wl1 = WaveformLikelihood(1, 6000, MODES, N)
    h, _ = wl1.strain(torch.tensor(inj[None, :], device="cuda"), cfg.dt, N)
    data, amp = workload.make_data(h[0].real.cpu().numpy(), N, cfg.index)
    return torch, cfg, params, data, amp, N


def _run(torch, cfg, params, data, amp, N, precision):
    from eobgpu_gb300.pipeline import WaveformLikelihood
    opts = None
    from eobgpu_gb300 import _lib
    opts = _lib.default_options()
    opts.precision = precision
    wl = WaveformLikelihood(len(params), 6000, MODES, N, options=opts)
    p = torch.tensor(params, device="cuda")
    lnl, st = wl.run(p, torch.tensor(data, device="cuda"), cfg.dt, amp)
    hs, st2 = wl.strain(p, cfg.dt, N)
    return lnl.cpu().numpy(), st.cpu().numpy(), hs.cpu().numpy()


def test_mixed_vs_fp64(env):
    torch, cfg, params, data, amp, N = env
    l64, s64, h64 = _run(torch, cfg, params, data, amp, N, 0)
    lmx, smx, hmx = _run(torch, cfg, params, data, amp, N, 1)
    assert np.all(s64 == 0) and np.all(smx == 0)
    assert np.all(np.isfinite(lmx))
    assert np.max(np.abs(lmx - l64)) <= 1e-3, np.max(np.abs(lmx - l64))
    for b in range(len(params)):
        a, c = h64[b], hmx[b]
        ov = np.real(np.vdot(a, c)) / np.sqrt(np.real(np.vdot(a, a)) * np.real(np.vdot(c, c)))
        assert 1 - ov <= 1e-6, (b, 1 - ov)


def test_mixed_requires_mixed_spline_build(env):
    """lnL with precision 1 on a workspace prepared at precision 0 is NaN, not garbage."""
    torch, cfg, params, data, amp, N = env
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    wl = WaveformLikelihood(4, 6000, MODES, N)
    p = torch.tensor(params[:4], device="cuda")
    wl.prepare(p, cfg.dt)
    wl.options.precision = 1
    lnl, st = wl.synth_lnl(4, torch.tensor(data, device="cuda"), cfg.dt, amp)
    assert np.all(np.isnan(lnl.cpu().numpy()))


def test_mixed_vs_oracle(env, oracle):
    """Mixed precision against the FP64 oracle on a sample of the batch:
    mismatch <= 1e-6, |dlnL| <= 1e-3, phase at the amplitude peak within
    1e-5 rad.  The worst values are written to $EOB_ACCURACY_OUT if set."""
    import json
    import os
    torch, cfg, params, data, amp, N = env
    lmx, smx, hmx = _run(torch, cfg, params, data, amp, N, 1)
    worst = {"max_dphi_rad": 0.0, "max_mismatch": 0.0, "max_abs_dlnl": 0.0, "sample": 0}
    for b in range(0, len(params), 8):
        r = oracle.lnl_one(params[b], cfg.dt, N, MODES, data, amp, max_step=6000, want_detail=True)
        assert r["status"] == 0
        a, c = r["h"], hmx[b]
        ov = np.real(np.vdot(a, c)) / np.sqrt(np.real(np.vdot(a, a)) * np.real(np.vdot(c, c)))
        k = int(np.argmax(np.abs(a)))
        dphi = abs((np.angle(c[k]) - np.angle(a[k]) + np.pi) % (2 * np.pi) - np.pi)
        dl = abs(lmx[b] - r["lnl"])
        worst["max_dphi_rad"] = max(worst["max_dphi_rad"], float(dphi))
        worst["max_mismatch"] = max(worst["max_mismatch"], float(1 - ov))
        worst["max_abs_dlnl"] = max(worst["max_abs_dlnl"], float(dl))
        worst["sample"] += 1
        assert 1 - ov <= 1e-6, (b, 1 - ov)
        assert dl <= 1e-3, (b, dl)
        assert dphi <= 1e-5, (b, dphi)
    out = os.environ.get("EOB_ACCURACY_OUT")
    if out:
        with open(out, "w") as f:
            json.dump({"config": "3 (mixed precision, 5 modes, N=2^15 sample)", **worst}, f)
