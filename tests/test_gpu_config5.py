"""Configuration-5 shape (large stress: low masses from 10 Hz, the longest
trajectories of the benchmark) on the GPU against the oracle: eight binaries
-- the longest corner of the prior (M = 10 Msun, q = 4, chi = 0.8, about
8700 rows) and seven prior draws (M 10-40, q 1-4, chi up to 0.8) -- at
dt = 1/4096 s over N = 2^20 samples, in mixed precision (FP64 dynamics, phase
and spline solve; FP32 amplitude, sincos and compensated residual).

Replay (the oracle on the GPU's own knots): mismatch <= 1e-6, |dlnL| <= 1e-3
and phase at the peak within 1e-5 rad for the mixed path; the FP64 tolerances
(amplitude within 1e-8 of its peak, phase at the peak within 1e-5 rad,
relative lnL within 1e-9) for the FP64 path.

Free-running (each side on its own steps): the same bounds for the mixed
path, with this rule for a template whose last sample differs from the
oracle's (the two samplings of the trajectory end on different sides of a
sample time; that last sample, at the merger, carries h^2 ~ 25-50 of lnL):
both templates are compared on the samples they both cover -- mismatch,
phase, and the likelihood with each template cut to the common samples --
and the last sample's share is reported apart."""
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CORNER = [8.0, 2.0, 0.8, 0.8, 10.0]
MAX_STEPS = 16000


@pytest.fixture(scope="module")
def cfg5_runs():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import _lib, workload
    from eobgpu_gb300.pipeline import WaveformLikelihood
    from oracle.oracle import detail_job
    cfg = workload.CONFIGS[5]
    params = np.ascontiguousarray(np.vstack([np.array(CORNER)[None, :], workload.draw_params(cfg, batch=7)]))
    N = cfg.n_samples
    wl1 = WaveformLikelihood(1, MAX_STEPS, [(2, 2)], N)
    h, _ = wl1.strain(torch.tensor(workload.injection_params(cfg)[None, :], device="cuda"), cfg.dt, N)
    data, amp = workload.make_data(h[0].real.cpu().numpy(), N, cfg.index)
    del wl1
    P = torch.tensor(params, device="cuda")
    D = torch.tensor(data, device="cuda")
    runs = {}
    for prec in (1, 0):
        o = _lib.default_options()
        o.precision = prec
        wl = WaveformLikelihood(len(params), MAX_STEPS, [(2, 2)], N, options=o)
        lnl, st = wl.run(P, D, cfg.dt, amp)
        hs, _ = wl.strain(P, cfg.dt, N)
        nsteps, npts, _, trajs = wl.trajectories()
        runs[prec] = {"lnl": lnl.cpu().numpy(), "status": st.cpu().numpy(), "h": hs.cpu().numpy(), "npts": npts,
                      "nsteps": nsteps, "t": [t for t, _ in trajs]}
        del wl, hs
        torch.cuda.empty_cache()
    jobs = [(p, cfg.dt, N, [(2, 2)], data, amp, MAX_STEPS, None) for p in params]
    jobs += [(p, cfg.dt, N, [(2, 2)], data, amp, MAX_STEPS, runs[0]["t"][b]) for b, p in enumerate(params)]
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        res = pool.map(detail_job, jobs, chunksize=1)
    return params, data, amp, runs, res[:len(params)], res[len(params):]


def _cmp(a, c, n):
    """mismatch, phase at a's peak over the first n samples"""
    a, c = a[:n], c[:n]
    ov = np.real(np.vdot(a, c)) / np.sqrt(np.real(np.vdot(a, a)) * np.real(np.vdot(c, c)))
    k = int(np.argmax(np.abs(a)))
    return 1 - ov, abs(np.angle(c[k] / a[k])), k


def _lnl_cut(data, amp, h, n):
    """lnL of template h cut to its first n samples."""
    r = data.copy()
    r[:n] -= amp * h[:n].real
    return -0.5 * float(np.dot(r, r))


def test_config5_corner_is_long(cfg5_runs):
    params, data, amp, runs, free, rep = cfg5_runs
    assert np.all(runs[1]["status"] == 0) and np.all(runs[0]["status"] == 0)
    assert runs[0]["nsteps"][0] > 8000, runs[0]["nsteps"][0]
    # the trajectory does not depend on the synthesis precision
    np.testing.assert_array_equal(runs[0]["nsteps"], runs[1]["nsteps"])


def test_config5_replay(cfg5_runs):
    """On the GPU's knots.  FP64: amplitude |h| within 1e-8 of its peak, the
    phase at the peak within 1e-5 rad, relative lnL within 1e-9 (the complex
    difference, which adds the phase error, is reported: the orbital phase of
    the corner binary reaches ~1e4 rad over 8800 rows)."""
    params, data, amp, runs, free, rep = cfg5_runs
    print("\nbinary rows | mixed: mismatch dphi |dlnL| | fp64: amplitude dphi rel_lnl complex_diff")
    for b in range(len(params)):
        r = rep[b]
        assert r["status"] == 0 and r["npts"] == runs[0]["npts"][b]
        n = int(r["npts"])
        mm, dphi, k = _cmp(r["h"], runs[1]["h"][b], n)
        dl_mixed = abs(runs[1]["lnl"][b] - r["lnl"])
        h64, ho = runs[0]["h"][b, :n], r["h"][:n]
        peak = abs(ho[k])
        amp64 = np.max(np.abs(np.abs(h64) - np.abs(ho))) / peak
        dphi64 = abs(np.angle(h64[k] / ho[k]))
        cdiff = np.max(np.abs(h64 - ho)) / peak
        rel64 = abs(runs[0]["lnl"][b] / r["lnl"] - 1)
        print(b, runs[0]["nsteps"][b], f"| {mm:.2e} {dphi:.2e} {dl_mixed:.2e} | {amp64:.2e} {dphi64:.2e} "
                                       f"{rel64:.2e} {cdiff:.2e}")
        assert mm <= 1e-6 and dphi <= 1e-5 and dl_mixed <= 1e-3, (b, mm, dphi, dl_mixed)
        assert amp64 <= 1e-8 and dphi64 <= 1e-5 and rel64 <= 1e-9, (b, amp64, dphi64, rel64)


def test_config5_free_running(cfg5_runs):
    params, data, amp, runs, free, rep = cfg5_runs
    g = runs[1]
    print("\nbinary npts_gpu npts_oracle mismatch dphi |dlnL_common| last_sample_share")
    for b in range(len(params)):
        r = free[b]
        assert r["status"] == 0
        assert abs(int(r["npts"]) - int(g["npts"][b])) <= 1
        n = min(int(r["npts"]), int(g["npts"][b]), len(data))
        mm, dphi, _ = _cmp(r["h"], g["h"][b], n)
        if int(r["npts"]) == int(g["npts"][b]):
            dl = abs(g["lnl"][b] - r["lnl"])
            last = 0.0
        else:
            # mixed-precision lnL with the GPU template cut to the common
            # samples: the GPU's own lnL minus its last sample's share
            last = _lnl_cut(data, amp, g["h"][b], n) - _lnl_cut(data, amp, g["h"][b], n + 1)
            dl = abs((g["lnl"][b] + last) - _lnl_cut(data, amp, r["h"], n))
        print(b, g["npts"][b], r["npts"], f"{mm:.2e} {dphi:.2e} {dl:.2e} {last:.2e}")
        assert mm <= 1e-6 and dphi <= 1e-5 and dl <= 1e-3, (b, mm, dphi, dl)
