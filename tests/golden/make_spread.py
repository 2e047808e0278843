"""Measure how far the reference's algorithm moves by itself on the
ragged-batching workload (1024 binaries, M 20-200, q 1-8, chi up to 0.9,
f0 10-20 Hz, dt = 1/2048 s, N = 2^17), and store it as a fixture.

The oracle (the CPU restatement of the reference path) runs every 16th
binary three times: with the reference's first step h = 0.01 M and with that
step moved by one ulp up and down.  The adaptive controller's error estimate
is a difference of slopes that cancels to ~1e-12 of the state, so a one-ulp
change re-samples the same trajectory on other knots; the differences between
the three runs are the spread that any two FP64 implementations of the
reference's algorithm show, however exact each is.  tests/test_gpu_config2.py
sets its free-running bounds from this spread, and compares the CUDA path
with the oracle at the FP64 tolerances on identical knots (replay).

Usage:  python tests/golden/make_spread.py   (writes config2_spread.npz here)
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

STRIDE = 16
MAX_STEP = 6000


def _peak(h):
    k = int(np.argmax(np.abs(h)))
    return k, h[k]


def one(args):
    """(lnL, rows, samples) at h = 0.01 M, then per perturbed run: |dlnL| /
    |lnL|, |dlnL|, rows changed, samples changed, phase and relative amplitude
    change at the amplitude peak."""
    p, dt, N, data, amp = args
    from oracle.oracle import Oracle
    o = Oracle()
    r0 = o.lnl_one(p, dt, N, [(2, 2)], data, amp, max_step=MAX_STEP, want_detail=True)
    k, h0 = _peak(r0["h"])
    out = [r0["lnl"], r0["nsteps"], r0["npts"]]
    for h in (np.nextafter(0.01, 1.0), np.nextafter(0.01, 0.0)):
        r = o.lnl_one(p, dt, N, [(2, 2)], data, amp, max_step=MAX_STEP, want_detail=True, h_init=h)
        out += [abs(r["lnl"] / r0["lnl"] - 1), abs(r["lnl"] - r0["lnl"]), int(r["nsteps"] != r0["nsteps"]),
                int(r["npts"] != r0["npts"]), abs(np.angle(r["h"][k] / h0)), abs(abs(r["h"][k]) / abs(h0) - 1)]
    return out


def data_vector(cfg):
    """The workload's data from the oracle's own injection (white noise + the
    injection at SNR 30)."""
    from eobgpu_gb300 import workload
    from oracle.oracle import Oracle
    inj = workload.injection_params(cfg)
    ri = Oracle().lnl_one(inj, cfg.dt, cfg.n_samples, [(2, 2)], np.zeros(cfg.n_samples), 1.0, max_step=MAX_STEP,
                          want_detail=True)
    return workload.make_data(ri["h"].real, cfg.n_samples, cfg.index)


def main():
    from eobgpu_gb300 import workload
    cfg = workload.CONFIGS[2]
    params = workload.draw_params(cfg)
    data, amp = data_vector(cfg)
    idx = np.arange(0, len(params), STRIDE)
    jobs = [(params[b], cfg.dt, cfg.n_samples, data, amp) for b in idx]
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        res = np.array(pool.map(one, jobs, chunksize=1))
    per = res[:, 3:].reshape(len(idx), 2, 6)
    out = {"index": idx, "lnl": res[:, 0], "rows": res[:, 1].astype(int), "samples": res[:, 2].astype(int),
           "rel_dlnl": per[:, :, 0].max(axis=1), "abs_dlnl": per[:, :, 1].max(axis=1),
           "rows_changed": per[:, :, 2].max(axis=1).astype(int), "samples_changed": per[:, :, 3].max(axis=1).astype(int),
           "dphi_peak": per[:, :, 4].max(axis=1), "damp_peak": per[:, :, 5].max(axis=1)}
    np.savez_compressed(os.path.join(HERE, "config2_spread.npz"), **out)
    rel = out["rel_dlnl"]
    print(f"{len(idx)} binaries: rel dlnL max {rel.max():.3e} median {np.median(rel):.3e} "
          f"(<= 1e-9: {np.mean(rel <= 1e-9):.2f}); |dlnL| max {out['abs_dlnl'].max():.3e}; "
          f"peak phase {out['dphi_peak'].max():.3e} rad, amplitude {out['damp_peak'].max():.3e}; "
          f"rows changed in {out['rows_changed'].sum()}, samples in {out['samples_changed'].sum()}")


if __name__ == "__main__":
    main()
