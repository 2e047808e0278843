"""Measure how far the merger-ringdown completion moves by itself on a
sample of the ragged-batching workload (16 of its 1024 seeded binaries:
M 20-200 Msun, q 1-8, chi up to 0.9, f0 10-20 Hz, dt = 1/2048 s, N = 2^17),
and store it as a fixture.

For each binary the oracle (the CPU restatement of the path, with the
restated completion of oracle/imr_oracle.py) runs the IMR waveform on its own
trajectory knots and on the same knots moved by one ulp.  Where the NQC
system is ill-conditioned (coefficients up to ~1e7 that cancel, as for high
mass ratio and high aligned spins near the end of a short trajectory), a
one-ulp change of the inputs moves the whole NQC-corrected waveform by up
to ~1e-3 of its peak; elsewhere by 1e-11 .. 1e-8.  tests/test_gpu_imr.py
holds the CUDA path to a multiple of this spread where it exceeds the FP64
tolerance.

Usage:  python tests/golden/make_imr_spread.py   (writes imr_spread.npz here)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

STRIDE = 64


def main():
    from eobgpu_gb300 import workload
    from oracle.oracle import Oracle
    from oracle import imr_oracle as imr
    orc = Oracle()
    cfg = workload.CONFIGS[2]
    params = workload.draw_params(cfg, stream=0)[::STRIDE]
    N, dt = cfg.n_samples, cfg.dt
    data = np.zeros(N)
    strain, lnl, amax = [], [], []
    for p in params:
        _, info = imr.waveform(orc, p, dt, [(2, 2)])
        t0 = info["knots"]["t"].copy()
        t1 = t0.copy()
        t1[1:] = np.nextafter(t1[1:], np.inf)
        h0, l0, _ = imr.strain_and_lnl(orc, p, dt, [(2, 2)], data, 1.0, replay_t=t0)
        h1, l1, _ = imr.strain_and_lnl(orc, p, dt, [(2, 2)], data, 1.0, replay_t=t1)
        strain.append(np.max(np.abs(h1 - h0)) / np.max(np.abs(h0)))
        lnl.append(abs(l1 / l0 - 1))
        c = info["nqc"][0]
        amax.append(max(abs(c["a1"]), abs(c["a2"]), abs(c["a3"]), abs(c["b1"]), abs(c["b2"])))
        print(f"{len(strain) - 1:2d} strain {strain[-1]:.2e} lnl {lnl[-1]:.2e} max|nqc| {amax[-1]:.1e}", flush=True)
    np.savez(os.path.join(HERE, "imr_spread.npz"), params=params, strain=np.array(strain), lnl=np.array(lnl),
             nqc_max=np.array(amax), stride=STRIDE)


if __name__ == "__main__":
    main()
