"""Synthetic workloads of the batched EOB waveform + likelihood path.

The reference (mikekatz04/EOBGPU) publishes no benchmark data set; its timing
script draws binaries and builds zero-noise data (test_eob.py:32-71).  The
workloads here are seeded synthetic stand-ins with the shapes and parameter
ranges of the five benchmark configurations:

  1  small plain FP64 case        B=8,     M~U[40,80],  q~U[1,3], chi~U[-0.3,0.3], f0=20 Hz,    (2,2),     dt=1/1024, N=8192
  2  ragged batching              B=1024,  M~U[20,200], q~U[1,8], chi~U[-0.9,0.9], f0~U[10,20], (2,2),     dt=1/2048, N=2^17
  3  mixed precision, all modes   B=4096,  drawn as 1,                                            5 modes,   dt=1/2048, N=2^17
  4  serving                      requests of 1-512 walkers (80% Gaussian ball, 20% config-1 prior)
  5  large stress                 B=65536, M~U[10,40],  q~U[1,4], chi~U[-0.8,0.8], f0=10 Hz,    (2,2),     dt=1/4096, N=2^20

Parameters per binary: (m1, m2, chi1, chi2, f0) with m1 = M q/(1+q),
m2 = M/(1+q) in solar masses.  Data model: d_k = A Re sum_lm h_lm(t_k) of
one seed-drawn injection plus unit-variance white Gaussian noise, with the
amplitude A fixed so that the injection's optimal SNR is 30; a template's
likelihood is lnL = -1/2 sum_k (d_k - A Re sum_lm h_lm(t_k))^2 over the first
N samples of its waveform (zero beyond its end).

All draws use numpy's PCG64 generator, which gives identical streams on x86
and Arm hosts; seed = 1000 * config + stream.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

ALL_MODES = [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)]


@dataclass(frozen=True)
class Config:
    index: int
    batch: int
    total_mass: tuple
    mass_ratio: tuple
    chi: tuple
    f0: tuple
    modes: tuple
    dt: float
    n_samples: int
    name: str = ""


CONFIGS = {
    1: Config(1, 8, (40.0, 80.0), (1.0, 3.0), (-0.3, 0.3), (20.0, 20.0), ((2, 2),), 1.0 / 1024, 8192,
              "plain FP64, B=8"),
    2: Config(2, 1024, (20.0, 200.0), (1.0, 8.0), (-0.9, 0.9), (10.0, 20.0), ((2, 2),), 1.0 / 2048, 2 ** 17,
              "ragged batching, B=1024"),
    3: Config(3, 4096, (40.0, 80.0), (1.0, 3.0), (-0.3, 0.3), (20.0, 20.0), tuple(ALL_MODES), 1.0 / 2048,
              2 ** 17, "mixed precision, B=4096, 5 modes"),
    5: Config(5, 65536, (10.0, 40.0), (1.0, 4.0), (-0.8, 0.8), (10.0, 10.0), ((2, 2),), 1.0 / 4096, 2 ** 20,
              "large stress, B=65536"),
}


def rng(config: int, stream: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(1000 * config + stream))


def draw_params(cfg: Config, batch: int | None = None, stream: int = 0) -> np.ndarray:
    """Seeded parameters, shape (batch, 5): m1, m2, chi1, chi2, f0."""
    b = cfg.batch if batch is None else batch
    g = rng(cfg.index, stream)
    M = g.uniform(*cfg.total_mass, size=b)
    q = g.uniform(*cfg.mass_ratio, size=b)
    chi1 = g.uniform(*cfg.chi, size=b)
    chi2 = g.uniform(*cfg.chi, size=b)
    if cfg.f0[0] == cfg.f0[1]:
        f0 = np.full(b, cfg.f0[0])
    else:
        f0 = g.uniform(*cfg.f0, size=b)
    m1 = M * q / (1.0 + q)
    m2 = M / (1.0 + q)
    return np.ascontiguousarray(np.stack([m1, m2, chi1, chi2, f0], axis=1))


def injection_params(cfg: Config) -> np.ndarray:
    """The injected binary: one draw from the configuration's prior (stream 99)."""
    return draw_params(cfg, 1, stream=99)[0]


def make_data(h_injection_re: np.ndarray, n_samples: int, cfg_index: int, snr: float = 30.0):
    """Data d = A * h_injection_re (zero-padded to n_samples) + white noise.

    Returns (d, A).  A makes sqrt(sum (A h)^2) = snr."""
    h = np.zeros(n_samples)
    m = min(len(h_injection_re), n_samples)
    h[:m] = h_injection_re[:m]
    norm = float(np.sqrt(np.sum(h * h)))
    amp = snr / norm if norm > 0 else 1.0
    noise = rng(cfg_index, 7).standard_normal(n_samples)
    return amp * h + noise, amp


@dataclass
class ServingTrace:
    """Serving workload (configuration 4): Poisson arrivals of walker batches."""
    arrivals: np.ndarray            # arrival times [s]
    sizes: np.ndarray               # walkers per request
    params: list = field(default_factory=list)  # per request (size, 5) arrays


def serving_trace(n_requests: int, rate_hz: float, stream: int = 0) -> ServingTrace:
    cfg = CONFIGS[1]
    g = rng(4, stream)
    gaps = g.exponential(1.0 / rate_hz, size=n_requests)
    arrivals = np.cumsum(gaps)
    sizes = g.integers(1, 513, size=n_requests)
    inj = injection_params(cfg)
    Minj = inj[0] + inj[1]
    qinj = inj[0] / inj[1]
    out = []
    for s in sizes:
        ball = g.uniform(size=s) < 0.8
        M = np.where(ball, Minj * (1 + 0.01 * g.standard_normal(s)), g.uniform(*cfg.total_mass, size=s))
        q = np.where(ball, np.maximum(1.0, qinj * (1 + 0.05 * g.standard_normal(s))), g.uniform(*cfg.mass_ratio, size=s))
        c1 = np.where(ball, np.clip(inj[2] + 0.05 * g.standard_normal(s), -0.99, 0.99), g.uniform(*cfg.chi, size=s))
        c2 = np.where(ball, np.clip(inj[3] + 0.05 * g.standard_normal(s), -0.99, 0.99), g.uniform(*cfg.chi, size=s))
        m1 = M * q / (1 + q)
        m2 = M / (1 + q)
        out.append(np.ascontiguousarray(np.stack([m1, m2, c1, c2, np.full(s, cfg.f0[0])], axis=1)))
    return ServingTrace(arrivals, sizes, out)
