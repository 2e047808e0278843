"""Sampler-facing interface of the waveform path.

The reference's parameter-estimation script (test_pe_eob.py) samples eleven
parameters per walker,

    [M_total (Msun), q = m1/m2, chi1z, chi2z, distance (Mpc), phiRef,
     cos(inclination), ra, sin(dec), psi, geocent_time],

maps them to BBHWaveformTD's arguments through eryn's TransformContainer
(test_pe_eob.py:57-62: (M, q) -> (m1, m2), Mpc -> m, arccos, arcsin), puts
box priors on them with three periodic dimensions (:81-100) and asks
lisatools' vectorised Likelihood for every walker of every temperature at
once (:104-116).  eryn and lisatools are not needed here: this module holds
the same layout, transforms, priors and start-point recipe (:154-170), and a
vectorised log-likelihood that evaluates any array of walkers in batches on
the GPU through BBHWaveformTD.get_ll (the fused waveform, one FFT per
binary and the fused frequency-domain likelihood).
"""
from __future__ import annotations

import numpy as np

PC_SI = 3.085677581491367e16  # parsec [m]
NDIM = 11
NAMES = ["mt", "q", "chi1z", "chi2z", "distance_mpc", "phiRef", "cos_inc", "ra", "sin_dec", "psi", "geocent_time"]


def transform(x):
    """Sampling parameters [..., 11] -> get_ll parameters [11, n] (n = the
    product of the leading dimensions): m1 = M q / (1 + q), m2 = M / (1 + q),
    distance in m, inclination = arccos, dec = arcsin."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, NDIM)
    mt, q = x[:, 0], x[:, 1]
    out = x.T.copy()
    out[0] = mt * q / (1.0 + q)
    out[1] = mt / (1.0 + q)
    out[4] = x[:, 4] * 1e6 * PC_SI
    out[6] = np.arccos(x[:, 6])
    out[8] = np.arcsin(x[:, 8])
    return out


class UniformPrior:
    """Independent uniform priors on each of the eleven parameters, with
    optional periodic dimensions (wrapped into [low, low + period))."""

    def __init__(self, low, high, periodic=None):
        self.low = np.asarray(low, dtype=np.float64)
        self.high = np.asarray(high, dtype=np.float64)
        if self.low.shape != (NDIM,) or self.high.shape != (NDIM,) or np.any(self.high <= self.low):
            raise ValueError("need 11 lower and 11 larger upper bounds")
        self.periodic = dict(periodic or {})
        self._logvol = -float(np.sum(np.log(self.high - self.low)))

    @classmethod
    def reference(cls, Tobs: float):
        """The box of test_pe_eob.py:81-100 (periodic phiRef, ra, psi)."""
        lo = [58.0, 1.0, -0.1, -0.1, 10.0, 0.0, -1.0, 0.0, -1.0, 0.0, 0.0]
        hi = [62.0, 5.0, 0.1, 0.1, 1000.0, 2 * np.pi, 1.0, 2 * np.pi, 1.0, np.pi, float(Tobs)]
        return cls(lo, hi, periodic={5: 2 * np.pi, 7: 2 * np.pi, 9: np.pi})

    def wrap(self, x):
        x = np.array(x, dtype=np.float64, copy=True)
        for d, p in self.periodic.items():
            x[..., d] = self.low[d] + np.mod(x[..., d] - self.low[d], p)
        return x

    def logpdf(self, x):
        x = np.asarray(x, dtype=np.float64)
        inside = np.all((x >= self.low) & (x <= self.high), axis=-1)
        return np.where(inside, self._logvol, -np.inf)

    def rvs(self, size, rng=None):
        rng = np.random.default_rng() if rng is None else rng
        return self.low + (self.high - self.low) * rng.uniform(size=tuple(np.atleast_1d(size)) + (NDIM,))


def start_points(mean, ntemps: int, nwalkers: int, factor: float, cov=None, rng=None):
    """Walkers scattered around `mean` (test_pe_eob.py:158-170): mean x (1 +
    factor cov N(0, 1)) per coordinate, phases wrapped, cos/sin clipped to
    [-0.99, 0.99]; shape (ntemps, nwalkers, 1, 11)."""
    rng = np.random.default_rng() if rng is None else rng
    cov = np.full(NDIM, 1e-3) if cov is None else np.asarray(cov, dtype=np.float64)
    mean = np.asarray(mean, dtype=np.float64)
    x = np.tile(mean, (ntemps, nwalkers, 1, 1)) * (1 + factor * cov * rng.standard_normal((ntemps, nwalkers, 1, NDIM)))
    x[..., 5] %= 2 * np.pi
    x[..., 7] %= 2 * np.pi
    x[..., 9] %= np.pi
    x[..., 6] = np.clip(x[..., 6], -0.99, 0.99)
    x[..., 8] = np.clip(x[..., 8], -0.99, 0.99)
    return x


class VectorizedLikelihood:
    """log L for any array of walkers [..., 11] in sampling parameters,
    evaluated on the GPU in batches of at most max_batch binaries through
    bbh.get_ll (BBHWaveformTD with its detectors' data).  Walkers outside the
    prior (if one is given) get -inf without a waveform evaluation."""

    def __init__(self, bbh, waveform_kwargs=None, prior=None, max_batch: int = 2048):
        self.bbh = bbh
        kw = dict(waveform_kwargs or {})
        kw.pop("return_type", None)  # get_ll works on the geocenter FFTs
        self.kw = kw
        self.prior = prior
        self.max_batch = int(max_batch)

    def __call__(self, x):
        x = np.asarray(x, dtype=np.float64)
        lead = x.shape[:-1]
        flat = x.reshape(-1, NDIM)
        out = np.full(len(flat), -np.inf)
        ok = np.ones(len(flat), dtype=bool) if self.prior is None else np.isfinite(self.prior.logpdf(flat))
        idx = np.nonzero(ok)[0]
        for lo in range(0, len(idx), self.max_batch):
            sel = idx[lo:lo + self.max_batch]
            out[sel] = self.bbh.get_ll(list(transform(flat[sel])), **self.kw)
        return out.reshape(lead)

    def log_prob(self, x):
        """log prior + log L (the prior's constant included)."""
        if self.prior is None:
            raise ValueError("no prior given")
        lp = self.prior.logpdf(x)
        return lp + np.where(np.isfinite(lp), self(x), 0.0)
