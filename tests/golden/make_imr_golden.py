"""Golden outputs of the reference's merger-ringdown completion, computed by
the reference's own Python functions.

Runs in the build container only (needs the reference checkout).  The
functions are taken out of eob/seobnrv4phm.py and eob/eobstuff.py by their
syntax tree -- the modules themselves import cupy, lal, lalsimulation and
pesummary, which are absent -- and executed with numpy:

  EOBGetNRSpinPeakDeltaTv4, EOBGetNRSpinPeakAmplitudeV4, ...ADotV4,
  ...ADDotV4, ...OmegaV4, ...OmegaDotV4                   (seobnrv4phm.py:878-1463)
  EOBCalculateNQCCoefficientsV4_freeattach, EOBNonQCCorrection (:1465-1700)
  compute_MR_mode_free                                     (:1779-1844)
  compute_final_mass_SEOBNRv4, EOBCalculateRD*Coefficient*  (eobstuff.py:6-342)

Stand-ins for the absent libraries, stored in the fixture with the outputs:
lalsimulation's Kerr ISCO radius and energy are the Bardeen-Press-Teukolsky
closed forms; compute_QNM returns the complex frequencies given in the
fixture; the reference's spline class (CubicSplineInterpolantTD, whose native
kernel is interpolate.cu's not-a-knot spline) is a numpy restatement of that
spline with the class's index rule and derivative formulas.  Those three
stand-ins are not the reference's code; everything else is.  Two readings
where the reference's code does not run as written under numpy:
linalg.solve takes the right-hand sides as stacks of vectors (numpy 1 and
cupy semantics), and compute_MR_mode_free's masked assignment
c1f[mask] = sigmaR / (2 tanh c2f) assigns the masked elements.

Usage:  python tests/golden/make_imr_golden.py [--ref /root/reference]
"""
from __future__ import annotations

import argparse
import ast
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

SEOB_FUNCS = ["EOBGetNRSpinPeakDeltaTv4", "CombineTPLEQMFits", "EOBGetNRSpinPeakAmplitudeV4",
              "EOBGetNRSpinPeakADotV4", "EOBGetNRSpinPeakADDotV4", "EOBGetNRSpinPeakOmegaV4",
              "EOBGetNRSpinPeakOmegaDotV4", "EOBCalculateNQCCoefficientsV4_freeattach", "EOBNonQCCorrection",
              "compute_MR_mode_free"]
STUFF_FUNCS = ["compute_final_mass_SEOBNRv4", "EOBCalculateRDAmplitudeCoefficient1",
               "EOBCalculateRDAmplitudeCoefficient2", "EOBCalculateRDPhaseCoefficient1",
               "EOBCalculateRDPhaseCoefficient2", "EOBCalculateRDAmplitudeConstraintedCoefficient1",
               "EOBCalculateRDAmplitudeConstraintedCoefficient2", "EOBCalculateRDPhaseConstraintedCoefficient1"]
VECTORIZED = ["EOBGetNRSpinPeakAmplitudeV4", "EOBGetNRSpinPeakADotV4", "EOBGetNRSpinPeakADDotV4",
              "EOBGetNRSpinPeakOmegaV4", "EOBGetNRSpinPeakOmegaDotV4", "compute_final_mass_SEOBNRv4"]
MODES = [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)]


def functions(path, names):
    tree = ast.parse(open(path).read())
    defs = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name in names]
    assert sorted(d.name for d in defs) == sorted(names), [d.name for d in defs]
    return ast.Module(body=defs, type_ignores=[])


class _Lalsim:
    """lalsimulation's Kerr ISCO (Bardeen, Press & Teukolsky 1972)."""

    @staticmethod
    def SimRadiusKerrISCO(a):
        z1 = 1.0 + np.cbrt(1.0 - a * a) * (np.cbrt(1.0 + a) + np.cbrt(1.0 - a))
        z2 = np.sqrt(3.0 * a * a + z1 * z1)
        return 3.0 + z2 - np.sign(a) * np.sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2))

    @staticmethod
    def SimEnergyKerrISCO(r):
        return np.sqrt(1.0 - 2.0 / (3.0 * r))


class SplineTD:
    """numpy restatement of CubicSplineInterpolantTD (eob/seobnrv4phm.py:161-386)
    for nsubs = 1: not-a-knot spline per interpolant (src/interpolate.cu:10-267),
    index searchsorted(right) - 1 (the last knot keeps its own row), values and
    derivatives of the cubic."""

    def __init__(self, x, y_all, lengths, nsubs, num_bin_all, use_gpu=False):
        assert nsubs == 1
        self.lengths = np.asarray(lengths).astype(int)
        L = len(x) // num_bin_all
        self.t = np.asarray(x).reshape(L, num_bin_all).T
        self.y = np.asarray(y_all).reshape(L, num_bin_all).T
        self.c = [self._coeffs(self.t[i, :n], self.y[i, :n]) for i, n in enumerate(self.lengths)]

    @staticmethod
    def _coeffs(x, y):
        n = len(x)
        B, ud, dg, ld = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
        for i in range(n):
            if i == n - 1:
                i0, i1, i2 = n - 3, n - 2, n - 1
            elif i == 0:
                i0, i1, i2 = 0, 1, 2
            else:
                i0, i1, i2 = i - 1, i, i + 1
            dx1, dx2, dd = x[i1] - x[i0], x[i2] - x[i1], x[i2] - x[i0]
            s1, s2 = (y[i1] - y[i0]) / dx1, (y[i2] - y[i1]) / dx2
            if i == n - 1:
                B[i] = (dx2 * dx2 * s1 + (2 * dd + dx2) * dx1 * s2) / dd; dg[i] = dx1; ld[i] = dd
            elif i == 0:
                B[i] = ((dx1 + 2 * dd) * dx2 * s1 + dx1 * dx1 * s2) / dd; ud[i] = dd; dg[i] = dx2
            else:
                B[i] = 3.0 * (dx2 * s1 + dx1 * s2); dg[i] = 2 * (dx1 + dx2); ud[i] = dx1; ld[i] = dx2
        for i in range(1, n):
            w = ld[i] / dg[i - 1]
            dg[i] = dg[i] - w * ud[i - 1]
            B[i] = B[i] - w * B[i - 1]
        B[n - 1] = B[n - 1] / dg[n - 1]
        for i in range(n - 2, -1, -1):
            B[i] = (B[i] - ud[i] * B[i + 1]) / dg[i]
        c1, c2, c3 = np.zeros(n), np.zeros(n), np.zeros(n)
        for i in range(n - 1):
            dx = x[i + 1] - x[i]
            slope = (y[i + 1] - y[i]) / dx
            t = (B[i] + B[i + 1] - 2 * slope) / dx
            c1[i] = B[i]; c2[i] = (slope - B[i]) / dx - t; c3[i] = t / dx
        c1[n - 1], c2[n - 1], c3[n - 1] = 0.0, dg[n - 1], ld[n - 1]
        return c1, c2, c3

    def __call__(self, tnew, deriv_order=0):
        tnew = np.atleast_2d(tnew)
        out = np.zeros(tnew.shape)
        for i, n in enumerate(self.lengths):
            x, y = self.t[i, :n], self.y[i, :n]
            c1, c2, c3 = self.c[i]
            j = np.searchsorted(x, tnew[i], side="right") - 1
            j[j == n] -= 1
            xx = tnew[i] - x[j]
            if deriv_order == 0:
                out[i] = y[j] + c1[j] * xx + c2[j] * xx * xx + c3[j] * xx * xx * xx
            elif deriv_order == 1:
                out[i] = c1[j] + 2 * c2[j] * xx + 3 * c3[j] * xx * xx
            else:
                out[i] = 2 * c2[j] + 6 * c3[j] * xx
        return out.squeeze()


class _Dev(np.ndarray):
    """numpy array with cupy's .get()"""

    def get(self):
        return np.asarray(self)


class _Linalg:
    @staticmethod
    def solve(a, b):
        # numpy 1 / cupy semantics: b [..., M] is a stack of vectors
        b = np.asarray(b)
        if b.ndim == np.ndim(a) - 1:
            return np.linalg.solve(a, b[..., None])[..., 0]
        return np.linalg.solve(a, b)


class _MaskArray(np.ndarray):
    """a[mask] = v with v of a's full shape assigns v[mask] (the reading of
    compute_MR_mode_free's c1f[mask] = sigmaR / (2 tanh c2f), which numpy
    rejects as written)."""

    def __setitem__(self, key, value):
        if isinstance(key, np.ndarray) and key.dtype == bool and np.shape(value) == self.shape:
            value = np.asarray(value)[key]
        np.ndarray.__setitem__(self, key, value)


class _Numpy:
    """numpy as the reference used it: numpy 1 broadcasting of linalg.solve,
    and asarray results that take full-shape masked assignments."""
    linalg = _Linalg

    @staticmethod
    def asarray(*a, **k):
        return np.asarray(*a, **k).view(_MaskArray)

    def __getattr__(self, name):
        return getattr(np, name)


def reference_namespace(ref, qnm_values):
    npx = _Numpy()
    ns = {"np": npx, "xp": npx, "cp": object(), "lalsim": _Lalsim, "CubicSplineInterpolantTD": SplineTD}

    def compute_QNM(ell, m, n, af, Mf):
        # one value per binary, as the reference's vectorised compute_QNM
        return np.full(np.shape(af), np.conjugate(qnm_values[(int(ell), int(m))]))

    ns["compute_QNM"] = compute_QNM
    exec(compile(functions(os.path.join(ref, "eob", "seobnrv4phm.py"), SEOB_FUNCS), "seobnrv4phm", "exec"), ns)
    exec(compile(functions(os.path.join(ref, "eob", "eobstuff.py"), STUFF_FUNCS), "eobstuff", "exec"), ns)
    for name in VECTORIZED:
        ns[name] = np.vectorize(ns[name])
    return ns


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    g = np.random.Generator(np.random.PCG64(31337))
    # QNM values given to the ringdown (conjugated as compute_QNM returns them)
    qnm = {lm: complex(0.3 + 0.15 * k, 0.08 + 0.002 * k) for k, lm in enumerate(MODES)}
    ns = reference_namespace(args.ref, qnm)
    out = {"modes": np.array(MODES)}

    # (1) NR fits on a grid of binaries (both mass orders)
    nb = 48
    m1 = g.uniform(0.1, 0.9, nb)
    m2 = 1.0 - m1
    chi1 = g.uniform(-0.95, 0.95, nb)
    chi2 = g.uniform(-0.95, 0.95, nb)
    chiS, chiA = 0.5 * (chi1 + chi2), 0.5 * (chi1 - chi2)
    eta = m1 * m2 / (m1 + m2) ** 2
    chi = chiS + chiA * (m1 - m2) / (m1 + m2) / (1.0 - 2.0 * eta)
    out.update(m1=m1, m2=m2, chi1=chi1, chi2=chi2)
    out["delta_t22"] = ns["EOBGetNRSpinPeakDeltaTv4"](2, 2, m1, m2, chi1, chi2)
    fit = np.zeros((6, len(MODES), nb))
    rd = np.zeros((4, len(MODES), nb))
    for k, (l, m) in enumerate(MODES):
        L, Mm = np.full(nb, l), np.full(nb, m)
        fit[0, k] = ns["EOBGetNRSpinPeakAmplitudeV4"](L, Mm, m1, m2, chiS, chiA)
        fit[1, k] = ns["EOBGetNRSpinPeakADotV4"](L, Mm, m1, m2, chiS, chiA)
        fit[2, k] = ns["EOBGetNRSpinPeakADDotV4"](L, Mm, m1, m2, chiS, chiA)
        fit[3, k] = ns["EOBGetNRSpinPeakOmegaV4"](L, Mm, eta, chi)
        fit[4, k] = ns["EOBGetNRSpinPeakOmegaDotV4"](L, Mm, eta, chi)
        fit[5, k] = ns["EOBGetNRSpinPeakDeltaTv4"](l, m, m1, m2, chi1, chi2)
    ell, emm = np.array([l for l, _ in MODES]), np.array([m for _, m in MODES])
    for b in range(nb):
        rd[0, :, b] = ns["EOBCalculateRDAmplitudeCoefficient1"](ell, emm, eta[b], chi[b])
        rd[1, :, b] = ns["EOBCalculateRDAmplitudeCoefficient2"](ell, emm, eta[b], chi[b])
        rd[2, :, b] = ns["EOBCalculateRDPhaseCoefficient1"](ell, emm, eta[b], chi[b])
        rd[3, :, b] = ns["EOBCalculateRDPhaseCoefficient2"](ell, emm, eta[b], chi[b])
    out["nr_fits"] = fit     # amp, adot, addot, omega, omegadot, delta_t (with the (5,5) offset)
    out["rd_free"] = rd      # c1f, c2f, d1f, d2f
    # final mass of the binaries (q = m1 / m2 as the reference takes it)
    out["final_mass"] = ns["compute_final_mass_SEOBNRv4"](m1, m2, chi1, chi2)

    # (2) NQC correction on random inputs
    n = 40
    r, pr = g.uniform(2.0, 6.0, n), g.uniform(-0.9, -0.01, n)
    om = g.uniform(0.05, 0.3, n)
    coeffs = {k: g.uniform(-2, 2, n) for k in ("a1", "a2", "a3", "a3S", "a4", "a5", "b1", "b2", "b3", "b4")}
    for k in ("a3S", "a4", "a5", "b3", "b4"):
        coeffs[k] = np.zeros(n)
    out.update(nqc_r=r, nqc_pr=pr, nqc_omega=om, **{"nqc_" + k: v for k, v in coeffs.items()})
    out["nqc_factor"] = ns["EOBNonQCCorrection"](r, None, pr, None, om, coeffs)

    # (3) NQC coefficients of two binaries, five modes, on smooth windows of
    # a uniform grid around the attachment time
    B, K, Ng = 2, len(MODES), 60
    dT = 0.8
    t_grid = np.tile(np.arange(Ng) * dT + 100.0, (B, 1))
    s = (t_grid - 130.0) / 20.0
    amp = np.stack([[0.3 * (1 + 0.2 * k) * np.exp(-s[b] ** 2) * (1 + 0.1 * b) for k in range(K)] for b in range(B)])
    phase = np.stack([[(k + 1) * (0.2 * t_grid[b] + 0.03 * s[b] ** 3) for k in range(K)] for b in range(B)])
    rr = 2.5 + 0.5 * np.tanh(-s) + 0.1 * np.arange(B)[:, None]
    prr = -0.3 - 0.1 * np.tanh(s)
    omr = 0.15 + 0.05 * np.tanh(s)
    tpk = np.array([131.0, 128.5])
    mb1, mb2 = np.array([0.7, 0.55]), np.array([0.3, 0.45])
    cb1, cb2 = np.array([0.4, -0.2]), np.array([0.1, 0.6])
    dts = np.stack([ns["EOBGetNRSpinPeakDeltaTv4"](2, 2, mb1, mb2, cb1, cb2)] * K, axis=1)
    dts = dts + 10.0 * ((ell == 5) & (emm == 5))[None, :]
    # one (binary, mode) per call: the reference gathers windows of different
    # lengths into one padded array (index == length is not masked), so its
    # batched form depends on the other windows; each binary alone is what a
    # single-binary call computes
    nqc = {k: np.zeros((B, K)) for k in ("a1", "a2", "a3", "b1", "b2")}
    for b in range(B):
        for k in range(K):
            res = ns["EOBCalculateNQCCoefficientsV4_freeattach"](
                amp[b:b + 1, k:k + 1], phase[b:b + 1, k:k + 1], rr[b:b + 1], prr[b:b + 1], omr[b:b + 1],
                ell[k:k + 1], emm[k:k + 1], tpk[b:b + 1], t_grid[b:b + 1], mb1[b:b + 1], mb2[b:b + 1],
                cb1[b:b + 1], cb2[b:b + 1], dts[b:b + 1, k:k + 1], np.array([Ng]))
            for key in nqc:
                nqc[key][b, k] = res[key][0, 0]
    out.update(nqcw_t=t_grid, nqcw_amp=amp, nqcw_phase=phase, nqcw_r=rr, nqcw_pr=prr, nqcw_omega=omr,
               nqcw_tpeak=tpk, nqcw_m1=mb1, nqcw_m2=mb2, nqcw_chi1=cb1, nqcw_chi2=cb2, nqcw_dt=dts,
               **{"nqcw_" + k: v for k, v in nqc.items()})

    # (4) ringdown: attachment values given, QNMs from the stand-in
    tm = np.array([3.0, -1.5])
    t_rd = tm[:, None] + np.arange(80)[None, :] * 0.9
    attach = {"amp": g.uniform(0.05, 0.4, (B, K)), "damp": g.uniform(-0.01, 0.01, (B, K)),
              "omega": g.uniform(0.2, 1.0, (B, K)),
              "final_mass": np.array([0.95, 0.96]).view(_Dev), "final_spin": np.array([0.68, 0.52]).view(_Dev)}
    phim = g.uniform(-3, 3, (B, K))
    hring, philm = ns["compute_MR_mode_free"](t_rd, mb1, mb2, cb1, cb2, attach, ell, emm, t_match=tm,
                                              phi_match=phim, xp=ns["xp"])
    out.update(rd_t=t_rd, rd_tmatch=tm, rd_amp=attach["amp"], rd_damp=attach["damp"], rd_omega=attach["omega"],
               rd_phimatch=phim, rd_qnm=np.array([qnm[lm] for lm in MODES]), rd_h=hring)
    np.savez_compressed(os.path.join(HERE, "imr.npz"), **out)
    print("imr.npz written", {k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
