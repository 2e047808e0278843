"""Generate the golden fixtures of the EOB path from the reference itself.

Runs in the build container only (needs the reference checkout): it builds
oracle/_ref/libeobref.so from the reference's own sources
(oracle/ref/build_ref.sh) and drives those kernels through a numpy restatement
of the reference's Python glue (eob/seobnrv4phm.py, eob/new_Dormand_horiz.py),
one binary at a time.  The outputs are small .npz files committed next to
this script; the tests compare the oracle and the CUDA path against them.

Usage:  python tests/golden/make_golden.py [--ref /root/reference]
"""
from __future__ import annotations

import argparse
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
from scipy.special import gamma as sgamma

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
from eobgpu_gb300 import workload  # noqa: E402

MTSUN_SI = 4.925491025543576e-06
P = ctypes.POINTER(ctypes.c_double)
PI32 = ctypes.POINTER(ctypes.c_int)


def dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(P)


def ip(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(PI32)


class Ref:
    """ctypes view of the reference's host-compiled kernels."""

    def __init__(self, path):
        self.lib = lib = ctypes.CDLL(path)
        lib.ref_eob_create.restype = ctypes.c_void_p
        for name in ["ref_eob_update", "ref_eob_dealloc", "ref_eob_coeffs", "ref_eob_ode", "ref_eob_rr_force",
                     "ref_eob_root_find_scalar_all", "ref_eob_ic_diss", "ref_eob_waveform", "ref_dopr_steps",
                     "ref_eob_destroy"]:
            getattr(lib, name).argtypes = None
        self.ncoef = lib.ref_coeffs_ndouble()

    # --- src/eob.pyx wrappers ---
    def evaluate_H(self, r, phi, pr, pphi, m1, m2, c1, c2):
        n = len(r)
        out = np.zeros(n)
        z = ctypes.c_double(0.0)
        self.lib.ref_evaluate_H(dp(out), dp(r), dp(phi), dp(pr), dp(pphi), dp(m1), dp(m2), dp(c1), dp(c2), z, z, z, z,
                                ctypes.c_int(n))
        return out

    def grad_H(self, arg, add, n):
        g = np.zeros(4 * n)
        self.lib.ref_grad_H(dp(arg), dp(g), dp(add), ctypes.c_int(n))
        return g

    def hessian_H(self, arg, add, n):
        h = np.zeros(16 * n)
        self.lib.ref_hessian_H(dp(arg), dp(h), dp(add), ctypes.c_int(n))
        return h


def field_names(ref_root):
    txt = open(os.path.join(ref_root, "include", "EOB.hh")).read()
    body = txt[txt.index("typedef struct FacWaveformCoeffsTag"):txt.index("} FacWaveformCoeffs;")]
    return re.findall(r"double\s+(\w+);", body)


# ---------------------------------------------------------------------------
# numpy restatement of the reference's Python glue
def factorial2(n):
    n = np.atleast_1d(n)
    out = np.zeros_like(n, dtype=np.float64)
    odd = (n % 2).astype(bool)
    out[odd] = sgamma(n[odd] / 2 + 1) * 2 ** ((n[odd] + 1) / 2) / np.sqrt(np.pi)
    out[~odd] = 2 ** (n[~odd] / 2) * sgamma(n[~odd] / 2 + 1)
    return out


def newton_prefixes(m1, m2):
    """eob/seobnrv4phm.py:1703-1776 for one binary -> complex[35]."""
    ls, ms = [], []
    for l in range(2, 9):
        for m in range(1, l + 1):
            ls.append(l)
            ms.append(m)
    l = np.asarray(ls)
    m = np.asarray(ms)
    tot = m1 + m2
    eps = (l + m) % 2
    x1, x2 = m1 / tot, m2 / tot
    eta = m1 * m2 / (tot * tot)
    sign = np.where(np.abs(m % 2) == 0, 1, -1)
    test1 = (m1 != m2) | (sign == 1)
    c = (test1 * (np.power(x2, l + eps - 1) + sign * np.power(x1, l + eps - 1))
         + (~test1 & (l == 2)) * -1.0 + (~test1 & (l == 3)) * -1.0 + (~test1 & (l == 4)) * -0.5
         + (~test1 & (l == 5)) * -0.5)
    n = np.zeros(len(l), dtype=np.complex128)
    i0 = eps == 0
    n[i0] = (1j * m[i0]) ** l[i0]
    n[i0] *= 8.0 * np.pi / factorial2(2 * l[i0] + 1)
    n[i0] *= np.sqrt(((l[i0] + 1) * (l[i0] + 2)) / (l[i0] * (l[i0] - 1)))
    i1 = eps == 1
    n[i1] = -((1j * m[i1]) ** l[i1])
    mult2 = (2.0 * l[i1] + 1) * (l[i1] + 2) * (l[i1] * l[i1] - m[i1] * m[i1])
    mult2 = mult2 / ((2.0 * l[i1] - 1) * (l[i1] + 1) * l[i1] * (l[i1] - 1))
    n[i1] *= 1j * 16.0 * np.pi / factorial2(2 * l[i1] + 1)
    n[i1] *= np.sqrt(mult2)
    return n * eta * c


def add_args(m1s, m2s, c1, c2, omega0):
    """setup_class packing, eob/seobnrv4phm.py:1947-1960 (one binary)."""
    a = np.zeros((80, 1))
    a[0], a[1], a[2], a[3], a[4] = m1s, m2s, c1, c2, omega0
    pre = newton_prefixes(m1s, m2s)
    a[10::2, 0] = pre.real
    a[11::2, 0] = pre.imag
    return a


class RefBinary:
    """One binary through the reference: update_information + IC + trajectory."""

    def __init__(self, ref: Ref, m1, m2, c1, c2, f0, max_step):
        self.ref = ref
        lib = ref.lib
        mt = m1 + m2
        self.mt = mt
        self.m1s, self.m2s = m1 / mt, m2 / mt
        self.c1, self.c2 = c1, c2
        self.omega0 = f0 * (mt * MTSUN_SI * np.pi)
        self.add = add_args(self.m1s, self.m2s, c1, c2, self.omega0)
        eta = self.m1s * self.m2s / (self.m1s + self.m2s) ** 2
        chiS, chiA = (c1 + c2) / 2, (c1 - c2) / 2
        tpl = (1 - 2 * eta) * chiS + (self.m1s - self.m2s) / (self.m1s + self.m2s) * chiA
        self.obj = ctypes.c_void_p(lib.ref_eob_create())
        arr = lambda v: np.array([v], dtype=np.float64)
        pre = newton_prefixes(self.m1s, self.m2s)
        self.prefixes_hlms = pre
        pk = np.ascontiguousarray(np.stack([pre.real, pre.imag], axis=1).ravel()[:2])
        lib.ref_eob_update(self.obj, dp(arr(self.m1s)), dp(arr(self.m2s)), dp(arr(eta)), dp(arr(tpl)), dp(arr(chiS)),
                           dp(arr(chiA)), ctypes.c_int(1), ctypes.c_int(1), dp(pk))
        self.max_step = max_step
        self.idx = np.zeros(1, dtype=np.int32)

    def coeffs(self):
        out = np.zeros(self.ref.ncoef)
        self.ref.lib.ref_eob_coeffs(self.obj, dp(out), ctypes.c_int(1))
        return out

    def close(self):
        self.ref.lib.ref_eob_dealloc(self.obj)
        self.ref.lib.ref_eob_destroy(self.obj)

    def ode(self, y):
        k = np.zeros(4)
        x = np.zeros(1)
        self.ref.lib.ref_eob_ode(self.obj, dp(x), dp(np.ascontiguousarray(y, dtype=np.float64)), dp(k),
                                 dp(np.ascontiguousarray(self.add.ravel())), ctypes.c_int(1), ip(self.idx))
        return k

    def initial_conditions(self, max_iter=1000, err=1e-12):
        """eob/seobnrv4phm.py:1966-2070."""
        lib = self.ref.lib
        add = np.ascontiguousarray(self.add.ravel())
        r_guess = self.omega0 ** (-2.0 / 3)
        x0 = np.array([r_guess, np.sqrt(r_guess)])
        xout = np.zeros(2)
        args = np.zeros(4)
        lib.ref_root_find_all(dp(xout), dp(x0), dp(args), dp(add), ctypes.c_int(max_iter), ctypes.c_double(err),
                              ctypes.c_int(1), ctypes.c_int(2), ctypes.c_int(4), ctypes.c_int(80))
        r0, pphi0 = xout
        pr0 = np.zeros(1)
        bounds = np.array([-3e-2, 0.0])
        args = np.array([r0, 0.0, 0.0, pphi0])
        add = np.ascontiguousarray(self.add.ravel())
        lib.ref_eob_root_find_scalar_all(self.obj, dp(pr0), dp(bounds), dp(args), dp(add), ctypes.c_int(max_iter),
                                         ctypes.c_double(err), ctypes.c_int(1), ctypes.c_int(4), ctypes.c_int(80))
        return r0, pphi0, pr0[0]

    def integrate(self, t, traj, step_num, hInit, fix_step, tmax=1e7 * 1e6):
        """eob/new_Dormand_horiz.py:424-778 with numSys = 1."""
        lib = self.ref.lib
        x = np.array([t[step_num]])
        solOld = traj[step_num].copy()
        add = np.ascontiguousarray(self.add.ravel())
        h = np.array([hInit])
        hfix = hInit
        errOld = np.array([1e-4])
        prev = np.zeros(1, dtype=np.uint8)
        stop = True
        old_omegas = np.zeros(self.max_step)
        while True:
            ks = [np.zeros(4) for _ in range(10)]
            xc = np.zeros(1)
            arg = np.zeros(4)
            ak = np.zeros(4)
            solNew = np.zeros(4)
            err = np.zeros(1)
            flag = np.zeros(1, dtype=np.uint8)
            so = solOld.copy()
            lib.ref_dopr_steps(dp(x), dp(xc), dp(so), dp(h), dp(arg), dp(add), *[dp(k) for k in ks], dp(ak),
                               ctypes.c_int(4), ctypes.c_int(1), ctypes.c_int(80), self.obj, ip(self.idx))
            k1, k2, k3, k4, k5, k6, k7, k8, k9, k10 = ks
            lib.ref_dopr_error(dp(err), dp(so), dp(solNew), dp(h), dp(k1), dp(k2), dp(k3), dp(k6), dp(k7), dp(k8),
                               dp(k9), dp(k10), ctypes.c_int(1), ctypes.c_int(4))
            hOld = h[0]
            lib.ref_dopr_controller(flag.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), dp(err), dp(errOld),
                                    prev.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), dp(h), dp(x),
                                    ctypes.c_int(1), ctypes.c_int(4))
            ok = bool(flag[0])
            if fix_step and not ok:
                hfix /= 2
            if fix_step:
                h[0] = hfix
            if ok:
                solOld = solNew.copy()
                x[0] = x[0] + hOld
                step_num += 1
                traj[step_num] = solOld
                t[step_num] = x[0]
                stop = self._stop(solOld, step_num, old_omegas) != 0
            if x[0] >= tmax or step_num >= self.max_step - 1 or stop:
                break
        return step_num

    def _stop(self, y, step, old_omegas):
        """StoppingCriterion.__call__ (eob/seobnrv4phm.py:82-150), numSys = 1."""
        k = self.ode(y)
        r, drdt, omega, dprdt = y[0], k[0], k[1], k[2]
        stop = 0
        if r < 1.0:
            stop = 2
        elif r < 6.0 and drdt > 0.0:
            stop = 3
        elif r < 6.0 and dprdt > 0.0:
            stop = 4
        elif step > 5:
            c1 = r < 6.0
            c2 = omega < old_omegas[step - 1]
            c3 = bool(np.all(np.diff(old_omegas[step - 4:step]) < 0.0))
            stop = 5 * int(c1 and c2 and c3)
        old_omegas[step] = omega
        return stop

    def trajectory(self, r0, pphi0, pr0, step_back=10.0, fine_step=0.05):
        """run_trajectory, eob/seobnrv4phm.py:2072-2136 (times in units of M)."""
        t = np.zeros(self.max_step)
        traj = np.zeros((self.max_step, 4))
        traj[0] = [r0, 0.0, pr0, pphi0]
        S = self.integrate(t, traj, 0, 0.01, False)
        b = t[1:].astype(bool).astype(int)
        last = np.where(np.diff(b) == -1)[0]
        t_stop = t[last[0]]
        idx = int(np.argmin(np.abs(t - (t_stop - step_back))))
        t[idx:] = 0.0
        traj[idx:] = 0.0
        S = self.integrate(t, traj, idx - 1, fine_step, True)
        L = S + 1
        return t[:L].copy(), traj[:L].copy(), S

    def modes(self, t, traj, ells, mms, inputs=None):
        """get_hlms, eob/seobnrv4phm.py:2138-2221 -> complex[K][L]; `inputs`
        (a dict, if given) receives the per-row v, H_real and vPhi passed to
        EOBGetSpinFactorizedWaveform."""
        lib = self.ref.lib
        L = len(t)
        r, phi, pr, pphi = [np.ascontiguousarray(traj[:, j]) for j in range(4)]
        add = np.ascontiguousarray(np.repeat(self.add[:, :, None], L, axis=-1).ravel())
        args = np.ascontiguousarray(np.array([r, phi, pr, pphi]).ravel())
        g = self.ref.grad_H(args, add, L).reshape(4, L)
        args0 = np.ascontiguousarray(np.array([r, phi, np.zeros(L), pphi]).ravel())
        g0 = self.ref.grad_H(args0, add, L).reshape(4, L)
        omega, omega_c = g[3], g0[3]
        vPhi = np.ascontiguousarray(1 / (omega_c ** 2 * r ** 3))
        M = self.m1s + self.m2s
        nu = (self.m1s * self.m2s / M) / M
        H = self.ref.evaluate_H(r, phi, pr, pphi, np.full(L, self.m1s), np.full(L, self.m2s), np.full(L, self.c1),
                                np.full(L, self.c2))
        Hval = np.ascontiguousarray(nu * H)
        v = np.ascontiguousarray(omega ** (1.0 / 3))
        out = np.zeros((len(ells), L), dtype=np.complex128)
        tmp = np.zeros(2 * L)
        for j, (l, m) in enumerate(zip(ells, mms)):
            pre = self.prefixes_hlms[(l - 2) * (l + 1) // 2 + (m - 1)]
            pk = np.array([pre.real, pre.imag])
            lib.ref_eob_waveform(self.obj, dp(tmp), dp(r), dp(phi), dp(pr), dp(pphi), dp(v), dp(Hval),
                                 dp(np.array([nu])), dp(vPhi), ctypes.c_int(l), ctypes.c_int(m), dp(pk),
                                 ctypes.c_double(0.0), ctypes.c_int(1), ctypes.c_int(L), ip(self.idx))
            out[j] = tmp[0::2] + 1j * tmp[1::2]
        if inputs is not None:
            inputs.update({"v": v, "Hreal": Hval, "vPhi": vPhi, "eta": nu})
        return out


def ref_spline(ref: Ref, x, y_all, nsubs):
    """interpolate_TD for one binary; y_all (nsubs, L) -> c1, c2, c3 (nsubs, L)."""
    L = len(x)
    yv = np.ascontiguousarray(y_all.T.ravel())     # [L][nsubs][1]
    B = np.zeros(L * nsubs)
    ud = np.zeros(L * nsubs)
    dg = np.zeros(L * nsubs)
    ld = np.zeros(L * nsubs)
    lengths = np.array([L], dtype=np.int32)
    ref.lib.ref_interpolate_TD(dp(np.ascontiguousarray(x)), dp(yv), dp(B), dp(ud), dp(dg), dp(ld), ip(lengths),
                               ctypes.c_int(1), ctypes.c_int(nsubs))
    return ud.reshape(L, nsubs).T, dg.reshape(L, nsubs).T, ld.reshape(L, nsubs).T


def spline_eval(x, y, c1, c2, c3, tnew):
    """CubicSplineInterpolantTD.__call__ (eob/seobnrv4phm.py:274-386), one binary."""
    i = np.searchsorted(x, tnew, side="right") - 1
    i[i == len(x)] -= 1
    xx = tnew - x[i]
    x2 = xx * xx
    x3 = x2 * xx
    return y[..., i] + c1[..., i] * xx + c2[..., i] * x2 + c3[..., i] * x3


def synthesize(ref: Ref, t_M, traj, hlms, mms, mt, dt):
    """compute_full_waveform up to the mode sum (eob/seobnrv4phm.py:2310-2372), one binary.

    Real and imaginary parts of each mode are paired per mode (the reference's
    0::2 / 1::2 slicing pairs them correctly only for one mode)."""
    t_sec = t_M * mt * MTSUN_SI
    t_in = t_sec / (mt * MTSUN_SI)
    dT = dt / (mt * MTSUN_SI)
    phi = traj[:, 1]
    pc1, pc2, pc3 = ref_spline(ref, t_in, phi[None, :], 1)
    npts = int((t_in[-1] - t_in[0]) / dT) + 1
    t_new = np.arange(npts) * dT + t_in[0]
    t_new[t_new > t_in.max()] = t_in.max()
    phi_i = spline_eval(t_in, phi[None, :], pc1, pc2, pc3, t_new)[0]
    K = len(mms)
    tmp = hlms * np.exp(1j * np.asarray(mms)[:, None] * phi[None, :])
    yy = np.concatenate([tmp.real, tmp.imag], axis=0)
    c1, c2, c3 = ref_spline(ref, t_in, yy, 2 * K)
    res = spline_eval(t_in, yy, c1, c2, c3, t_new)
    modes = res[:K] + 1j * res[K:]
    modes = modes * np.exp(-1j * np.asarray(mms)[:, None] * phi_i[None, :])
    return modes.sum(axis=0), npts


# ---------------------------------------------------------------------------
def make_modes5(ref: Ref, max_step: int):
    """Every mode the reference's waveform class computes, (2,2), (2,1), (3,3),
    (4,4), (5,5) (eob/seobnrv4phm.py:1869), for the eight configuration-1
    binaries (unequal masses, q 1-3): EOBGetSpinFactorizedWaveform on the
    reference's own trajectories (src/EOB.cu:1235-1677) with the per-row
    inputs it was given, the five-mode strain on the uniform grid and the
    five-mode likelihood against the configuration-1 data."""
    cfg = workload.CONFIGS[1]
    c1 = dict(np.load(os.path.join(HERE, "config1.npz")))
    modes = workload.ALL_MODES
    ells = [l for l, _ in modes]
    mms = [m for _, m in modes]
    params = c1["params"]
    data, amp, N = c1["data"], float(c1["amp"]), int(c1["N"])
    L = int(c1["nsteps"].max())
    B = len(params)
    out = {"modes": np.array(modes), "params": params, "nsteps": c1["nsteps"], "traj_t": c1["traj_t"],
           "traj_y": c1["traj_y"], "hlm": np.zeros((B, 5, L), dtype=np.complex128), "v": np.zeros((B, L)),
           "Hreal": np.zeros((B, L)), "vPhi": np.zeros((B, L)), "eta": np.zeros(B), "prefix": np.zeros((B, 5),
                                                                                                        dtype=complex),
           "lnl": np.zeros(B), "npts": np.zeros(B, dtype=int)}
    for b, p in enumerate(params):
        n = int(c1["nsteps"][b])
        t, traj = c1["traj_t"][b, :n], c1["traj_y"][b, :n]
        rb = RefBinary(ref, p[0], p[1], p[2], p[3], p[4], max_step)
        inp = {}
        hl = rb.modes(t, traj, ells, mms, inputs=inp)
        hs, npts = synthesize(ref, t, traj, hl, mms, p[0] + p[1], cfg.dt)
        out["prefix"][b] = [rb.prefixes_hlms[(l - 2) * (l + 1) // 2 + (m - 1)] for l, m in modes]
        rb.close()
        out["hlm"][b, :, :n] = hl
        for k in ("v", "Hreal", "vPhi"):
            out[k][b, :n] = inp[k]
        out["eta"][b] = inp["eta"]
        h = np.zeros(N)
        m = min(npts, N)
        h[:m] = amp * hs[:m].real
        out["lnl"][b] = -0.5 * np.sum((data - h) ** 2)
        out["npts"][b] = npts
        out[f"h_{b}"] = hs[:N]
        print(f"binary {b}: q={p[0] / p[1]:.3f} rows={n} npts={npts} lnL(5 modes)={out['lnl'][b]:.6f}")
    np.savez_compressed(os.path.join(HERE, "modes5.npz"), **out)
    print("modes5.npz written")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--max-step", type=int, default=20000)
    ap.add_argument("--only", choices=["modes5"], default=None,
                    help="write only this fixture (modes5 needs config1.npz)")
    args = ap.parse_args()
    subprocess.check_call([os.path.join(ROOT, "oracle", "ref", "build_ref.sh"), args.ref])
    ref = Ref(os.path.join(ROOT, "oracle", "_ref", "libeobref.so"))
    if args.only == "modes5":
        make_modes5(ref, args.max_step)
        return
    out = {}

    # (1) Hamiltonian, gradient, Hessian, ODE RHS and RR force on random states
    g = np.random.Generator(np.random.PCG64(20240))
    nb = 6
    binaries = np.array([[0.6, 0.4, 0.3, -0.2], [0.5, 0.5, 0.9, 0.9], [0.89, 0.11, -0.9, 0.5],
                         [0.75, 0.25, 0.1, 0.1], [0.55, 0.45, -0.3, 0.25], [0.8, 0.2, 0.8, -0.8]])
    ns = 64
    states, adds, H, grads, hess, rhs, forces, bidx = [], [], [], [], [], [], [], []
    for bi, (m1s, m2s, c1, c2) in enumerate(binaries):
        rb = RefBinary(ref, m1s * 60.0, m2s * 60.0, c1, c2, 20.0, 100)
        r = g.uniform(2.0, 25.0, ns)
        pr = g.uniform(-0.3, 0.0, ns) * (10.0 / r)
        pphi = np.sqrt(r) * g.uniform(0.9, 1.1, ns)
        phi = g.uniform(0, 2 * np.pi, ns)
        st = np.stack([r, phi, pr, pphi])
        addn = np.ascontiguousarray(np.repeat(rb.add, ns, axis=1))
        addn[4] = g.uniform(0.01, 0.1, ns)  # omega slot (used by RR_force only)
        argf = np.ascontiguousarray(st.ravel())
        addf = np.ascontiguousarray(addn.ravel())
        H.append(ref.evaluate_H(r, phi, pr, pphi, np.full(ns, rb.m1s), np.full(ns, rb.m2s), np.full(ns, c1),
                                np.full(ns, c2)))
        grads.append(ref.grad_H(argf, addf, ns).reshape(4, ns))
        hess.append(ref.hessian_H(argf, addf, ns).reshape(16, ns))
        k = np.zeros(4 * ns)
        x = np.zeros(1)
        idx = np.zeros(ns, dtype=np.int32)
        ref.lib.ref_eob_ode(rb.obj, dp(x), dp(argf), dp(k), dp(addf), ctypes.c_int(ns), ip(idx))
        rhs.append(k.reshape(4, ns))
        f = np.zeros(2 * ns)
        gbuf = np.zeros(4 * ns)
        argc = argf.copy()
        ref.lib.ref_eob_rr_force(rb.obj, dp(f), dp(gbuf), dp(argc), dp(addf), ctypes.c_int(ns), ip(idx))
        forces.append(f.reshape(2, ns))
        states.append(st)
        adds.append(addn)
        bidx.append(np.full(ns, bi))
        rb.close()
    out["state"] = np.concatenate(states, axis=1)
    out["add"] = np.concatenate(adds, axis=1)
    out["H"] = np.concatenate(H)
    out["grad"] = np.concatenate(grads, axis=1)
    out["hess"] = np.concatenate(hess, axis=1)
    out["rhs"] = np.concatenate(rhs, axis=1)
    out["force"] = np.concatenate(forces, axis=1)
    out["binary"] = binaries
    np.savez_compressed(os.path.join(HERE, "ham_rhs.npz"), **out)
    print("ham_rhs.npz", {k: v.shape for k, v in out.items()})

    # (2) factorized-waveform coefficients (raw reference struct + field names)
    names = field_names(args.ref)
    assert len(names) == ref.ncoef, (len(names), ref.ncoef)
    coefs = []
    for (m1s, m2s, c1, c2) in binaries:
        rb = RefBinary(ref, m1s * 60.0, m2s * 60.0, c1, c2, 20.0, 100)
        coefs.append(rb.coeffs())
        rb.close()
    np.savez_compressed(os.path.join(HERE, "fac_coeffs.npz"), coeffs=np.array(coefs), names=np.array(names),
                        binary=binaries)
    print("fac_coeffs.npz", len(names))

    # (3) splines on a known cubic and on a ragged EOB-like series
    xs = np.cumsum(g.uniform(0.5, 2.0, 40))
    ys = np.stack([1.0 - 2.0 * xs + 0.5 * xs ** 2 - 0.01 * xs ** 3, np.sin(0.3 * xs) * np.exp(-0.01 * xs)])
    s1, s2, s3 = ref_spline(ref, xs, ys, 2)
    np.savez_compressed(os.path.join(HERE, "spline.npz"), x=xs, y=ys, c1=s1, c2=s2, c3=s3)
    print("spline.npz")

    # (4) configuration 1 end to end: IC, trajectories, modes, synthesis, lnL
    cfg = workload.CONFIGS[1]
    params = workload.draw_params(cfg)
    inj = workload.injection_params(cfg)
    ells = [l for l, _ in cfg.modes]
    mms = [m for _, m in cfg.modes]

    def run(p):
        rb = RefBinary(ref, p[0], p[1], p[2], p[3], p[4], args.max_step)
        ic = rb.initial_conditions()
        t, traj, S = rb.trajectory(*ic)
        hl = rb.modes(t, traj, ells, mms)
        hs, npts = synthesize(ref, t, traj, hl, mms, p[0] + p[1], cfg.dt)
        rb.close()
        return ic, t, traj, hl, hs, npts

    _, _, _, _, hinj, _ = run(inj)
    data, amp = workload.make_data(hinj.real, cfg.n_samples, cfg.index)
    res = {"params": params, "injection": inj, "data": data, "amp": np.array(amp), "dt": np.array(cfg.dt),
           "N": np.array(cfg.n_samples)}
    ics, lnls, npts_all, nsteps = [], [], [], []
    traj_t, traj_y, hmodes, hsum = [], [], [], []
    for b, p in enumerate(params):
        ic, t, traj, hl, hs, npts = run(p)
        N = cfg.n_samples
        h = np.zeros(N)
        m = min(npts, N)
        h[:m] = amp * hs[:m].real
        lnls.append(-0.5 * np.sum((data - h) ** 2))
        ics.append(ic)
        npts_all.append(npts)
        nsteps.append(len(t))
        traj_t.append(t)
        traj_y.append(traj)
        hmodes.append(hl)
        hsum.append(hs[:N])
        print(f"binary {b}: M={p[0] + p[1]:.2f} q={p[0] / p[1]:.3f} steps={len(t)} npts={npts} lnL={lnls[-1]:.6f}")
    res["ic"] = np.array(ics)
    res["lnl"] = np.array(lnls)
    res["npts"] = np.array(npts_all)
    res["nsteps"] = np.array(nsteps)
    Lmax = max(nsteps)
    tt = np.zeros((len(params), Lmax))
    yy = np.zeros((len(params), Lmax, 4))
    hm = np.zeros((len(params), len(ells), Lmax), dtype=np.complex128)
    for b in range(len(params)):
        L = nsteps[b]
        tt[b, :L] = traj_t[b]
        yy[b, :L] = traj_y[b]
        hm[b, :, :L] = hmodes[b]
    res["traj_t"] = tt
    res["traj_y"] = yy
    res["modes_traj"] = hm
    # summed complex strain of the first two binaries (full length up to N)
    for b in range(2):
        res[f"h_{b}"] = hsum[b]
    np.savez_compressed(os.path.join(HERE, "config1.npz"), **res)
    print("config1.npz written")
    make_modes5(ref, args.max_step)


if __name__ == "__main__":
    main()
