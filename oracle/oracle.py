"""ORACLE -- test infrastructure, never part of the product path.

ctypes wrapper over oracle/eob_oracle.cpp, the serial CPU restatement of the
reference's EOB waveform + likelihood path.  Only tests/, the smoke check of
__graft_entry__ and the CPU-baseline leg of bench.py use it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
P = ctypes.POINTER(ctypes.c_double)
PI32 = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with the host C++ compiler (x86 or Arm)."""
    src = os.path.join(HERE, "eob_oracle.cpp")
    deps = [src, os.path.join(HERE, "oracle_dual.h"),
            os.path.join(HERE, "..", "eobgpu_gb300", "csrc", "physics", "fac_coeffs.h"),
            os.path.join(HERE, "..", "eobgpu_gb300", "csrc", "physics", "ham_coeffs.h"),
            os.path.join(HERE, "..", "eobgpu_gb300", "csrc", "physics", "imr_fits.h"),
            os.path.join(HERE, "..", "eobgpu_gb300", "csrc", "physics", "qnm_table.h")]
    if not force and os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(d) for d in deps):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".{os.getpid()}.tmp"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-o", tmp, src])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(P)


def _ip(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(PI32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    def __init__(self):
        self.lib = lib = ctypes.CDLL(build())
        lib.oracle_ctx_create.restype = ctypes.c_void_p
        lib.oracle_ctx_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_ctx_coeffs.argtypes = [ctypes.c_void_p, ctypes.c_int, P]
        lib.oracle_lnl_one.restype = ctypes.c_double
        lib.oracle_lnl_ex.restype = ctypes.c_double
        self.nfac = lib.oracle_fac_ndouble()

    # --- Hamiltonian -------------------------------------------------------
    def evaluate_H(self, r, phi, pr, pphi, m1, m2, chi1, chi2, K=0.0, d5=0.0, dSO=0.0, dSS=0.0):
        r, phi, pr, pphi, m1, m2, chi1, chi2 = map(_f64, (r, phi, pr, pphi, m1, m2, chi1, chi2))
        out = np.zeros(len(r))
        c = ctypes.c_double
        self.lib.oracle_evaluate_H(_dp(out), _dp(r), _dp(phi), _dp(pr), _dp(pphi), _dp(m1), _dp(m2), _dp(chi1),
                                   _dp(chi2), c(K), c(d5), c(dSO), c(dSS), ctypes.c_int(len(r)))
        return out

    def grad_H(self, state, add):
        state, add = _f64(state), _f64(add)
        n = state.shape[1]
        g = np.zeros((4, n))
        self.lib.oracle_grad_H(_dp(state), _dp(g), _dp(add), ctypes.c_int(n))
        return g

    def hessian_H(self, state, add):
        state, add = _f64(state), _f64(add)
        n = state.shape[1]
        h = np.zeros((16, n))
        self.lib.oracle_hessian_H(_dp(state), _dp(h), _dp(add), ctypes.c_int(n))
        return h

    # --- per-binary coefficient context (SEOBNRv5 class) ------------------
    def context(self, m1, m2, chi1, chi2, use_hm=1):
        m1, m2, chi1, chi2 = map(_f64, (m1, m2, chi1, chi2))
        eta = _f64(m1 * m2 / (m1 + m2) ** 2)
        chiS, chiA = _f64((chi1 + chi2) / 2), _f64((chi1 - chi2) / 2)
        tpl = _f64((1 - 2 * eta) * chiS + (m1 - m2) / (m1 + m2) * chiA)
        p = self.lib.oracle_ctx_create(_dp(m1), _dp(m2), _dp(eta), _dp(tpl), _dp(chiS), _dp(chiA),
                                       ctypes.c_int(use_hm), ctypes.c_int(len(m1)))
        return OracleContext(self, ctypes.c_void_p(p), len(m1))

    # --- whole path --------------------------------------------------------
    def lnl_one(self, params, dt, N, modes, data, amp, max_step=20000, rtol=1e-12, atol=1e-12, want_detail=False,
                h_init=0.01, replay_t=None):
        """The whole path for one binary (IC, trajectory, modes, splines,
        synthesis, lnL).  replay_t: knot times [M] of a trajectory computed
        elsewhere (row 0 at t = 0); the oracle then carries its own state
        from knot to knot with one accepted DOPR853 step each, instead of
        choosing the steps itself.  h_init: first adaptive step [M]."""
        params = _f64(params)
        ls = np.ascontiguousarray([l for l, _ in modes], dtype=np.int32)
        ms = np.ascontiguousarray([m for _, m in modes], dtype=np.int32)
        data = _f64(data)
        ic = np.zeros(3)
        nsteps = ctypes.c_int(0)
        npts = ctypes.c_int(0)
        status = ctypes.c_int(0)
        rt = None
        if replay_t is not None:
            rt = _f64(replay_t)
            max_step = max(max_step, len(rt))
        tt = np.zeros(max_step) if want_detail else None
        yy = np.zeros((max_step, 4)) if want_detail else None
        hh = np.zeros(2 * N) if want_detail else None
        lnl = self.lib.oracle_lnl_ex(_dp(params), ctypes.c_double(dt), ctypes.c_int(N), _ip(ls), _ip(ms),
                                     ctypes.c_int(len(ls)), ctypes.c_int(max_step), ctypes.c_double(rtol),
                                     ctypes.c_double(atol), ctypes.c_double(h_init),
                                     _dp(rt) if rt is not None else None, ctypes.c_int(0 if rt is None else len(rt)),
                                     _dp(data), ctypes.c_double(amp), _dp(ic),
                                     ctypes.byref(nsteps), _dp(tt) if tt is not None else None,
                                     _dp(yy) if yy is not None else None, ctypes.byref(npts),
                                     _dp(hh) if hh is not None else None, ctypes.byref(status))
        out = {"lnl": lnl, "ic": ic, "nsteps": nsteps.value, "npts": npts.value, "status": status.value}
        if want_detail:
            L = nsteps.value
            out["t"] = tt[:L]
            out["y"] = yy[:L]
            out["h"] = hh[0::2] + 1j * hh[1::2]
        return out

    def lnl_batch(self, params, dt, N, modes, data, amp, max_step=20000, rtol=1e-12, atol=1e-12):
        params = _f64(params)
        B = params.shape[0]
        ls = np.ascontiguousarray([l for l, _ in modes], dtype=np.int32)
        ms = np.ascontiguousarray([m for _, m in modes], dtype=np.int32)
        lnl = np.zeros(B)
        status = np.zeros(B, dtype=np.int32)
        self.lib.oracle_lnl_batch(_dp(params), ctypes.c_int(B), ctypes.c_double(dt), ctypes.c_int(N), _ip(ls),
                                  _ip(ms), ctypes.c_int(len(ls)), ctypes.c_int(max_step), ctypes.c_double(rtol),
                                  ctypes.c_double(atol), _dp(_f64(data)), ctypes.c_double(amp), _dp(lnl), _ip(status))
        return lnl, status

    def interpolate_td(self, t, y, lengths, nbin, nsubs):
        t, y = _f64(t), _f64(y)
        lengths = np.ascontiguousarray(lengths, dtype=np.int32)
        Lmax = int(lengths.max())
        c1, c2, c3 = np.zeros_like(y), np.zeros_like(y), np.zeros_like(y)
        self.lib.oracle_interpolate_td(_dp(t), _dp(y), _dp(c1), _dp(c2), _dp(c3), _ip(lengths), ctypes.c_int(nbin),
                                       ctypes.c_int(nsubs), ctypes.c_int(Lmax))
        return c1, c2, c3


class OracleContext:
    def __init__(self, orc: Oracle, handle, n):
        self.o, self.h, self.n = orc, handle, n

    def __del__(self):
        try:
            self.o.lib.oracle_ctx_destroy(self.h)
        except Exception:
            pass

    def coeffs(self, i):
        out = np.zeros(self.o.nfac)
        self.o.lib.oracle_ctx_coeffs(self.h, ctypes.c_int(i), _dp(out))
        return out

    def ode(self, state, add, idx=None):
        state, add = _f64(state), _f64(add)
        n = state.shape[1]
        idx = np.zeros(n, dtype=np.int32) if idx is None else np.ascontiguousarray(idx, dtype=np.int32)
        k = np.zeros((4, n))
        self.o.lib.oracle_ctx_ode(self.h, _dp(state), _dp(k), _dp(add), ctypes.c_int(n), _ip(idx))
        return k

    def waveform(self, r, phi, pr, pphi, v, Hreal, eta, vPhi, l, m, prefix, h22_calib=0.0):
        """EOBGetSpinFactorizedWaveform for binary 0 of this context over one
        trajectory (src/EOB.cu:1235-1613): complex h_lm per row."""
        r, phi, pr, pphi, v, Hreal, vPhi = map(_f64, (r, phi, pr, pphi, v, Hreal, vPhi))
        n = len(r)
        out = np.zeros(2 * n)
        pre = _f64([np.real(prefix), np.imag(prefix)])
        idx = np.zeros(1, dtype=np.int32)
        self.o.lib.oracle_ctx_waveform(self.h, _dp(out), _dp(r), _dp(phi), _dp(pr), _dp(pphi), _dp(v), _dp(Hreal),
                                       _dp(_f64([eta])), _dp(vPhi), ctypes.c_int(l), ctypes.c_int(m), _dp(pre),
                                       ctypes.c_double(h22_calib), ctypes.c_int(1), ctypes.c_int(n), _ip(idx))
        return out[0::2] + 1j * out[1::2]

    def rr_force(self, state, add, idx=None):
        state, add = _f64(state), _f64(add)
        n = state.shape[1]
        idx = np.zeros(n, dtype=np.int32) if idx is None else np.ascontiguousarray(idx, dtype=np.int32)
        f = np.zeros((2, n))
        self.o.lib.oracle_ctx_rr_force(self.h, _dp(f), _dp(state), _dp(add), ctypes.c_int(n), _ip(idx))
        return f


def detail_job(job):
    """One whole-path oracle run for a process pool (start the pool with the
    'spawn' method): job = (params, dt, N, modes, data, amp, max_step,
    replay_t or None).  Returns lnl, status, nsteps, npts, h."""
    params, dt, N, modes, data, amp, max_step, replay_t = job
    r = Oracle().lnl_one(params, dt, N, modes, data, amp, max_step=max_step, want_detail=True, replay_t=replay_t)
    return {k: r[k] for k in ("lnl", "status", "nsteps", "npts", "h")}
