"""ORACLE -- test infrastructure, never part of the product path.

numpy restatement of the merger-ringdown completion of the reference's
waveform (SEOBNRv4PHM.compute_full_waveform, eob/seobnrv4phm.py:2374-2557),
for one binary at a time:

  attachment time   t_peak(omega_orb) - Delta t_22 (EOBGetNRSpinPeakDeltaTv4, :878-930)
  NQC coefficients  a1..a3, b1, b2 from splines over the uniform-grid samples
                    from 7 before the attachment sample to the end
                    (EOBCalculateNQCCoefficientsV4_freeattach, :1465-1683)
  NQC correction    (EOBNonQCCorrection, :1686-1700) on every sample
  ringdown          attached at the sample nearest the attachment time, fitted
                    on the 20 M before it (compute_MR_mode_free, :1779-1844;
                    eob/eobstuff.py:44-342), 30 (2,2) damping times long

The NR fits, ringdown coefficients and remnant properties come from the C++
oracle (physics/imr_fits.h through oracle_imr_fits), pinned against the
reference's own fit functions by tests/golden/imr.npz; the Kerr QNMs are
Leaver's continued fractions (the reference asks lalsimulation).  Where the
reference's batched code depends on the other binaries of a batch (padded
windows, the ringdown length of the longest), each binary is treated as a
call of its own.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .oracle import Oracle, _dp, _ip, _f64

MTSUN_SI = 4.925491025543576e-06
NQC_BACK = 7        # samples before the attachment in the NQC fit window
RD_FIT_M = 20.0     # length of the ringdown fit window [M]
RD_DAMPING = 30.0   # ringdown length in (2,2) damping times


class Spline:
    """Not-a-knot cubic spline of the reference (src/interpolate.cu:10-267) on
    knots x; evaluation as CubicSplineInterpolantTD.__call__
    (eob/seobnrv4phm.py:274-386): interval searchsorted(right) - 1, the last
    knot keeping its own (degenerate) row."""

    def __init__(self, x, y):
        x, y = np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64)
        n = len(x)
        if n < 3:
            raise ValueError("a spline needs three knots")
        B, ud, dg, ld = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
        dx = np.diff(x)
        s = np.diff(y) / dx
        # interior rows
        B[1:-1] = 3.0 * (dx[1:] * s[:-1] + dx[:-1] * s[1:])
        dg[1:-1] = 2.0 * (dx[:-1] + dx[1:])
        ud[1:-1] = dx[:-1]
        ld[1:-1] = dx[1:]
        # not-a-knot ends
        d0 = x[2] - x[0]
        B[0] = ((dx[0] + 2 * d0) * dx[1] * s[0] + dx[0] * dx[0] * s[1]) / d0
        ud[0], dg[0] = d0, dx[1]
        dn = x[-1] - x[-3]
        B[-1] = (dx[-1] * dx[-1] * s[-2] + (2 * dn + dx[-1]) * dx[-2] * s[-1]) / dn
        dg[-1], ld[-1] = dx[-2], dn
        for i in range(1, n):
            w = ld[i] / dg[i - 1]
            dg[i] -= w * ud[i - 1]
            B[i] -= w * B[i - 1]
        B[-1] /= dg[-1]
        for i in range(n - 2, -1, -1):
            B[i] = (B[i] - ud[i] * B[i + 1]) / dg[i]
        self.x, self.y = x, y
        self.c1 = np.zeros(n)
        self.c2 = np.zeros(n)
        self.c3 = np.zeros(n)
        t = (B[:-1] + B[1:] - 2 * s) / dx
        self.c1[:-1] = B[:-1]
        self.c2[:-1] = (s - B[:-1]) / dx - t
        self.c3[:-1] = t / dx
        self.c1[-1], self.c2[-1], self.c3[-1] = 0.0, dg[-1], ld[-1]

    def __call__(self, t, deriv=0):
        t = np.asarray(t, dtype=np.float64)
        j = np.searchsorted(self.x, t, side="right") - 1
        j = np.clip(j, 0, len(self.x) - 1)
        xx = t - self.x[j]
        if deriv == 0:
            return self.y[j] + self.c1[j] * xx + self.c2[j] * xx * xx + self.c3[j] * xx * xx * xx
        if deriv == 1:
            return self.c1[j] + 2 * self.c2[j] * xx + 3 * self.c3[j] * xx * xx
        return 2 * self.c2[j] + 6 * self.c3[j] * xx


_FIT_NAMES = ["delta_t22", "amp", "adot", "addot", "omega", "omegadot", "c1f", "c2f", "d1f", "d2f", "final_mass",
              "final_spin", "qnm_re", "qnm_im"]


def fits(orc: Oracle, l, m, m1, m2, chi1, chi2):
    """The fits of mode (l, m) for one binary (physics/imr_fits.h)."""
    out = np.zeros(14)
    orc.lib.oracle_imr_fits(ctypes.c_int(l), ctypes.c_int(m), ctypes.c_double(m1), ctypes.c_double(m2),
                            ctypes.c_double(chi1), ctypes.c_double(chi2), _dp(out))
    return dict(zip(_FIT_NAMES, out))


def qnm_table(orc: Oracle, l, m, a):
    """M omega of the (l, m, 0) Kerr mode at spin a from the table the device uses."""
    out = np.zeros(2)
    orc.lib.oracle_qnm(ctypes.c_int(l), ctypes.c_int(m), ctypes.c_double(a), _dp(out))
    return out[0] + 1j * out[1]


def nqc_factor(r, pr, omega, c):
    """EOBNonQCCorrection (eob/seobnrv4phm.py:1686-1700) with a3S = a4 = a5 =
    b3 = b4 = 0, as the reference sets them."""
    sqrtR = np.sqrt(r)
    rOmega = r * omega
    mag = 1.0 + (pr * pr / (rOmega * rOmega)) * (c["a1"] + c["a2"] / r + c["a3"] / (r * sqrtR))
    phase = c["b1"] * pr / rOmega + pr * pr * pr / rOmega * c["b2"]
    return mag * np.cos(phase) + 1j * mag * np.sin(phase)


def nqc_coefficients(orc, t, amp, phase, r, pr, omega, npts, t_nr, l, m, m1, m2, chi1, chi2):
    """NQC coefficients of one mode (eob/seobnrv4phm.py:1465-1683): splines
    over samples idx - 7 .. npts - 1 (idx the sample nearest t_nr) of
    q_j |h| and p_j, their values and derivatives at t_nr, two linear solves."""
    idx = int(np.argmin(np.abs(t[:npts] - t_nr)))
    lo = idx - NQC_BACK
    if lo < 0 or npts - lo < 3:
        raise ValueError("NQC window outside the waveform")
    w = slice(lo, npts)
    tw, rw, pw, ow = t[w], r[w], pr[w], omega[w]
    rO = rw * ow
    q1 = pw ** 2 / rO ** 2
    q2 = q1 / rw
    q3 = q2 / np.sqrt(rw)
    p1 = pw / rO
    p2 = p1 * pw ** 2
    a = amp[w]
    Q = np.array([[Spline(tw, q * a)(t_nr, i) for q in (q1, q2, q3)] for i in range(3)])
    f = fits(orc, l, m, m1, m2, chi1, chi2)
    sa = Spline(tw, a)
    rhs = np.array([abs(f["amp"]) - sa(t_nr, 0), f["adot"] - sa(t_nr, 1), f["addot"] - sa(t_nr, 2)])
    a123 = np.linalg.solve(Q, rhs)
    P = np.array([[-Spline(tw, p)(t_nr, i) for p in (p1, p2)] for i in (1, 2)])
    sp = Spline(tw, phase[w])
    om, omd = sp(t_nr, 1), sp(t_nr, 2)
    omd = abs(omd) if om * omd > 0.0 else -abs(omd)
    om = abs(om)
    b12 = np.linalg.solve(P, np.array([f["omega"] - om, f["omegadot"] - omd]))
    return {"a1": a123[0], "a2": a123[1], "a3": a123[2], "b1": b12[0], "b2": b12[1], "idx": idx}


def ringdown(t, t_match, amp, damp, omega, phi_match, l, m, m1, m2, chi1, chi2, omega_complex, f):
    """compute_MR_mode_free (eob/seobnrv4phm.py:1779-1844) for one mode:
    omega_complex = omega_R + i / tau (the reference's sign), f = its fits."""
    eta = m1 * m2 / (m1 + m2) ** 2
    sigmaR, sigmaI = -omega_complex.imag, -omega_complex.real
    c1f, c2f, d1f, d2f = f["c1f"], f["c2f"], f["d1f"], f["d2f"]
    if (l, m) == (2, 2) and sigmaR > 2.0 * c1f * np.tanh(c2f):
        c1f = sigmaR / (2.0 * np.tanh(c2f))
    c1c = 1.0 / (c1f * eta) * (damp - sigmaR * amp) * np.cosh(c2f) ** 2
    c2c = amp / eta - 1.0 / (c1f * eta) * (damp - sigmaR * amp) * np.cosh(c2f) * np.sinh(c2f)
    d1c = (omega - sigmaI) * (1 + d2f) / (d1f * d2f)
    x = t - t_match
    A = c1c * np.tanh(c1f * x + c2f) + c2c
    ph = phi_match - d1c * np.log((1 + d2f * np.exp(-d1f * x)) / (1 + d2f))
    w = -omega_complex.real + 1j * omega_complex.imag
    return eta * A * np.exp(1j * ph) * np.exp(1j * w * x)


def knots(orc: Oracle, params, modes, max_step=20000, replay_t=None, h_init=0.01, rtol=1e-12, atol=1e-12):
    """IC, trajectory and the multipoles on it for one binary."""
    params = _f64(params)
    ls = np.ascontiguousarray([l for l, _ in modes], dtype=np.int32)
    ms = np.ascontiguousarray([m for _, m in modes], dtype=np.int32)
    rt = None if replay_t is None else _f64(replay_t)
    if rt is not None:
        max_step = max(max_step, len(rt))
    tt, yy = np.zeros(max_step), np.zeros((max_step, 4))
    hl = np.zeros(2 * len(modes) * max_step)
    st = ctypes.c_int(0)
    L = orc.lib.oracle_knots_ex(_dp(params), _ip(ls), _ip(ms), ctypes.c_int(len(ls)), ctypes.c_int(max_step),
                                ctypes.c_double(rtol), ctypes.c_double(atol), ctypes.c_double(h_init),
                                _dp(rt) if rt is not None else None, ctypes.c_int(0 if rt is None else len(rt)),
                                _dp(tt), _dp(yy), _dp(hl), ctypes.byref(st))
    if st.value != 0:
        raise ValueError("trajectory failed")
    hl = (hl[0::2] + 1j * hl[1::2])[:len(modes) * L].reshape(len(modes), L)
    return {"t": tt[:L], "y": yy[:L], "hlm": hl, "params": params}


def waveform(orc, params, dt, modes, imr=True, max_step=20000, replay_t=None):
    """Modes on the uniform grid t_k = k dt from the binary's start: the
    inspiral (k < npts), NQC-corrected and followed by the ringdown when imr.
    Returns (modes [K, n], info)."""
    kn = knots(orc, params, modes, max_step, replay_t)
    m1, m2, chi1, chi2 = params[0], params[1], params[2], params[3]
    Mt = m1 + m2
    m1s, m2s = m1 / Mt, m2 / Mt
    tin = (kn["t"] * Mt * MTSUN_SI) / (Mt * MTSUN_SI)
    dT = dt / (Mt * MTSUN_SI)
    y = kn["y"]
    ms = np.array([m for _, m in modes])
    sphi = Spline(tin, y[:, 1])
    npts = int((tin[-1] - tin[0]) / dT) + 1
    t = np.arange(npts) * dT + tin[0]
    t = np.minimum(t, tin[-1])
    phi = sphi(t)
    hk = kn["hlm"] * np.exp(1j * ms[:, None] * y[None, :, 1])
    out = np.zeros((len(modes), npts), dtype=complex)
    for q in range(len(modes)):
        re, im = Spline(tin, hk[q].real)(t), Spline(tin, hk[q].imag)(t)
        out[q] = (re + 1j * im) * np.exp(-1j * ms[q] * phi)
    info = {"npts": npts, "t": t, "knots": kn}
    if not imr:
        return out, info
    # ---- attachment time (eob/seobnrv4phm.py:2361-2379)
    om_knots = sphi(tin, 1)
    t_peak = tin[int(np.argmax(om_knots))]
    f22 = fits(orc, 2, 2, m1s, m2s, chi1, chi2)
    dt22 = f22["delta_t22"]
    t_attach = t_peak - dt22
    omega = sphi(t, 1)
    r = Spline(tin, y[:, 0])(t)
    pr = Spline(tin, y[:, 2])(t)
    amp = np.abs(out)
    phase = np.unwrap(np.angle(out), axis=-1)
    # ---- NQC per mode (:2398-2436)
    coeffs = []
    for q, (l, m) in enumerate(modes):
        t_nr = t_peak - (dt22 + (10.0 if (l, m) == (5, 5) else 0.0))
        c = nqc_coefficients(orc, t, amp[q], phase[q], r, pr, omega, npts, t_nr, l, m, m1s, m2s, chi1, chi2)
        coeffs.append(c)
        out[q] = out[q] * nqc_factor(r, pr, omega, c)
    amp = np.abs(out)
    phase = np.unwrap(np.angle(out), axis=-1)
    # ---- ringdown (:2438-2557)
    t_max = t[int(np.argmax(amp[0]))]
    idx = int(np.argmin(np.abs(t - t_attach)))
    ts = t - t_max
    dts = ts[1] - ts[0]
    nfit = int(RD_FIT_M / dts) + 1
    t_match = ts[idx]
    Mf = fits(orc, 2, 2, m1s, m2s, chi1, chi2)["final_mass"]
    af = f22["final_spin"]
    lo = idx - nfit
    if lo < 0 or npts - lo < 3:
        raise ValueError("ringdown fit window outside the waveform")
    tw = ts[lo:npts]
    modes_out = []
    oc22 = None
    rd = []
    for q, (l, m) in enumerate(modes):
        f = fits(orc, l, m, m1s, m2s, chi1, chi2)
        oc = (f["qnm_re"] - 1j * f["qnm_im"]) / Mf
        if q == 0:
            oc22 = oc
        tq = t_match - (10.0 if (l, m) == (5, 5) else 0.0)
        sa, sp = Spline(tw, amp[q, lo:npts]), Spline(tw, phase[q, lo:npts])
        rd.append((f, oc, sa(tq), sa(tq, 1), sp(tq), sp(tq, 1)))
    ringdown_time = int(RD_DAMPING / oc22.imag)
    num_add = int(ringdown_time / dts) + 1
    t_rd = t_match + np.arange(num_add) * dts
    for q, (l, m) in enumerate(modes):
        f, oc, a0, da0, ph0, om0 = rd[q]
        h = ringdown(t_rd, t_match, a0, da0, om0, ph0, l, m, m1s, m2s, chi1, chi2, oc, f)
        modes_out.append(np.concatenate([out[q, :idx + 1], h[1:]]))
    info.update({"t_peak": t_peak, "t_attach": t_attach, "idx_attach": idx, "nqc": coeffs, "final_mass": Mf,
                 "final_spin": af, "num_add": num_add, "npts_imr": idx + num_add})
    return np.array(modes_out), info


def strain_and_lnl(orc, params, dt, modes, data, amp, imr=True, max_step=20000, replay_t=None):
    """(summed strain h[N], lnL = -1/2 sum (d - amp Re h)^2, info) with the
    template zero past its own end."""
    md, info = waveform(orc, params, dt, modes, imr, max_step, replay_t)
    N = len(data)
    h = np.zeros(N, dtype=complex)
    n = min(md.shape[1], N)
    h[:n] = md[:, :n].sum(axis=0)
    r = data - amp * h.real
    return h, -0.5 * float(np.dot(r, r)), info
