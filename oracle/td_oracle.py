"""ORACLE -- test infrastructure, never part of the product path.

NumPy restatement of the reference's time-domain synthesis and
frequency-domain likelihood kernels of src/interpolate.cu, which cannot be
compiled for the host (they use threadIdx and kernel launches):

  td_interp2             TD2 / TDInterp2          src/interpolate.cu:441-549
  td_interp              TD / TDInterp            src/interpolate.cu:323-438
  all_in_one_likelihood  all_in_one_likelihood    src/interpolate.cu:553-627
  tdinterp_inputs        the caller's set-up      eob/seobnrv4phm.py:389-500 (TDInterp.__call__)

Loops over binaries and vectorised over samples; complex arrays are numpy
complex128.  Parity unpinned against the reference's own execution (its GPU
code does not run here); the restatement follows the cited lines, and the
tests check it on cases with closed-form answers.
"""
from __future__ import annotations

import numpy as np

SUM_BINS = 1024  # NUM_THREADS_SUM, src/interpolate.cu:551


def _cubic(y, c1, c2, c3, j, x):
    # the reference's expression y + c1 x + c2 x^2 + c3 x^3 with x2 = x x, x3 = x x2
    x2 = x * x
    x3 = x * x2
    return y[j] + c1[j] * x + c2[j] * x2 + c3[j] * x3


def _modes(y, c1, c2, c3, base, stride, ind, x, K, ms):
    # src/interpolate.cu:480-530 / 350-390: sum_k (re + i im) exp(-i m phi)
    phi = _cubic(y, c1, c2, c3, base + 2 * K * stride + ind, x)
    h = np.zeros(len(ind), dtype=np.complex128)
    for k in range(K):
        re = _cubic(y, c1, c2, c3, base + k * stride + ind, x)
        im = _cubic(y, c1, c2, c3, base + (K + k) * stride + ind, x)
        h += (re + 1j * im) * np.exp(1j * (-(ms[k] * phi)))
    return h


def td_interp2(dataTime, ts, y, c1, c2, c3, old_length, old_lengths, data_length, B, K, ms, inds, lengths,
               max_length):
    """TD2: templateChannels[b * data_length + i], i < lengths[b]."""
    out = np.zeros(B * data_length, dtype=np.complex128)
    for b in range(B):
        n = int(lengths[b])
        i = np.arange(n)
        ind = np.asarray(inds[max_length * b + i], dtype=np.int64)
        x = dataTime[i] - ts[b * old_length + ind]
        base = b * (2 * K + 1) * old_length
        out[b * data_length + i] = _modes(y, c1, c2, c3, base, int(old_lengths[b]), ind, x, K, ms)
    return out


def td_interp(outs, dataTime, ts_list, y_list, c1_list, c2_list, c3_list, old_lengths, data_length, K, ms,
              inds_list, inds_start, ind_lengths):
    """TD per binary: outs[b][data_length + i] for i < ind_lengths[b] (outs modified in place)."""
    for b in range(len(outs)):
        n = int(ind_lengths[b])
        i = np.arange(n)
        ind = np.asarray(inds_list[b][:n], dtype=np.int64)
        x = dataTime[i + int(inds_start[b])] - ts_list[b][ind]
        outs[b][data_length + i] = _modes(y_list[b], c1_list[b], c2_list[b], c3_list[b], 0, int(old_lengths[b]),
                                         ind, x, K, ms)
    return outs


def all_in_one_likelihood(hp, hc, data, psd, Fplus, Fcross, time_shift, df, B, nch, N):
    """Per 1024-bin block partials of |d - h|^2 / psd, layout [(block * B + b) * nch + ch]."""
    nblk = (N + SUM_BINS - 1) // SUM_BINS
    out = np.zeros(nblk * B * nch, dtype=np.complex128)
    f = df * np.arange(N)
    for b in range(B):
        for ch in range(nch):
            fp, fc, tau = Fplus[ch * B + b], Fcross[ch * B + b], time_shift[ch * B + b]
            h = (fp * hp[b * N:(b + 1) * N] + fc * hc[b * N:(b + 1) * N]) * np.exp(-1j * 2.0 * np.pi * f * tau)
            r = data[ch * N:(ch + 1) * N] - h
            term = (np.conj(r) * r) / psd[ch * N:(ch + 1) * N]
            for q in range(nblk):
                out[(q * B + b) * nch + ch] = np.sum(term[q * SUM_BINS:(q + 1) * SUM_BINS])
    return out


def fd_lnl(temp_sum, df, B, nch):
    """The caller's reduction (eob/seobnrv4phm.py:806-809): -1/2 df 4 sum over blocks and channels."""
    return -0.5 * df * 4.0 * np.asarray(temp_sum).reshape(-1, B, nch).sum(axis=(0, 2))


def tdinterp_inputs(dataTime, t_shaped, lengths):
    """TDInterp.__call__'s index set-up (eob/seobnrv4phm.py:446-478): per
    binary the samples before its last knot time and, for each, the knot
    interval from a right-sided search; returns (lengths_out, inds, max_length)."""
    B = t_shaped.shape[0]
    ends = t_shaped.max(axis=1)
    st = np.searchsorted(dataTime, np.zeros(B), side="left")
    et = np.searchsorted(dataTime, ends, side="left")
    lens = et.astype(np.int32)
    max_length = int(lens.max())
    inds = np.zeros(B * max_length, dtype=np.int32)
    for b in range(B):
        inds[b * max_length + st[b]: b * max_length + et[b]] = (
            np.searchsorted(t_shaped[b], dataTime[st[b]:et[b]], side="right").astype(np.int32) - 1)
    return lens, inds, max_length


# ---------------------------------------------------------------------------
# Detector response and the frequency-domain get_ll flow (numpy restatement)
SPEED_OF_LIGHT = 299792458.0
# GPS times at which GPS - UTC grew by one second (1981-07-01 ... 2017-01-01 UTC)
LEAP_GPS = np.array([46828801, 78364802, 109900803, 173059204, 252028805, 315187206, 346723207, 393984008,
                     425520009, 457056010, 504489611, 551750412, 599184013, 820108814, 914803215, 1025136016,
                     1119744017, 1167264018], dtype=np.float64)


def gmst_from_gps(gps):
    """Greenwich mean sidereal time [rad] (IAU 1982, UT1 = UTC), the quantity
    the reference takes from lal through bilby (eob/seobnrv4phm.py:600-601)."""
    gps = np.asarray(gps, dtype=np.float64)
    leap = np.sum(gps[..., None] >= LEAP_GPS, axis=-1)
    days = (gps - leap) / 86400.0 - (2451545.0 - 2444244.5)
    T = days / 36525.0
    s = 67310.54841 + T * ((876600.0 * 3600.0 + 8640184.812866) + T * (0.093104 - 6.2e-6 * T))
    s = np.mod(s, 86400.0)
    return s * (2.0 * np.pi / 86400.0)


def detector_information(ra, dec, time, psi, detector_tensors, detector_vertex):
    """get_detector_information (eob/seobnrv4phm.py:597-634): F+, Fx and the
    delay from the geocenter, each [nch, B]."""
    gmst = np.fmod(gmst_from_gps(time), 2 * np.pi)
    phi = np.asarray(ra) - gmst
    theta = np.pi / 2 - np.asarray(dec)
    psi = np.asarray(psi)
    u = np.array([np.cos(phi) * np.cos(theta), np.cos(theta) * np.sin(phi), -np.sin(theta)]).T
    v = np.array([-np.sin(phi), np.cos(phi), np.zeros_like(phi)]).T
    m = -u * np.sin(psi)[:, None] - v * np.cos(psi)[:, None]
    n = -u * np.cos(psi)[:, None] + v * np.sin(psi)[:, None]
    ep = np.einsum("...i,...j->...ij", m, m) - np.einsum("...i,...j->...ij", n, n)
    ex = np.einsum("...i,...j->...ij", m, n) + np.einsum("...i,...j->...ij", n, m)
    Fp = np.einsum("kij,lij->kl", detector_tensors, ep)
    Fx = np.einsum("kij,lij->kl", detector_tensors, ex)
    omega = np.array([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)]).T
    tau = np.einsum("ij,kj->ki", omega, detector_vertex) / SPEED_OF_LIGHT
    return Fp, Fx, tau


def fd_get_ll(h_td, data, psd, ra, dec, psi, time, detector_tensors, detector_vertex, sampling_frequency,
              start_ind=0):
    """The rest of get_ll (eob/seobnrv4phm.py:736-744, 778-817) from the summed
    time-domain strain h_td [B, N] (complex: plus = real, cross = imaginary):
    two real FFTs, bins below start_ind zeroed, detector projection, PSD-
    weighted residual, lnL = -1/2 df 4 sum.  data, psd: [nch, N/2 + 1]."""
    B, N = h_td.shape
    nch = data.shape[0]
    hp = np.fft.rfft(h_td.real, axis=-1)
    hc = np.fft.rfft(h_td.imag, axis=-1)
    hp[:, :start_ind] = 0.0
    hc[:, :start_ind] = 0.0
    Fp, Fx, tau = detector_information(ra, dec, time, psi, detector_tensors, detector_vertex)
    Nf = hp.shape[1]
    df = 1.0 / (N / sampling_frequency)
    temp = all_in_one_likelihood(hp.ravel(), hc.ravel(), data.ravel(), psd.ravel(), Fp.ravel(), Fx.ravel(),
                                 tau.ravel(), df, B, nch, Nf)
    return fd_lnl(temp, df, B, nch).real
