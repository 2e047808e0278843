"""Drop-in for the reference's `eob.pytdinterp` extension (src/tdinterp.pyx)."""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from ._ptr import addr, stream


def interpolate_TD_wrap(t_arr, propArrays, B, upper_diag, diag, lower_diag, lengths, numBinAll, nsubs):
    """src/tdinterp.pyx:21: batched not-a-knot splines; c1/c2/c3 land in
    upper_diag/diag/lower_diag as in the reference."""
    _lib.check(_lib.load().eob_interpolate_td(addr(t_arr), addr(propArrays), addr(B), addr(upper_diag), addr(diag),
                                              addr(lower_diag), addr(lengths), int(numBinAll), int(nsubs), stream()),
               "interpolate_TD_wrap")


def _host_ll(a):
    """A host array of 64-bit integers (device addresses or counts) for the
    entry points that read per-binary metadata on the host, as the
    reference's host loop does (src/interpolate.cu:401-431)."""
    arr = np.ascontiguousarray(np.asarray([int(v) for v in a], dtype=np.int64))
    return arr, arr.ctypes.data_as(ctypes.c_void_p)


def _host_i32(a):
    arr = np.ascontiguousarray(np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.int32))
    return arr, arr.ctypes.data_as(ctypes.c_void_p)


def _dev_list(a):
    """Per-binary arrays: a sequence of device tensors / addresses."""
    return [addr(v).value or 0 for v in a]


def TDInterp_wrap(templateChannels_ptrs, dataTime, ts, propArrays, c1, c2, c3, old_lengths, data_length, numBinAll,
                  numModes, ls, ms, inds_ptrs, inds_start, ind_lengths):
    """src/tdinterp.pyx:40: per-binary synthesis (TD, src/interpolate.cu:323-438).
    templateChannels_ptrs, ts, propArrays, c1, c2, c3 and inds_ptrs are
    sequences with one device array (or address) per binary; old_lengths,
    inds_start and ind_lengths are host integer sequences; binary b writes its
    complex output from element data_length on, as the reference does."""
    keep = []
    ptrs = []
    for seq in (templateChannels_ptrs, ts, propArrays, c1, c2, c3, inds_ptrs):
        arr, p = _host_ll(_dev_list(seq))
        keep.append(arr)
        ptrs.append(p)
    ol, pol = _host_i32(old_lengths)
    st, pst = _host_i32(inds_start)
    il, pil = _host_i32(ind_lengths)
    _lib.check(_lib.load().eob_tdinterp(ptrs[0], addr(dataTime), ptrs[1], ptrs[2], ptrs[3], ptrs[4], ptrs[5], pol,
                                        int(data_length), int(numBinAll), int(numModes), addr(ls), addr(ms), ptrs[6],
                                        pst, pil, stream()), "TDInterp_wrap")


def TDInterp_wrap2(templateChannels, dataTime, ts, propArrays, c1, c2, c3, old_length, old_lengths, data_length,
                   numBinAll, numModes, ls, ms, inds, lengths, max_length):
    """src/tdinterp.pyx:60: batched synthesis (TD2, src/interpolate.cu:441-549)
    into templateChannels[numBinAll * data_length] (complex128)."""
    _lib.check(_lib.load().eob_tdinterp2(addr(templateChannels), addr(dataTime), addr(ts), addr(propArrays), addr(c1),
                                         addr(c2), addr(c3), int(old_length), addr(old_lengths), int(data_length),
                                         int(numBinAll), int(numModes), addr(ls), addr(ms), addr(inds), addr(lengths),
                                         int(max_length), stream()), "TDInterp_wrap2")


def all_in_one_likelihood(temp_sum, hp_fd, hc_fd, data, psd, Fplus, Fcross, time_shift, df, num_bin_all, nchannels,
                          data_length):
    """src/tdinterp.pyx:78: per-1024-bin partials of the frequency-domain
    residual power (src/interpolate.cu:553-627) into temp_sum (complex128,
    [ceil(data_length / 1024) * num_bin_all * nchannels])."""
    _lib.check(_lib.load().eob_all_in_one_likelihood(addr(temp_sum), addr(hp_fd), addr(hc_fd), addr(data), addr(psd),
                                                     addr(Fplus), addr(Fcross), addr(time_shift), float(df),
                                                     int(num_bin_all), int(nchannels), int(data_length), stream()),
               "all_in_one_likelihood")
