"""Drop-in for the reference's `eob.pytdinterp` extension (src/tdinterp.pyx)."""
from __future__ import annotations

from .. import _lib
from ._ptr import addr, stream


def interpolate_TD_wrap(t_arr, propArrays, B, upper_diag, diag, lower_diag, lengths, numBinAll, nsubs):
    """src/tdinterp.pyx:21: batched not-a-knot splines; c1/c2/c3 land in
    upper_diag/diag/lower_diag as in the reference."""
    _lib.check(_lib.load().eob_interpolate_td(addr(t_arr), addr(propArrays), addr(B), addr(upper_diag), addr(diag),
                                              addr(lower_diag), addr(lengths), int(numBinAll), int(nsubs), stream()),
               "interpolate_TD_wrap")


def TDInterp_wrap(*args, **kwargs):
    raise NotImplementedError("TDInterp (stream-per-binary synthesis, src/interpolate.cu:317-438) is unused by the "
                              "reference's pipeline; the fused synthesis of eob_synth_lnl/eob_synth_strain replaces it")


def TDInterp_wrap2(*args, **kwargs):
    raise NotImplementedError("TDInterp_wrap2 (src/interpolate.cu:440-549): use eob_synth_strain (per-mode or summed "
                              "uniform-grid synthesis) through eob.seobnrv4phm")


def all_in_one_likelihood(*args, **kwargs):
    raise NotImplementedError("the frequency-domain likelihood (src/interpolate.cu:551-627) is not part of the "
                              "time-domain white-noise path built here")
