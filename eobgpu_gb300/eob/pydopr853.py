"""Drop-in for the reference's `eob.pydopr853` extension (src/dopr853.pyx)."""
from __future__ import annotations

from .. import _lib
from ._ptr import addr, stream


def dormandPrinceSteps(x, xCurrent, solOld, h, arg, additionalArgs, k1, k2, k3, k4, k5, k6, k7, k8, k9, k10,
                       ak_term_buffer, nargs, numEq, num_add_args, ode_class, hCoeffs_index):
    """src/dopr853.pyx:67: the 12 stages of one DOPR853 step in one launch."""
    _lib.check(_lib.load().eob_dopr853_steps(addr(x), addr(xCurrent), addr(solOld), addr(h), addr(arg),
                                             addr(additionalArgs), addr(k1), addr(k2), addr(k3), addr(k4), addr(k5),
                                             addr(k6), addr(k7), addr(k8), addr(k9), addr(k10),
                                             addr(ak_term_buffer), int(nargs), int(numEq), int(num_add_args),
                                             addr(ode_class.conceiled_ptr), addr(hCoeffs_index), stream()),
               "dormandPrinceSteps")


def error(err, solOld, solNew, h, k1, k2, k3, k6, k7, k8, k9, k10, nargs, numEq):
    """src/dopr853.pyx:139.  As in the reference, the values are forwarded in
    order into the C slots (numEq, nargs), so callers pass (numEq, nargs)
    positionally (eob/new_Dormand_horiz.py:669-670)."""
    _lib.check(_lib.load().eob_dopr853_error(addr(err), addr(solOld), addr(solNew), addr(h), addr(k1), addr(k2),
                                             addr(k3), addr(k6), addr(k7), addr(k8), addr(k9), addr(k10), int(nargs),
                                             int(numEq), stream()), "error")


def controllerSuccess(flagSuccess, err, errOld, previousReject, h, x, numEq, nargs):
    """src/dopr853.pyx:187 (bool arrays as uint8/bool tensors)."""
    _lib.check(_lib.load().eob_dopr853_controller(addr(flagSuccess), addr(err), addr(errOld), addr(previousReject),
                                                  addr(h), addr(x), int(numEq), int(nargs), stream()),
               "controllerSuccess")
