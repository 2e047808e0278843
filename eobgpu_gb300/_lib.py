"""ctypes binding of libeobgb300.so (include/eobgb300.h).

There is no CPU fallback: if the library has not been built, or no CUDA
device is visible, loading fails with an error that says so.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libeobgb300.so")

c_double = ctypes.c_double
c_int = ctypes.c_int
c_size_t = ctypes.c_size_t
c_void_p = ctypes.c_void_p
c_ll = ctypes.c_longlong


class EobOptions(ctypes.Structure):
    _fields_ = [("rtol", c_double), ("atol", c_double), ("h_init", c_double), ("step_back", c_double),
                ("fine_step", c_double), ("ic_mode", c_int), ("precision", c_int), ("block", c_int),
                ("grid", c_int), ("max_tries", c_ll), ("lanes_per_binary", c_int), ("spline_tile", c_int),
                ("head_quads", c_int), ("imr", c_int)]


class EobViews(ctypes.Structure):
    _fields_ = [("bins", c_void_p), ("traj", c_void_p), ("nsteps", c_void_p), ("status", c_void_p), ("npts", c_void_p),
                ("row_off", c_void_p), ("tin", c_void_p), ("spline_y", c_void_p), ("spline_c1", c_void_p),
                ("spline_c2", c_void_p), ("spline_c3", c_void_p), ("row_capacity", c_int),
                ("rows_capacity", c_ll), ("nsubs", c_int), ("rhs", c_void_p)]


# name -> (restype, argtypes); every pointer is passed as an integer address
_P = c_void_p
_SIGS = {
    "eob_options_default": (None, [ctypes.POINTER(EobOptions)]),
    "eob_workspace_bytes": (c_size_t, [c_int, c_int, c_int, c_int]),
    "eob_workspace_bytes_imr": (c_size_t, [c_int, c_int, c_int, c_int]),
    "eob_waveform_lnl": (c_int, [_P, c_size_t, c_int, c_int, c_int, c_int, _P, _P, c_int, _P, _P, c_int, c_double,
                                 _P, c_int, c_double, ctypes.POINTER(EobOptions), _P, _P, _P]),
    "eob_waveform_strain": (c_int, [_P, c_size_t, c_int, c_int, c_int, c_int, _P, _P, c_int, _P, _P, c_int,
                                    c_double, c_int, ctypes.POINTER(EobOptions), _P, _P, _P]),
    "eob_prepare": (c_int, [_P, c_size_t, c_int, c_int, c_int, c_int, _P, _P, c_int, _P, _P, c_int, c_double,
                            ctypes.POINTER(EobOptions), _P, _P]),
    "eob_prepare_stages": (c_int, [_P, c_size_t, c_int, c_int, c_int, c_int, _P, _P, c_int, _P, _P, c_int,
                                   c_double, ctypes.POINTER(EobOptions), c_int, _P]),
    "eob_synth_lnl": (c_int, [_P, c_size_t, c_int, c_int, c_int, c_int, c_int, _P, c_int, c_double, _P, c_int,
                              c_double, ctypes.POINTER(EobOptions), _P, _P, _P]),
    "eob_synth_strain": (c_int, [_P, c_size_t, c_int, c_int, c_int, c_int, c_int, _P, c_int, c_double, c_int, c_int,
                                 _P, _P, _P]),
    "eob_workspace_counters": (c_int, [_P, c_int, c_int, c_int, c_int, _P, _P]),
    "eob_fp64_probe": (c_int, [_P, c_int, c_int, c_int, _P]),
    "eob_math_probe": (c_int, [_P, c_int, _P, _P]),
    "eob_sync_expiry_hook": (c_int, [c_int, c_int, ctypes.c_uint, c_int, c_int, c_ll, _P, c_int, _P]),
    "eob_noalloc_scratch_bytes": (c_size_t, []),
    "eob_waveform_lnl_noalloc": (c_int, [_P, c_int, _P, _P, c_int, c_double, _P, c_int, c_double,
                                         ctypes.POINTER(EobOptions), _P, _P, _P]),
    "eob_workspace_views": (c_int, [_P, c_int, c_int, c_int, c_int, ctypes.POINTER(EobViews)]),
    "eob_evaluate_ham": (c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P, c_double, c_double, c_double, c_double, c_int,
                                 _P]),
    "eob_grad_ham": (c_int, [_P, _P, _P, c_int, _P]),
    "eob_hessian_ham": (c_int, [_P, _P, _P, c_int, _P]),
    "eob_ic_cons": (c_int, [_P, _P, _P, _P, _P, c_int, _P]),
    "eob_root_find_all": (c_int, [_P, _P, _P, _P, c_int, c_double, c_int, c_int, c_int, c_int, _P]),
    "eob_ctx_bytes": (c_size_t, [c_int]),
    "eob_ctx_update_information": (c_int, [_P, _P, _P, _P, _P, _P, _P, c_int, c_int, _P]),
    "eob_ctx_ode": (c_int, [_P, _P, _P, _P, _P, c_int, _P, _P]),
    "eob_ctx_rr_force": (c_int, [_P, _P, _P, _P, _P, c_int, _P, _P]),
    "eob_ctx_root_find_scalar_all": (c_int, [_P, _P, _P, _P, _P, c_int, c_double, c_int, c_int, c_int, c_int, _P]),
    "eob_ctx_compute_hlms": (c_int, [_P] * 11 + [c_int, _P, _P, c_int, c_int, _P, c_int, _P, _P]),
    "eob_ctx_waveform": (c_int, [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P, c_int, c_int, _P, c_double, c_int, c_int,
                                 _P, _P]),
    "eob_dopr853_steps": (c_int, [_P] * 17 + [c_int, c_int, c_int, _P, _P, _P]),
    "eob_dopr853_error": (c_int, [_P] * 12 + [c_int, c_int, _P]),
    "eob_dopr853_controller": (c_int, [_P] * 6 + [c_int, c_int, _P]),
    "eob_interpolate_td": (c_int, [_P] * 7 + [c_int, c_int, _P]),
    "eob_tdinterp2": (c_int, [_P] * 7 + [c_int, _P, c_int, c_int, c_int, _P, _P, _P, _P, c_int, _P]),
    "eob_tdinterp": (c_int, [_P] * 8 + [c_int, c_int, c_int, _P, _P, _P, _P, _P, _P]),
    "eob_all_in_one_likelihood": (c_int, [_P] * 8 + [c_double, c_int, c_int, c_int, _P]),
    "eob_detector_response": (c_int, [_P] * 6 + [c_int, c_int, _P, _P, _P, _P]),
    "eob_fd_lnl_scratch_bytes": (c_size_t, [c_int, c_int]),
    "eob_fd_lnl_from_fft": (c_int, [_P, c_int, c_int, _P, _P, _P, _P, _P, c_double, c_int, c_int, _P, c_size_t, _P,
                                    _P]),
}

_lib = None


class EOBError(RuntimeError):
    pass


def load():
    """The loaded library (raises if it is missing: build it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise EOBError(f"{LIB_PATH} is missing: build the CUDA extension with "
                       "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int, what: str):
    if rc != 0:
        raise EOBError(f"{what} failed with status {rc}")


def default_options() -> EobOptions:
    o = EobOptions()
    load().eob_options_default(ctypes.byref(o))
    return o
