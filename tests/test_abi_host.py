"""The C-ABI library on the host (no GPU): it loads, exports every function
include/eobgb300.h declares, the ctypes mirror matches the C struct layouts,
and the host-only entry points (defaults, workspace sizing) behave."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from eobgpu_gb300 import _lib

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HEADER = os.path.join(ROOT, "include", "eobgb300.h")


def _declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|size_t|void)\s+\**(eob_[a-z0-9_]+)\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("native library not built")
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib._SIGS, f"{n} has no ctypes signature"


def test_struct_layouts_match_header(lib):
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "eobgb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(eob_options), offsetof(eob_options, ic_mode),
         offsetof(eob_options, max_tries), offsetof(eob_options, lanes_per_binary), sizeof(eob_views));
  printf("%zu %zu %zu %zu\n", offsetof(eob_views, row_capacity), offsetof(eob_views, rows_capacity),
         offsetof(eob_views, nsubs), offsetof(eob_views, rhs));
  return 0;
}
"""
    cuda_inc = "/usr/local/cuda/include"
    if not os.path.isdir(cuda_inc):
        pytest.skip("CUDA headers not found")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "l")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, c, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    o, v = _lib.EobOptions, _lib.EobViews
    want = [ctypes.sizeof(o), o.ic_mode.offset, o.max_tries.offset, o.lanes_per_binary.offset, ctypes.sizeof(v),
            v.row_capacity.offset, v.rows_capacity.offset, v.nsubs.offset, v.rhs.offset]
    assert [int(x) for x in out] == want


def test_default_options(lib):
    o = _lib.default_options()
    # the reference's controller and two-pass constants
    assert o.rtol == 1e-12 and o.atol == 1e-12
    assert o.h_init == 0.01 and o.step_back == 10.0 and o.fine_step == 0.05
    assert o.ic_mode == 0 and o.precision == 0


def test_workspace_sizing(lib):
    f = lib.eob_workspace_bytes
    a = f(8, 4000, 1, 8192)
    assert a > 0 and a % 256 == 0
    assert f(16, 4000, 1, 8192) > a
    assert f(8, 8000, 1, 8192) > a
    assert f(8, 4000, 5, 8192) > a
    assert f(8, 4000, 1, 1 << 17) > a
    # invalid dimensions are refused with 0
    assert f(0, 4000, 1, 8192) == 0
    assert f(8, 4000, 6, 8192) == 0


def test_noalloc_scratch_is_static(lib):
    n = lib.eob_noalloc_scratch_bytes()
    assert n >= lib.eob_workspace_bytes(16, 4096, 1, 8192)


def test_product_refuses_without_library(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(_lib.EOBError):
        _lib.load()


def test_chunk_size_for_budget(lib):
    from eobgpu_gb300.pipeline import chunk_size_for_budget
    f = lib.eob_workspace_bytes
    for B in (1, 7, 100, 4096):
        budget = f(B, 16000, 1, 1 << 20)
        assert chunk_size_for_budget(budget, 16000, 1, 1 << 20, 10 ** 6) == B
        assert chunk_size_for_budget(budget - 1, 16000, 1, 1 << 20, 10 ** 6) == B - 1
    assert chunk_size_for_budget(10, 16000, 1, 1 << 20, 100) == 0


def test_invalid_arguments_are_refused_before_any_launch(lib):
    """eob_waveform_lnl and the allocation-free entry point check every size,
    pointer and mode before any CUDA call, so the refusals run on the host:
    EOB_E_ARG (1), outputs untouched.  Host buffers stand in for device ones
    (nothing is dereferenced)."""
    import numpy as np
    E_ARG = 1
    mb, ms, mk, mn = 4, 100, 1, 64
    wsb = lib.eob_workspace_bytes(mb, ms, mk, mn)
    ws = np.zeros(16, dtype=np.uint8)
    params = np.zeros((mb, 5))
    data = np.zeros(mn)
    lnl = np.full(mb, 7.0)
    st = np.full(mb, 7, dtype=np.int32)
    P = lambda a: a.ctypes.data if a is not None else None

    def call(ws_=ws, wsb_=wsb, mb_=mb, ms_=ms, mk_=mk, mn_=mn, params_=params, B=2, ells=(2,), mms=(2,), dt=1e-3,
             data_=data, N=mn, lnl_=lnl, opt=None):
        e = np.ascontiguousarray(ells, dtype=np.int32)
        m = np.ascontiguousarray(mms, dtype=np.int32)
        return lib.eob_waveform_lnl(P(ws_), wsb_, mb_, ms_, mk_, mn_, P(params_), None, B, P(e), P(m), len(e), dt,
                                    P(data_), N, 1.0, ctypes.byref(opt) if opt is not None else None, P(lnl_),
                                    P(st), None)

    imr = _lib.default_options()
    imr.imr = 1
    cases = {
        "B = 0": dict(B=0), "B > max_batch": dict(B=mb + 1),
        "no modes": dict(ells=(), mms=()), "K > max_modes": dict(ells=(2, 2), mms=(2, 1)),
        "l > 8": dict(ells=(9,), mms=(1,)), "m > l": dict(ells=(2,), mms=(3,)), "m < 1": dict(ells=(2,), mms=(0,)),
        "dt = 0": dict(dt=0.0), "dt NaN": dict(dt=float("nan")),
        "N = 0": dict(N=0), "N > max_samples": dict(N=mn + 1),
        "no workspace": dict(ws_=None), "workspace too small": dict(wsb_=wsb - 1),
        "max_steps < 4": dict(ms_=3), "no params": dict(params_=None), "no data": dict(data_=None),
        "no lnl": dict(lnl_=None), "imr without its section": dict(opt=imr),
    }
    for name, kw in cases.items():
        assert call(**kw) == E_ARG, name
    assert np.all(lnl == 7.0) and np.all(st == 7)
    # the allocation-free entry point: at most 16 binaries, one mode, 8192 samples
    na = lib.eob_waveform_lnl_noalloc
    e = np.array([2], dtype=np.int32)
    for B, K, N in ((17, 1, 64), (0, 1, 64), (2, 2, 64), (2, 1, 8193), (2, 1, 0)):
        pp = np.zeros((max(B, 1), 5))
        ee = np.repeat(e, max(K, 1))
        out = np.full(max(B, 1), 7.0)
        assert na(P(pp), B, P(ee), P(ee), K, 1e-3, P(np.zeros(max(N, 1))), N, 1.0, None, P(out), P(st), None) == E_ARG
        assert np.all(out == 7.0)
