"""The allocation-free entry point (eob_waveform_lnl_noalloc), for callers that
cannot allocate device memory (a framework's memory pool, a plugin host
without allocator access): through the C ABI, its lnL must equal the regular
entry point's on the same inputs, on two calls in a row (the shared scratch
keeps the first call's contents), calls beyond its fixed limits must be
refused without touching the outputs, and a binary longer than its 4096
trajectory rows must end exactly as the regular entry point does at the same
row capacity.  Collected last so that a failure here never hides the other
GPU tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(golden):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    c = golden["config1"]
    P = torch.tensor(c["params"], dtype=torch.float64, device="cuda")
    D = torch.tensor(c["data"], dtype=torch.float64, device="cuda")
    wl = WaveformLikelihood(max_batch=len(P), max_steps=4096, modes=[(2, 2)], max_samples=int(c["N"]))
    ref, st = wl.run(P, D, float(c["dt"]), float(c["amp"]))
    torch.cuda.synchronize()
    return torch, _lib, P, D, c, ref.cpu().numpy(), st.cpu().numpy()


def _call(torch, lib, P, D, c, B, K=1, N=None):
    lnl = torch.full((B,), float("nan"), dtype=torch.float64, device="cuda")
    st = torch.full((B,), -1, dtype=torch.int32, device="cuda")
    ells = (ctypes.c_int * 2)(2, 2)
    mms = (ctypes.c_int * 2)(2, 1)
    N = int(c["N"]) if N is None else N
    rc = lib.load().eob_waveform_lnl_noalloc(ctypes.c_void_p(P.data_ptr()), B, ells, mms, K, float(c["dt"]),
                                             ctypes.c_void_p(D.data_ptr()), N, float(c["amp"]), None,
                                             ctypes.c_void_p(lnl.data_ptr()), ctypes.c_void_p(st.data_ptr()),
                                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc, lnl.cpu().numpy(), st.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice(setup):
    torch, lib, P, D, c, ref, ref_st = setup
    B = P.shape[0]
    for _ in range(2):
        rc, lnl, st = _call(torch, lib, P, D, c, B)
        assert rc == 0
        np.testing.assert_array_equal(st, ref_st)
        assert np.all(np.abs(lnl / ref - 1) < 1e-9), (lnl, ref)
        # and the reference's own likelihood (golden, FP64 tolerance)
        assert np.all(np.abs(lnl / c["lnl"] - 1) < 1e-9), (lnl, c["lnl"])
    # a smaller batch after a larger one: stale scratch must not leak in
    rc, lnl, st = _call(torch, lib, P[:3].contiguous(), D, c, 3)
    assert rc == 0
    assert np.all(np.abs(lnl / ref[:3] - 1) < 1e-9)


def test_noalloc_refuses_oversize(setup):
    """More than 16 binaries, more than one mode or more than 8192 samples:
    EOB_E_ARG (1), outputs untouched."""
    torch, lib, P, D, c, ref, ref_st = setup
    big = P.repeat(3, 1).contiguous()  # 24 binaries > 16
    rc, lnl, st = _call(torch, lib, big, D, c, big.shape[0])
    assert rc == 1 and np.all(np.isnan(lnl)) and np.all(st == -1)
    rc, lnl, st = _call(torch, lib, P, D, c, P.shape[0], K=2)
    assert rc == 1 and np.all(np.isnan(lnl)) and np.all(st == -1)
    D_long = torch.zeros(8193, dtype=torch.float64, device="cuda")
    rc, lnl, st = _call(torch, lib, P, D_long, c, P.shape[0], N=8193)
    assert rc == 1 and np.all(np.isnan(lnl)) and np.all(st == -1)


def test_noalloc_long_trajectory_ends_like_regular(setup):
    """A 10 Msun, q = 4, chi = 0.8 binary from 10 Hz needs about 8700 rows:
    past the 4096-row limit it ends with EOB_ST_MAXSTEP, and status and lnL
    equal the regular entry point's at max_steps = 4096."""
    torch, lib, P, D, c, ref, ref_st = setup
    from eobgpu_gb300.pipeline import WaveformLikelihood
    long_p = torch.tensor([[8.0, 2.0, 0.8, 0.8, 10.0], list(c["params"][0])], dtype=torch.float64, device="cuda")
    wl = WaveformLikelihood(max_batch=2, max_steps=4096, modes=[(2, 2)], max_samples=int(c["N"]))
    lr, sr = wl.run(long_p, D, float(c["dt"]), float(c["amp"]))
    lr, sr = lr.cpu().numpy(), sr.cpu().numpy()
    assert sr[0] & 2, sr  # EOB_ST_MAXSTEP
    assert sr[1] == 0
    rc, lnl, st = _call(torch, lib, long_p, D, c, 2)
    assert rc == 0
    np.testing.assert_array_equal(st, sr)
    np.testing.assert_allclose(lnl, lr, rtol=1e-9, equal_nan=True)
