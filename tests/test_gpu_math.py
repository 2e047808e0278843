"""The hot path's own reciprocal (seed + third-order Newton step), reciprocal
cube root and step-controller eighth root (single-precision seeds +
third-order steps), table-driven log and reciprocal square root on the GPU, through eob_math_probe, against
correctly rounded references and the device library's functions."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _ulps(v, ref_hi):
    """|v - ref| in units of the last place of the float64 result, ref in
    extended precision (numpy longdouble)."""
    sp = np.spacing(np.abs(ref_hi.astype(np.float64))).astype(np.longdouble)
    return np.abs((v.astype(np.longdouble) - ref_hi) / sp).astype(np.float64)


def test_hot_path_math_accuracy(torch_cuda):
    torch = torch_cuda
    from eobgpu_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(7)
    n = 1 << 18
    x = np.concatenate([np.exp(rng.uniform(np.log(1e-6), np.log(1e6), n // 2)),  # wide range
                        rng.uniform(0.5, 2.0, n // 4),                           # one binade and its neighbours
                        rng.uniform(1.0, 40.0, n // 4)])                         # radii of the trajectories
    xd = torch.tensor(x, device="cuda")
    out = torch.empty(10 * n, dtype=torch.float64, device="cuda")
    rc = lib.eob_math_probe(ctypes.c_void_p(xd.data_ptr()), n, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(n, 10)
    xl = x.astype(np.longdouble)
    # reciprocal: faithful (within one ulp), and equal to the division in almost every case
    np.testing.assert_array_equal(o[:, 1], 1.0 / x)
    u = _ulps(o[:, 0], 1 / xl)
    assert u.max() < 1.0, u.max()
    assert np.mean(o[:, 0] == o[:, 1]) > 0.99
    # reciprocal cube root: within one ulp; within one ulp of the device's rcbrt
    u = _ulps(o[:, 2], 1 / np.cbrt(xl))
    assert u.max() < 1.0, u.max()
    assert np.max(np.abs(o[:, 2] - o[:, 3]) / np.spacing(o[:, 3])) <= 1.0
    # log (|log x| bounded away from 0 where the ulp is relative to a tiny result)
    far = np.abs(np.log(x)) > 0.1
    u = _ulps(o[far, 4], np.log(xl[far]))
    assert u.max() < 1.0, u.max()
    assert np.max(np.abs(o[:, 4] - o[:, 5])) <= 4 * np.finfo(float).eps * np.max(np.abs(o[:, 5]))
    # reciprocal square root
    u = _ulps(o[:, 6], 1 / np.sqrt(xl))
    assert u.max() < 1.0, u.max()
    # the step controller's x^(-1/8) (arguments inside its clamp [1e-30, 1e30])
    u = _ulps(o[:, 7], 1 / np.sqrt(np.sqrt(np.sqrt(xl))))
    assert u.max() < 1.0, u.max()
    # the m factors' e^(-y) - 1 (y = min(x, 600)): within 1.5e-16 absolute
    # of the extended-precision value (the table entry's rounding, the
    # rounding of S - 1 and of the last fma; at most 6e-15 relative to
    # 1 - e^(-y) >= 0.0107), and within 2 ulp where y < ln2/64 (no
    # cancellation there)
    y = np.minimum(xl, 600)
    ref = np.expm1(-y)
    err = np.abs(o[:, 8].astype(np.longdouble) - ref)
    assert err.max() < 1.5e-16, float(err.max())
    assert np.max(err / np.abs(ref)) < 6e-15, float(np.max(err / np.abs(ref)))
    small = np.asarray(y < np.log(2) / 64)
    assert small.sum() > 1000
    assert _ulps(o[small, 8], ref[small]).max() <= 2.0
    np.testing.assert_allclose(o[:, 8], o[:, 9], rtol=6e-15, atol=1.5e-16)
