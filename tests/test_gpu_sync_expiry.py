"""Bounded waits of the multi-warp integrator.

The warp-pair and four-warp integrators exchange values through a group
barrier (an mbarrier) whose wait is limited in time; a warp whose wait runs
out marks itself failed and skips every later barrier, and the integrator
ends that binary with EOB_ST_SYNC instead of hanging.  Through
eob_sync_expiry_hook (the same barrier function with a 1 ms limit), one warp
of chosen groups leaves without arriving; the test checks that the launch
returns, that exactly the other warps of those groups report the expiry after
waiting at least the limit, that every other group passes all its barriers
with every exchanged value intact, and that the context stays usable: a
warp-pair integration after the hook is bitwise equal to one before it."""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT_NS = 1_000_000  # 1 ms


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _pair_run(torch, c):
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    o = _lib.default_options()
    o.lanes_per_binary = 64
    o.head_quads = 0
    wl = WaveformLikelihood(max_batch=8, max_steps=4000, modes=[(2, 2)], max_samples=int(c["N"]), options=o)
    P = torch.tensor(c["params"], dtype=torch.float64, device="cuda")
    D = torch.tensor(c["data"], dtype=torch.float64, device="cuda")
    lnl, st = wl.run(P, D, float(c["dt"]), float(c["amp"]))
    torch.cuda.synchronize()
    return lnl.cpu().numpy(), st.cpu().numpy()


@pytest.mark.parametrize("group_warps", [2, 4])
def test_group_barrier_wait_runs_out(torch_cuda, golden, group_warps):
    torch = torch_cuda
    from eobgpu_gb300 import _lib
    lib = _lib.load()
    c = golden["config1"]
    before = _pair_run(torch, c)

    blocks, rounds, skip_round, skip_warp = 4, 16, 5, 1
    groups = blocks * 8 // group_warps
    skip = {1, groups - 2}
    mask = sum(1 << g for g in skip)
    out = torch.full((blocks * 8 * 4,), -7, dtype=torch.int32, device="cuda")
    t0 = time.perf_counter()
    rc = lib.eob_sync_expiry_hook(group_warps, rounds, mask, skip_round, skip_warp, LIMIT_NS,
                                  ctypes.c_void_p(out.data_ptr()), blocks,
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()  # the launch returns (raises on a device error)
    wall = time.perf_counter() - t0
    assert rc == 0
    assert wall < 5.0, wall
    o = out.view(blocks * 8, 4).cpu().numpy()
    for w in range(blocks * 8):
        g, role = w // group_warps, w % group_warps
        ok, passed, bad, waited_us = o[w]
        assert bad == 0, (w, o[w])
        if g in skip and role == skip_warp:
            # the warp that left: it never waited in vain
            assert (ok, passed, waited_us) == (1, skip_round, 0), (w, o[w])
        elif g in skip:
            # its partners: the wait at round skip_round ran out after the limit
            assert ok == 0 and passed == skip_round, (w, o[w])
            assert waited_us >= LIMIT_NS // 1000, (w, o[w])
            assert waited_us < 1_000_000, (w, o[w])
        else:
            assert (ok, passed, waited_us) == (1, rounds, 0), (w, o[w])

    # the context is intact: the warp-pair integrator gives the same bits
    after = _pair_run(torch, c)
    np.testing.assert_array_equal(after[1], before[1])
    np.testing.assert_array_equal(after[0], before[0])


def test_hook_rejects_bad_arguments(torch_cuda):
    torch = torch_cuda
    from eobgpu_gb300 import _lib
    lib = _lib.load()
    out = torch.zeros(8 * 4, dtype=torch.int32, device="cuda")
    p = ctypes.c_void_p(out.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.eob_sync_expiry_hook(3, 4, 0, 0, 0, LIMIT_NS, p, 1, s) == 1      # group size
    assert lib.eob_sync_expiry_hook(2, 4, 0, 4, 0, LIMIT_NS, p, 1, s) == 1      # skip round past the end
    assert lib.eob_sync_expiry_hook(2, 4, 0, 0, 2, LIMIT_NS, p, 1, s) == 1      # skip warp outside the group
    assert lib.eob_sync_expiry_hook(2, 4, 0, 0, 0, 10, p, 1, s) == 1            # limit below 1 us
    assert lib.eob_sync_expiry_hook(2, 4, 0, 0, 0, 3_000_000_000, p, 1, s) == 1  # limit above 2 s
