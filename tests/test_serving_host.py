"""Host logic of the request server: batch packing (whole requests in arrival
order, large requests split) and the serving trace generator."""
import collections

import numpy as np

from eobgpu_gb300 import workload


def _pack():
    # the module imports torch; packing itself is plain Python
    from eobgpu_gb300.serving import pack_batch
    return pack_batch


def test_pack_whole_requests_in_order():
    pack = _pack()
    sizes = [3, 4, 2, 10]
    q = collections.deque([[0, 0], [1, 0], [2, 0], [3, 0]])
    b1 = pack(q, sizes, 8)
    assert [(p.req, p.lo, p.hi) for p in b1] == [(0, 0, 3), (1, 0, 4), (2, 0, 1)]
    assert list(q)[0] == [2, 1]
    b2 = pack(q, sizes, 8)
    assert [(p.req, p.lo, p.hi) for p in b2] == [(2, 1, 2), (3, 0, 7)]
    b3 = pack(q, sizes, 8)
    assert [(p.req, p.lo, p.hi) for p in b3] == [(3, 7, 10)]
    assert not q


def test_pack_covers_every_row_once():
    pack = _pack()
    rng = np.random.default_rng(5)
    sizes = list(rng.integers(1, 513, 200))
    q = collections.deque([[i, 0] for i in range(len(sizes))])
    seen = [np.zeros(s, dtype=int) for s in sizes]
    while q:
        b = pack(q, sizes, 700)
        assert sum(p.hi - p.lo for p in b) <= 700
        for p in b:
            seen[p.req][p.lo:p.hi] += 1
    assert all(np.all(s == 1) for s in seen)


def test_serving_trace_is_seeded():
    a = workload.serving_trace(50, 20.0, stream=1)
    b = workload.serving_trace(50, 20.0, stream=1)
    assert np.array_equal(a.arrivals, b.arrivals) and np.array_equal(a.sizes, b.sizes)
    assert np.all(np.diff(a.arrivals) > 0)
    assert all(p.shape == (s, 5) for p, s in zip(a.params, a.sizes))
    assert all(np.all(p[:, 0] >= p[:, 1]) for p in a.params)
    assert np.all((a.sizes >= 1) & (a.sizes <= 512))
