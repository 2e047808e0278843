"""Host logic of the request server: batch packing (arrival order, large
requests split), routing by estimated trajectory length, slot admission
against an HBM budget, and the serving trace generator."""
import collections

import numpy as np
import pytest

from eobgpu_gb300 import workload

serving = pytest.importorskip("eobgpu_gb300.serving")


def _q(sizes):
    return collections.deque([[i, np.arange(s), 0] for i, s in enumerate(sizes)])


def test_pack_in_order_and_split():
    q = _q([3, 4, 2, 10])
    b1 = serving.pack_batch(q, 8)
    assert [(p.req, list(p.idx)) for p in b1] == [(0, [0, 1, 2]), (1, [0, 1, 2, 3]), (2, [0])]
    b2 = serving.pack_batch(q, 8)
    assert [(p.req, list(p.idx)) for p in b2] == [(2, [1]), (3, list(range(7)))]
    b3 = serving.pack_batch(q, 8)
    assert [(p.req, list(p.idx)) for p in b3] == [(3, [7, 8, 9])]
    assert not q


def test_pack_covers_every_row_once():
    rng = np.random.default_rng(5)
    sizes = list(rng.integers(1, 513, 200))
    q = _q(sizes)
    seen = [np.zeros(s, dtype=int) for s in sizes]
    while q:
        b = serving.pack_batch(q, 700)
        assert sum(len(p.idx) for p in b) <= 700
        for p in b:
            seen[p.req][p.idx] += 1
    assert all(np.all(s == 1) for s in seen)


def test_estimate_rows_bounds_configuration2():
    # the fit with its safety factor covers the measured rows of configuration 2
    cfg = workload.CONFIGS[2]
    p = workload.draw_params(cfg)
    est = serving.estimate_rows(p)
    assert np.all(est > 200) and np.all(est < 40000)
    # longer chirps get longer estimates
    short = serving.estimate_rows(np.array([[100.0, 90.0, 0.0, 0.0, 20.0]]))
    long_ = serving.estimate_rows(np.array([[12.0, 10.0, 0.0, 0.0, 10.0]]))
    assert long_[0] > 3 * short[0]


def test_route_and_admission():
    caps = [500, 2000, 8000]
    c = serving.route(np.array([10, 500, 501, 1999, 2000, 7999, 8000, 10 ** 6]), caps)
    assert list(c) == [0, 0, 1, 1, 1, 2, 2, 2]
    assert serving.admit_slots([10, 20, 40], [2, 2, 2], 1000) == [2, 2, 2]
    assert serving.admit_slots([10, 20, 40], [2, 2, 2], 100) == [2, 2, 1]
    assert serving.admit_slots([10, 20, 40], [3, 3, 3], 75) == [1, 1, 1]
    with pytest.raises(Exception):
        serving.admit_slots([10, 20, 40], [1, 1, 1], 60)


def test_serving_trace_is_seeded():
    a = workload.serving_trace(50, 20.0, stream=1)
    b = workload.serving_trace(50, 20.0, stream=1)
    assert np.array_equal(a.arrivals, b.arrivals) and np.array_equal(a.sizes, b.sizes)
    assert np.all(np.diff(a.arrivals) > 0)
    assert all(p.shape == (s, 5) for p, s in zip(a.params, a.sizes))
    assert all(np.all(p[:, 0] >= p[:, 1]) for p in a.params)
    assert np.all((a.sizes >= 1) & (a.sizes <= 512))
