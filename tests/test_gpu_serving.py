"""Serving (configuration 4 shape, scaled down): continuous batching over two
concurrent slots replays a seeded Poisson trace; every request completes with
status 0, and a request's lnL is bitwise the same alone and packed with
others (the lanes per binary are fixed by the server)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def server():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import workload
    from eobgpu_gb300.pipeline import WaveformLikelihood
    from eobgpu_gb300.serving import LikelihoodServer
    cfg = workload.CONFIGS[1]
    inj = workload.injection_params(cfg)
    wl = WaveformLikelihood(1, 4000, [(2, 2)], cfg.n_samples)
    h, _ = wl.strain(torch.tensor(inj[None, :], device="cuda"), cfg.dt, cfg.n_samples)
    data, amp = workload.make_data(h[0].real.cpu().numpy(), cfg.n_samples, cfg.index)
    return LikelihoodServer(data, cfg.dt, amp, max_batch=96, max_steps=4000, slots=2, lanes_per_binary=8)


def test_alone_vs_in_mix_bitwise(server):
    from eobgpu_gb300 import workload
    tr = workload.serving_trace(12, 1000.0, stream=3)
    reqs = [p[:40] for p in tr.params]
    alone = [server.evaluate(r)[0] for r in reqs]
    # all at once: requests get packed together (and split over batches of 96)
    res = server.run_trace(np.zeros(len(reqs)), reqs)
    for a, b, s in zip(alone, res["lnl"], res["status"]):
        assert np.all(s == 0)
        assert np.array_equal(a, b)


def test_trace_replay(server):
    from eobgpu_gb300 import workload
    tr = workload.serving_trace(30, 200.0, stream=4)
    reqs = [p[:64] for p in tr.params]
    res = server.run_trace(tr.arrivals, reqs)
    assert all(np.all(s == 0) for s in res["status"])
    assert all(np.all(np.isfinite(l)) for l in res["lnl"])
    assert np.all(res["latency_s"] > 0)
    assert res["p99_ms"] >= res["p50_ms"] > 0
    assert res["binaries"] == sum(len(r) for r in reqs)


def test_classes_requeue_matches_single_class(server):
    """Two trajectory-length classes with a deliberately short first class:
    binaries that outgrow it (status MAXSTEP) are re-run in the second, and
    every lnL equals the single-class server's bitwise."""
    from eobgpu_gb300 import workload
    from eobgpu_gb300.serving import LikelihoodServer
    tr = workload.serving_trace(6, 1000.0, stream=6)
    reqs = [p[:48] for p in tr.params]
    ref = server.run_trace(np.zeros(len(reqs)), reqs)
    cls = LikelihoodServer(server.data.cpu().numpy(), server.dt, server.amp, classes=[(350, 64, 1), (4000, 96, 1)],
                           lanes_per_binary=8, row_safety=0.3)
    res = cls.run_trace(np.zeros(len(reqs)), reqs)
    assert res["requeued"] > 0
    for a, b, s in zip(ref["lnl"], res["lnl"], res["status"]):
        assert np.all(s == 0)
        assert np.array_equal(a, b)
