"""The fused path captured as a CUDA graph: replays on new parameters copied
into the captured input give bitwise the eager result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_graph_replay_matches_eager():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import _lib, workload
    from eobgpu_gb300.pipeline import WaveformLikelihood
    cfg = workload.CONFIGS[1]
    inj = workload.injection_params(cfg)
    wl0 = WaveformLikelihood(1, 4000, [(2, 2)], cfg.n_samples)
    h, _ = wl0.strain(torch.tensor(inj[None, :], device="cuda"), cfg.dt, cfg.n_samples)
    data, amp = workload.make_data(h[0].real.cpu().numpy(), cfg.n_samples, cfg.index)
    D = torch.tensor(data, device="cuda")
    opts = _lib.default_options()
    opts.lanes_per_binary = 8
    wl = WaveformLikelihood(16, 4000, [(2, 2)], cfg.n_samples, options=opts)
    batches = [torch.tensor(workload.draw_params(cfg, batch=16, stream=s), device="cuda") for s in (11, 12, 13)]
    eager = [wl.run(b, D, cfg.dt, amp)[0].cpu().numpy() for b in batches]
    P = batches[0].clone()
    g = wl.capture(P, D, cfg.dt, amp)
    for b, ref in zip(batches[::-1], eager[::-1]):
        P.copy_(b)
        lnl, st = g.replay()
        torch.cuda.synchronize()
        assert np.all(st.cpu().numpy() == 0)
        assert np.array_equal(lnl.cpu().numpy(), ref)
