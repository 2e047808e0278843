"""Memory-admitted chunking (the configuration-5 mechanism, scaled down): a
batch run in chunks over two streams gives bitwise the lnL of one launch
when the lanes per binary are fixed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_chunked_equals_single_launch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import _lib, workload
    from eobgpu_gb300.pipeline import WaveformLikelihood, lnl_chunked
    cfg = workload.CONFIGS[1]
    params = workload.draw_params(cfg, batch=24, stream=5)
    inj = workload.injection_params(cfg)
    wl1 = WaveformLikelihood(1, 4000, [(2, 2)], cfg.n_samples)
    h, _ = wl1.strain(torch.tensor(inj[None, :], device="cuda"), cfg.dt, cfg.n_samples)
    data, amp = workload.make_data(h[0].real.cpu().numpy(), cfg.n_samples, cfg.index)
    opts = _lib.default_options()
    opts.lanes_per_binary = 4
    P = torch.tensor(params, device="cuda")
    D = torch.tensor(data, device="cuda")
    wl = WaveformLikelihood(24, 4000, [(2, 2)], cfg.n_samples, options=opts)
    ref, st = wl.run(P, D, cfg.dt, amp)
    budget = 2 * _lib.load().eob_workspace_bytes(7, 4000, 1, cfg.n_samples)
    lnl, st2, info = lnl_chunked(P, D, cfg.dt, amp, max_steps=4000, hbm_budget_bytes=budget, slots=2, options=opts)
    torch.cuda.synchronize()
    assert info["chunk"] == 7 and info["chunks"] == 4 and info["slots"] == 2
    assert np.all(st2.cpu().numpy() == 0)
    assert np.array_equal(lnl.cpu().numpy(), ref.cpu().numpy())


def test_chunked_with_head_equals_single_launch():
    """The longest binaries on their own concurrent workspace (same lanes per
    binary here, so the results must not move)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from eobgpu_gb300 import _lib, workload
    from eobgpu_gb300.pipeline import WaveformLikelihood, lnl_chunked
    cfg = workload.CONFIGS[1]
    params = workload.draw_params(cfg, batch=24, stream=8)
    data = workload.rng(1, 7).standard_normal(cfg.n_samples)
    opts = _lib.default_options()
    opts.lanes_per_binary = 4
    P = torch.tensor(params, device="cuda")
    D = torch.tensor(data, device="cuda")
    wl = WaveformLikelihood(24, 4000, [(2, 2)], cfg.n_samples, options=opts)
    ref, _ = wl.run(P, D, cfg.dt, 1.0)
    budget = 2 * _lib.load().eob_workspace_bytes(8, 4000, 1, cfg.n_samples) + \
        _lib.load().eob_workspace_bytes(5, 4000, 1, cfg.n_samples)
    lnl, st, info = lnl_chunked(P, D, cfg.dt, 1.0, max_steps=4000, hbm_budget_bytes=budget, slots=2, options=opts,
                                head=5, head_lanes=4)
    torch.cuda.synchronize()
    assert info["head"] == 5 and info["chunk"] == 8
    assert np.all(st.cpu().numpy() == 0)
    assert np.array_equal(lnl.cpu().numpy(), ref.cpu().numpy())
