"""The launch autotuner on a small batch: it times lanes-per-binary
candidates and heads of four-warp groups beside lane groups, and the options
it returns give the same lnL as a direct run with those options."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_autotune_small_batch(torch_cuda, golden):
    torch = torch_cuda
    from eobgpu_gb300 import _lib, autotune
    from eobgpu_gb300.pipeline import WaveformLikelihood
    c = golden["config1"]
    P = torch.tensor(c["params"], device="cuda")
    D = torch.tensor(c["data"], device="cuda")
    r = autotune.tune(P, D, float(c["dt"]), float(c["amp"]), max_steps=4096, lanes=(8, 64), blocks=(128,),
                      spline_tiles=(4,), heads=(2,))
    assert r.lanes_per_binary in (8, 16, 32, 64) and r.head_quads in (-1, 2) and r.ms > 0
    heads = [e for e in r.table if e["head_quads"] == 2]
    assert heads, r.table  # a head was timed beside lane groups
    opt = r.options()
    wl = WaveformLikelihood(8, 4096, [(2, 2)], int(c["N"]), options=opt)
    lnl, st = wl.run(P, D, float(c["dt"]), float(c["amp"]))
    assert np.all(st.cpu().numpy() == 0)
    assert np.all(np.abs(lnl.cpu().numpy() / c["lnl"] - 1) < 1e-9)
