"""The reference's time-domain synthesis entry points (TDInterp_wrap2,
TDInterp_wrap) and its frequency-domain likelihood (all_in_one_likelihood)
through the C ABI, against the oracle's restatement of
src/interpolate.cu:323-627 on ragged random inputs; and the TDInterp class
and the likelihood step of the drop-in module on spline containers built from
data."""
import numpy as np
import pytest

from oracle import td_oracle as T

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _ragged_case(B, K, seed):
    rng = np.random.default_rng(seed)
    old_lengths = rng.integers(5, 60, B).astype(np.int32)
    old_length = int(old_lengths.max())
    nsubs = 2 * K + 1
    ts = np.zeros(B * old_length)
    arrs = [rng.normal(size=B * nsubs * old_length) for _ in range(4)]
    for b in range(B):
        olh = int(old_lengths[b])
        tk = np.sort(rng.uniform(0.0, 20.0, olh))
        tk[0] = 0.0
        ts[b * old_length: b * old_length + olh] = tk
        # phase series with slopes of tens of radians over the span
        base = b * nsubs * old_length + 2 * K * olh
        arrs[0][base: base + olh] = 3.0 * tk + rng.normal(size=olh)
    data_time = np.linspace(0.0, 19.0, 300)
    max_length = 300
    lengths = rng.integers(50, 300, B).astype(np.int32)
    inds = np.zeros(B * max_length, dtype=np.int32)
    for b in range(B):
        tk = ts[b * old_length: b * old_length + old_lengths[b]]
        inds[b * max_length: b * max_length + lengths[b]] = np.clip(
            np.searchsorted(tk, data_time[:lengths[b]], side="right") - 1, 0, old_lengths[b] - 1)
    ms = rng.integers(1, 6, K).astype(np.int32)
    ls = np.maximum(ms, 2).astype(np.int32)
    return data_time, ts, arrs, old_lengths, old_length, ls, ms, inds, lengths, max_length


@pytest.mark.parametrize("K", [1, 5])
def test_tdinterp2_vs_oracle(torch_cuda, K):
    torch = torch_cuda
    from eobgpu_gb300.eob import pytdinterp
    B, data_length = 7, 320
    data_time, ts, (y, c1, c2, c3), old_lengths, old_length, ls, ms, inds, lengths, max_length = _ragged_case(B, K, K)
    ref = T.td_interp2(data_time, ts, y, c1, c2, c3, old_length, old_lengths, data_length, B, K, ms, inds, lengths,
                       max_length)
    d = lambda a, dt=torch.float64: torch.tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    out = torch.zeros(B * data_length, dtype=torch.complex128, device="cuda")
    pytdinterp.TDInterp_wrap2(out, d(data_time), d(ts), d(y), d(c1), d(c2), d(c3), old_length,
                              d(old_lengths, torch.int32), data_length, B, K, d(ls, torch.int32), d(ms, torch.int32),
                              d(inds, torch.int32), d(lengths, torch.int32), max_length)
    got = out.cpu().numpy()
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= 1e-12 * scale
    for b in range(B):  # untouched past each binary's length
        assert np.all(got[b * data_length + lengths[b]: (b + 1) * data_length] == 0)


def test_tdinterp_per_binary_vs_oracle(torch_cuda):
    torch = torch_cuda
    from eobgpu_gb300.eob import pytdinterp
    B, K, data_length = 4, 3, 40
    data_time, ts, (y, c1, c2, c3), old_lengths, old_length, ls, ms, inds, lengths, max_length = _ragged_case(B, K, 9)
    nsubs = 2 * K + 1
    starts = np.array([0, 3, 10, 0], dtype=np.int32)
    lens = np.array([200, 150, 0, 90], dtype=np.int32)
    host = {k: [] for k in ("ts", "y", "c1", "c2", "c3", "inds", "out")}
    for b in range(B):
        olh = int(old_lengths[b])
        tk = ts[b * old_length: b * old_length + olh]
        host["ts"].append(tk)
        blk = slice(b * nsubs * old_length, b * nsubs * old_length + nsubs * olh)
        for name, a in (("y", y), ("c1", c1), ("c2", c2), ("c3", c3)):
            host[name].append(a[blk].copy())
        host["inds"].append(np.clip(np.searchsorted(tk, data_time[starts[b]: starts[b] + lens[b]], side="right") - 1,
                                    0, olh - 1).astype(np.int32))
        host["out"].append(np.zeros(data_length + max(lens[b], 1), dtype=np.complex128))
    ref = T.td_interp([o.copy() for o in host["out"]], data_time, host["ts"], host["y"], host["c1"], host["c2"],
                      host["c3"], old_lengths, data_length, K, ms, host["inds"], starts, lens)
    dev = {k: [torch.tensor(a, device="cuda") for a in v] for k, v in host.items()}
    pytdinterp.TDInterp_wrap(dev["out"], torch.tensor(data_time, device="cuda"), dev["ts"], dev["y"], dev["c1"],
                             dev["c2"], dev["c3"], old_lengths, data_length, B, K,
                             torch.tensor(ls, device="cuda"), torch.tensor(ms, device="cuda"), dev["inds"], starts, lens)
    for b in range(B):
        got = dev["out"][b].cpu().numpy()
        assert np.max(np.abs(got - ref[b])) <= 1e-12 * max(1.0, np.max(np.abs(ref[b])))


def test_all_in_one_likelihood_vs_oracle(torch_cuda):
    torch = torch_cuda
    from eobgpu_gb300.eob import pytdinterp
    from eobgpu_gb300.eob.seobnrv4phm import fd_likelihood
    rng = np.random.default_rng(5)
    B, nch, N, df = 5, 3, 2600, 1.0 / 8.0
    hp = rng.normal(size=B * N) + 1j * rng.normal(size=B * N)
    hc = rng.normal(size=B * N) + 1j * rng.normal(size=B * N)
    data = rng.normal(size=nch * N) + 1j * rng.normal(size=nch * N)
    psd = rng.uniform(0.5, 2.0, nch * N)
    Fp, Fc = rng.uniform(-1, 1, nch * B), rng.uniform(-1, 1, nch * B)
    tau = rng.uniform(-0.03, 0.03, nch * B)
    ref = T.all_in_one_likelihood(hp, hc, data, psd, Fp, Fc, tau, df, B, nch, N)
    c = lambda a: torch.tensor(a, device="cuda")
    temp = torch.zeros(ref.shape[0], dtype=torch.complex128, device="cuda")
    pytdinterp.all_in_one_likelihood(temp, c(hp), c(hc), c(data), c(psd), c(Fp), c(Fc), c(tau), df, B, nch, N)
    got = temp.cpu().numpy()
    np.testing.assert_allclose(got.real, ref.real, rtol=1e-12)
    assert np.all(got.imag == 0)
    lnl = fd_likelihood(c(hp).view(B, N), c(hc).view(B, N), c(data).view(nch, N), c(psd).view(nch, N),
                        c(Fp), c(Fc), c(tau), df, B, nch).cpu().numpy()
    np.testing.assert_allclose(lnl, T.fd_lnl(ref, df, B, nch).real, rtol=1e-12)


def test_tdinterp_class_on_spline_container(torch_cuda):
    """The drop-in TDInterp on a CubicSplineInterpolantTD built from ragged
    data, against the oracle driven with the same container arrays."""
    torch = torch_cuda
    from eobgpu_gb300.eob.seobnrv4phm import CubicSplineInterpolantTD, TDInterp
    rng = np.random.default_rng(11)
    B, K, L = 3, 2, 40
    nsubs = 2 * K + 1
    lengths = np.array([40, 33, 25], dtype=np.int32)
    x = np.zeros((L, B))
    yall = np.zeros((L, nsubs, B))
    for b in range(B):
        tk = np.cumsum(rng.uniform(0.3, 0.6, L))
        tk -= tk[0]
        x[:, b] = tk
        for s in range(2 * K):
            yall[:, s, b] = np.sin(0.3 * (s + 1) * tk) + 0.1 * s
        yall[:, 2 * K, b] = 2.0 * tk
    spl = CubicSplineInterpolantTD(x.reshape(-1), yall.reshape(-1), lengths, nsubs, B)
    data_time = np.arange(0.0, 25.0, 0.05)
    ls, ms = np.array([2, 3], dtype=np.int32), np.array([2, 3], dtype=np.int32)
    out = TDInterp()(data_time, spl, L, len(data_time), K, ls, ms, B).cpu().numpy()
    ts = spl.t_shaped.cpu().numpy()
    lens, inds, ml = T.tdinterp_inputs(data_time, ts, lengths)
    ref = T.td_interp2(data_time, ts.reshape(-1), spl.y_shaped.contiguous().cpu().numpy().reshape(-1),
                       spl.c1_shaped.contiguous().cpu().numpy().reshape(-1),
                       spl.c2_shaped.contiguous().cpu().numpy().reshape(-1),
                       spl.c3_shaped.contiguous().cpu().numpy().reshape(-1), L, lengths, len(data_time), B, K, ms,
                       inds, lens, ml)
    assert np.max(np.abs(out - ref)) <= 1e-12 * np.max(np.abs(ref))
