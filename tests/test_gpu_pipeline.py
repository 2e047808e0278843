"""The fused CUDA path against the reference's golden outputs and the oracle
(configuration 1 and variations), through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.fixture(scope="module")
def cfg1_run(torch_cuda, golden):
    torch = torch_cuda
    from eobgpu_gb300.pipeline import WaveformLikelihood
    c = golden["config1"]
    P = torch.tensor(c["params"], dtype=torch.float64, device="cuda")
    d = torch.tensor(c["data"], dtype=torch.float64, device="cuda")
    wl = WaveformLikelihood(max_batch=len(P), max_steps=20000, modes=[(2, 2)], max_samples=int(c["N"]))
    lnl, st = wl.run(P, d, float(c["dt"]), float(c["amp"]))
    torch.cuda.synchronize()
    return wl, lnl.cpu().numpy(), st.cpu().numpy(), c


def test_config1_status_ok(cfg1_run):
    _, lnl, st, _ = cfg1_run
    assert np.all(st == 0), st
    assert np.all(np.isfinite(lnl))


def test_config1_initial_conditions(cfg1_run):
    wl, _, _, c = cfg1_run
    ic = wl.initial_conditions()
    np.testing.assert_allclose(ic[:, :2], c["ic"][:, :2], rtol=1e-11)
    assert np.all(np.abs(ic[:, 2]) < 2e-12)


def test_config1_trajectory_rows(cfg1_run):
    """Same number of trajectory rows and waveform samples as the reference;
    rows are not compared one by one because adaptive step sizes differ at the
    1e-5 level between implementations (the waveform comparison below is the
    size-independent check)."""
    wl, _, _, c = cfg1_run
    nsteps, npts, st, trajs = wl.trajectories()
    np.testing.assert_array_equal(nsteps, c["nsteps"])
    np.testing.assert_array_equal(npts, c["npts"])
    for b, (t, y) in enumerate(trajs):
        L = nsteps[b]
        assert t[0] == 0.0 and np.all(np.diff(t) > 0)
        # the fine pass takes fixed steps of 0.05 M, halved after each rejection
        d = np.diff(t[-20:])
        assert np.all(d <= 0.05 + 1e-9)
        ratio = 0.05 / d
        assert np.allclose(ratio, 2.0 ** np.round(np.log2(ratio)), rtol=1e-6)
        assert abs(t[-1] - c["traj_t"][b, L - 1]) < 0.05


def test_config1_strain_vs_reference(cfg1_run, torch_cuda):
    """Strain on the uniform grid vs the reference: |h| and the phase at the
    peak of |h| (FP64 bounds: relative amplitude 1e-8 of the peak, 1e-5 rad)."""
    torch = torch_cuda
    wl, _, _, c = cfg1_run
    P = torch.tensor(c["params"][:2], dtype=torch.float64, device="cuda")
    h, st = wl.strain(P, float(c["dt"]), int(c["N"]))
    h = h.cpu().numpy()
    for b in range(2):
        hr = c[f"h_{b}"]
        n = int(c["npts"][b])
        assert np.all(h[b, n:] == 0)
        peak = np.argmax(np.abs(hr[:n]))
        assert np.max(np.abs(h[b, :n] - hr[:n])) < 1e-8 * np.abs(hr[peak])
        dphi = np.angle(h[b, peak] / hr[peak])
        assert abs(dphi) < 1e-5, dphi


def test_config1_splines_vs_oracle(cfg1_run, oracle, torch_cuda):
    """The warp-partitioned spline build against the oracle's serial sweep on
    the same knots (phase and the two amplitude series of every binary)."""
    torch = torch_cuda
    wl, lnl, st, c = cfg1_run
    v = wl.views()
    B = wl.last_B
    nsteps = wl._dev_array(v.nsteps, B, torch.int32).cpu().numpy()
    roff = wl._dev_array(v.row_off, B, torch.int64).cpu().numpy()
    Rc = int(v.rows_capacity)
    tin = wl._dev_array(v.tin, Rc, torch.float64).cpu().numpy()
    arrs = [wl._dev_array(a, v.nsubs * Rc, torch.float64).cpu().numpy()
            for a in (v.spline_y, v.spline_c1, v.spline_c2, v.spline_c3)]
    for b in range(B):
        n = int(nsteps[b])
        o = int(roff[b])
        x = tin[o:o + n]
        for sub in range(v.nsubs):
            y = arrs[0][sub * Rc + o: sub * Rc + o + n]
            c1, c2, c3 = oracle.interpolate_td(x, y, [n], 1, 1)
            dx = np.diff(x)
            scale = np.max(np.abs(y))
            # each coefficient's contribution over its interval, against the
            # series' own scale (the phase runs to ~1e3 rad: its slopes carry
            # the rounding of y at that size)
            for pw, got, ref in zip((1, 2, 3), arrs[1:], (c1, c2, c3)):
                g = got[sub * Rc + o: sub * Rc + o + n - 1]
                r = ref[:n - 1]
                assert np.max(np.abs(g - r) * dx ** pw) <= 1e-12 * scale, (b, sub, pw)


def test_config1_lnl_vs_reference(cfg1_run):
    _, lnl, _, c = cfg1_run
    rel = np.abs(lnl / c["lnl"] - 1)
    assert np.all(rel < 1e-9), rel


def test_config1_lnl_vs_oracle(cfg1_run, oracle):
    _, lnl, _, c = cfg1_run
    for b in range(len(lnl)):
        r = oracle.lnl_one(c["params"][b], float(c["dt"]), int(c["N"]), [(2, 2)], c["data"], float(c["amp"]))
        assert abs(lnl[b] / r["lnl"] - 1) < 1e-9, (b, lnl[b], r["lnl"])


@pytest.mark.parametrize("G", [1, 2, 4, 8, 16, 32, 64, 128])
def test_config1_lanes_per_binary(torch_cuda, golden, G):
    """Every lanes-per-binary variant of the integrator gives the reference's lnL."""
    torch = torch_cuda
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    c = golden["config1"]
    opt = _lib.default_options()
    opt.lanes_per_binary = G
    wl = WaveformLikelihood(max_batch=8, max_steps=4096, modes=[(2, 2)], max_samples=int(c["N"]), options=opt)
    lnl, st = wl.run(torch.tensor(c["params"], device="cuda"), torch.tensor(c["data"], device="cuda"),
                     float(c["dt"]), float(c["amp"]))
    lnl = lnl.cpu().numpy()
    assert np.all(st.cpu().numpy() == 0)
    assert np.all(np.abs(lnl / c["lnl"] - 1) < 1e-9), (G, lnl / c["lnl"] - 1)
    nsteps, npts, _, _ = wl.trajectories()
    np.testing.assert_array_equal(nsteps, c["nsteps"])


@pytest.mark.parametrize("bulk", [64, 8, 32])
def test_config1_mixed_head(torch_cuda, golden, bulk):
    """Warp pairs (or lane groups of 8 and 32) with the longest binaries on
    four warps in the same launch (eob_options.head_quads): the reference's
    lnL and row counts, and the same bits as each group size run alone for
    its binaries."""
    torch = torch_cuda
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood, longest_first
    c = golden["config1"]
    P = torch.tensor(c["params"], device="cuda")
    D = torch.tensor(c["data"], device="cuda")
    order = longest_first(P)
    runs = {}
    for name, G, head in (("mixed", bulk, 3), ("pairs", bulk, 0), ("quads", 128, 0)):
        opt = _lib.default_options()
        opt.lanes_per_binary = G
        opt.head_quads = head
        wl = WaveformLikelihood(max_batch=8, max_steps=4096, modes=[(2, 2)], max_samples=int(c["N"]), options=opt)
        lnl, st = wl.run(P, D, float(c["dt"]), float(c["amp"]), order=order)
        assert np.all(st.cpu().numpy() == 0), name
        runs[name] = (lnl.cpu().numpy(), wl.trajectories()[0])
    lnl, nsteps = runs["mixed"]
    assert np.all(np.abs(lnl / c["lnl"] - 1) < 1e-9), lnl / c["lnl"] - 1
    np.testing.assert_array_equal(nsteps, c["nsteps"])
    head = order.cpu().numpy()[:3]
    rest = order.cpu().numpy()[3:]
    np.testing.assert_array_equal(lnl[head], runs["quads"][0][head])
    np.testing.assert_array_equal(lnl[rest], runs["pairs"][0][rest])


def test_config1_rtol_1e10_vs_oracle(torch_cuda, golden, oracle):
    """Configuration 1 as its benchmark states it, DOPR853 at rtol = atol =
    1e-10 (the reference hard-codes 1e-12), against the oracle at the same
    tolerances."""
    torch = torch_cuda
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    c = golden["config1"]
    opt = _lib.default_options()
    opt.rtol = opt.atol = 1e-10
    P = torch.tensor(c["params"], dtype=torch.float64, device="cuda")
    d = torch.tensor(c["data"], dtype=torch.float64, device="cuda")
    wl = WaveformLikelihood(len(P), 20000, [(2, 2)], int(c["N"]), options=opt)
    lnl, st = wl.run(P, d, float(c["dt"]), float(c["amp"]))
    nsteps = wl.trajectories()[0]
    lnl = lnl.cpu().numpy()
    assert np.all(st.cpu().numpy() == 0)
    same = 0
    for b in range(len(P)):
        r = oracle.lnl_one(c["params"][b], float(c["dt"]), int(c["N"]), [(2, 2)], c["data"], float(c["amp"]),
                           rtol=1e-10, atol=1e-10)
        assert r["status"] == 0
        # at rtol 1e-10 the step-size controller passes rounding-level RHS
        # differences on to the step sizes (~1e-9 rad of phase), so a template
        # far from the data (|lnL| ~ 5e3) agrees to a few 1e-9 relative
        if r["nsteps"] == nsteps[b]:
            same += 1
            assert abs(lnl[b] / r["lnl"] - 1) < 1e-8, b
        else:
            # a different step sequence: the local error per step is ~100x that
            # at rtol 1e-12, and so is the spread between two valid sequences
            assert abs(lnl[b] / r["lnl"] - 1) < 1e-5, b
    assert same >= len(P) // 2
