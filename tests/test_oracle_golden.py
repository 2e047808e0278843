"""The oracle against the reference's own outputs (tests/golden/, made by
tests/golden/make_golden.py from the reference's host-compiled kernels)."""
import os

import numpy as np
import pytest

from golden_map import dense_index


def test_hamiltonian_value(oracle, golden):
    g = golden["ham_rhs"]
    st, add = g["state"], g["add"]
    H = oracle.evaluate_H(st[0], st[1], st[2], st[3], add[0], add[1], add[2], add[3])
    ok = np.isfinite(g["H"])
    np.testing.assert_array_equal(np.isfinite(H), ok)
    assert np.max(np.abs(H[ok] / g["H"][ok] - 1)) < 1e-13


def test_hamiltonian_gradient(oracle, golden):
    g = golden["ham_rhs"]
    gr = oracle.grad_H(g["state"], g["add"])
    ok = np.all(np.isfinite(g["grad"]), axis=0)
    scale = np.abs(g["grad"][:, ok]).max(axis=0)
    assert np.max(np.abs(gr[:, ok] - g["grad"][:, ok]) / scale) < 1e-12


def test_hamiltonian_hessian(oracle, golden):
    """All entries match the reference except d2H/dr2, which the reference
    gets wrong (src/EOB.cu:322); that one is checked against a central
    difference of the reference's own gradient."""
    g = golden["ham_rhs"]
    hs = oracle.hessian_H(g["state"], g["add"])
    ok = np.all(np.isfinite(g["hess"]), axis=0)
    for q in range(1, 16):
        ref = g["hess"][q, ok]
        scale = np.maximum(np.abs(ref), 1e-6 * np.abs(g["hess"][15, ok]))
        assert np.max(np.abs(hs[q, ok] - ref) / scale) < 1e-9, q
    # d2H/dr2 from the oracle's gradient by central differences
    st = g["state"][:, ok][:, :32].copy()
    add = g["add"][:, ok][:, :32]
    h = 1e-5 * st[0]
    sp, sm = st.copy(), st.copy()
    sp[0] += h
    sm[0] -= h
    fd = (oracle.grad_H(sp, add)[0] - oracle.grad_H(sm, add)[0]) / (2 * h)
    an = oracle.hessian_H(st, add)[0]
    assert np.max(np.abs(fd - an) / np.abs(an)) < 1e-5
    # and the reference's value is off by orders of magnitude
    assert np.min(np.abs(g["hess"][0, ok][:32] / an)) > 1e3


def test_rhs_and_force(oracle, golden):
    g = golden["ham_rhs"]
    b = g["binary"]
    ns = g["state"].shape[1] // len(b)
    for bi in range(len(b)):
        sl = slice(bi * ns, (bi + 1) * ns)
        ctx = oracle.context(b[bi:bi + 1, 0], b[bi:bi + 1, 1], b[bi:bi + 1, 2], b[bi:bi + 1, 3])
        k = ctx.ode(g["state"][:, sl], g["add"][:, sl])
        ref = g["rhs"][:, sl]
        ok = np.all(np.isfinite(ref), axis=0)
        np.testing.assert_array_equal(np.all(np.isfinite(k), axis=0), ok)
        assert np.max(np.abs(k[:, ok] - ref[:, ok]) / np.abs(ref[:, ok]).max(axis=0)) < 1e-12
        f = ctx.rr_force(g["state"][:, sl], g["add"][:, sl])
        fr = g["force"][:, sl]
        assert np.max(np.abs(f[:, ok] - fr[:, ok]) / np.abs(fr[:, ok]).max(axis=0)) < 1e-12


def test_waveform_coefficients(oracle, golden):
    fc = golden["fac_coeffs"]
    names = [str(n) for n in fc["names"]]
    b = fc["binary"]
    checked = 0
    for bi in range(len(b)):
        ctx = oracle.context(b[bi:bi + 1, 0], b[bi:bi + 1, 1], b[bi:bi + 1, 2], b[bi:bi + 1, 3])
        dense = ctx.coeffs(0)
        for j, nm in enumerate(names):
            di = dense_index(nm)
            if di is None:
                continue
            rv = fc["coeffs"][bi, j]
            assert abs(dense[di] - rv) <= 1e-13 * max(1.0, abs(rv)), (bi, nm, rv, dense[di])
            checked += 1
    assert checked > 200 * len(b)


def test_spline_coefficients(oracle, golden):
    s = golden["spline"]
    x, y = s["x"], s["y"]
    L = len(x)
    yy = np.ascontiguousarray(y.T.ravel())
    c1, c2, c3 = oracle.interpolate_td(x, yy, np.array([L]), 1, 2)
    for ref, mine in ((s["c1"], c1), (s["c2"], c2), (s["c3"], c3)):
        mine = mine.reshape(L, 2).T
        sc = np.abs(ref[:, :-1]).max()
        assert np.max(np.abs(mine[:, :-1] - ref[:, :-1])) < 1e-12 * sc


def test_spline_reproduces_cubic(oracle):
    """Not-a-knot splines reproduce a cubic exactly."""
    x = np.cumsum(np.linspace(0.3, 1.7, 25))
    y = 0.2 - 1.5 * x + 0.25 * x ** 2 + 0.03 * x ** 3
    c1, c2, c3 = oracle.interpolate_td(x, y, np.array([len(x)]), 1, 1)
    xm = 0.5 * (x[1:] + x[:-1])
    dx = xm - x[:-1]
    ev = y[:-1] + c1[:-1] * dx + c2[:-1] * dx ** 2 + c3[:-1] * dx ** 3
    exact = 0.2 - 1.5 * xm + 0.25 * xm ** 2 + 0.03 * xm ** 3
    assert np.max(np.abs(ev - exact)) < 1e-10 * np.abs(exact).max()


@pytest.mark.parametrize("b", range(8))
def test_config1_end_to_end(oracle, golden, b):
    c = golden["config1"]
    r = oracle.lnl_one(c["params"][b], float(c["dt"]), int(c["N"]), [(2, 2)], c["data"], float(c["amp"]),
                       want_detail=True)
    assert r["status"] == 0
    assert r["nsteps"] == c["nsteps"][b]
    assert r["npts"] == c["npts"][b]
    np.testing.assert_allclose(r["ic"][:2], c["ic"][b][:2], rtol=1e-12)
    assert abs(r["ic"][2]) < 2e-12 and abs(c["ic"][b][2]) < 2e-12
    assert abs(r["lnl"] / c["lnl"][b] - 1) < 1e-9
    if f"h_{b}" in c:
        h, hr = r["h"], c[f"h_{b}"]
        m = min(len(hr), len(h))
        assert np.max(np.abs(h[:m] - hr[:m])) < 1e-8 * np.abs(hr).max()


@pytest.mark.parametrize("b", range(8))
def test_config1_replay_on_reference_knots(oracle, golden, b):
    """Replay mode: the oracle carried over the reference's own accepted knots
    (one DOPR853 step per pair of rows) reproduces the reference's trajectory
    rows and its likelihood -- the check that lets the CUDA path be compared
    with the oracle on identical knots."""
    c = golden["config1"]
    L = int(c["nsteps"][b])
    t = c["traj_t"][b, :L]
    r = oracle.lnl_one(c["params"][b], float(c["dt"]), int(c["N"]), [(2, 2)], c["data"], float(c["amp"]),
                       want_detail=True, replay_t=t)
    assert r["status"] == 0 and r["nsteps"] == L and r["npts"] == c["npts"][b]
    # rows within 1e-10 of each component's scale (measured: at most 4e-11,
    # in p_r on the last rows of the plunge; up to 1.3e-11 at r > 3)
    yr = c["traj_y"][b, :L]
    scale = np.max(np.abs(yr), axis=0)
    err = np.abs(r["y"] - yr) / scale
    assert np.all(err.max(axis=0) <= 1e-10), err.max(axis=0)
    assert np.all(err[yr[:, 0] > 3.0].max(axis=0) <= 3e-11), err[yr[:, 0] > 3.0].max(axis=0)
    # lnL on identical knots: measured within 1e-13 (free-running: up to 4e-11)
    assert abs(r["lnl"] / c["lnl"][b] - 1) < 1e-12, (r["lnl"], c["lnl"][b])
    if f"h_{b}" in c:
        h, hr = r["h"], c[f"h_{b}"]
        m = min(len(hr), len(h))
        assert np.max(np.abs(h[:m] - hr[:m])) < 1e-9 * np.abs(hr).max()


def test_config2_spread_fixture_reproduces():
    """tests/golden/config2_spread.npz (the oracle's own one-ulp spread on the
    ragged-batching sample, which sets the GPU's free-running bounds) is what
    tests/golden/make_spread.py computes: three binaries re-measured, the
    largest spread among them."""
    from golden import make_spread
    from eobgpu_gb300 import workload
    fx = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "config2_spread.npz")))
    cfg = workload.CONFIGS[2]
    params = workload.draw_params(cfg)
    data, amp = make_spread.data_vector(cfg)
    for j in (int(np.argmax(fx["rel_dlnl"])), 0, len(fx["index"]) - 1):
        b = int(fx["index"][j])
        out = make_spread.one((params[b], cfg.dt, cfg.n_samples, data, amp))
        assert out[0] == pytest.approx(fx["lnl"][j], rel=1e-12)
        assert max(out[3], out[9]) == pytest.approx(fx["rel_dlnl"][j], rel=1e-3, abs=1e-15)
