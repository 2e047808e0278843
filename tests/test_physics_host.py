"""The product's device physics (eobgpu_gb300/csrc/physics/*.h) compiled for
the host and checked against the reference's golden outputs: Hamiltonian and
gradient (u-jet evaluation), RHS (table-driven flux), the generic multipole
evaluator used by lane groups, and the Newtonian prefixes."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def phys(tmp_path_factory):
    out = tmp_path_factory.mktemp("phys") / "libphys.so"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-o", str(out),
                           os.path.join(HERE, "native", "physics_host.cpp")])
    return ctypes.CDLL(str(out))


P = ctypes.POINTER(ctypes.c_double)


def dp(a):
    return a.ctypes.data_as(P)


def test_ham_eval_vs_reference(phys, golden):
    g = golden["ham_rhs"]
    st, add = np.ascontiguousarray(g["state"]), np.ascontiguousarray(g["add"])
    n = st.shape[1]
    out = np.zeros(5 * n)
    phys.phys_ham(dp(st), dp(add), ctypes.c_int(n), dp(out))
    out = out.reshape(n, 5).T
    ok = np.isfinite(g["H"])
    assert np.max(np.abs(out[0][ok] / g["H"][ok] - 1)) < 1e-13
    gr = g["grad"]
    sc = np.abs(gr[:, ok]).max(axis=0)
    for j, q in ((1, 0), (2, 2), (3, 3)):
        assert np.max(np.abs(out[j][ok] - gr[q][ok]) / sc) < 1e-12


def test_ham_jets_match_ham_eval(phys, golden):
    """The 16-jet arrangement used by lane groups against the sequential
    evaluation and the reference."""
    g = golden["ham_rhs"]
    st, add = np.ascontiguousarray(g["state"]), np.ascontiguousarray(g["add"])
    n = st.shape[1]
    a = np.zeros(5 * n)
    b = np.zeros(5 * n)
    phys.phys_ham(dp(st), dp(add), ctypes.c_int(n), dp(a))
    phys.phys_ham_jets(dp(st), dp(add), ctypes.c_int(n), dp(b))
    a, b = a.reshape(n, 5).T, b.reshape(n, 5).T
    ok = np.all(np.isfinite(a), axis=0)
    np.testing.assert_array_equal(np.all(np.isfinite(b), axis=0), ok)
    well = ok & (st[0] >= 4.0)
    for j in range(5):
        sc = np.abs(a[1:4]).max(axis=0) if 1 <= j <= 3 else np.abs(a[j])
        rel = np.abs(b[j] - a[j]) / sc
        assert np.max(rel[ok]) < 1e-11, j
        assert np.max(rel[well]) < 1e-13, j
    gr = g["grad"]
    sc = np.abs(gr[:, ok]).max(axis=0)
    assert np.max(np.abs(b[0][ok] / g["H"][ok] - 1)) < 1e-13
    for j, q in ((1, 0), (2, 2), (3, 3)):
        assert np.max(np.abs(b[j][ok] - gr[q][ok]) / sc) < 1e-12


@pytest.mark.parametrize("fn", ["phys_ham_pair", "phys_ham_quad"])
def test_ham_pair_pieces_match_jets(phys, golden, fn):
    """The pieces two warps of a pair evaluate (jet halves and log part, the
    combination in four parts), and the pieces of four warps (log polynomials
    joined with log r, the combination in finer parts), against the
    single-group jet evaluation."""
    g = golden["ham_rhs"]
    st, add = np.ascontiguousarray(g["state"]), np.ascontiguousarray(g["add"])
    n = st.shape[1]
    a = np.zeros(5 * n)
    b = np.zeros(5 * n)
    phys.phys_ham_jets(dp(st), dp(add), ctypes.c_int(n), dp(a))
    getattr(phys, fn)(dp(st), dp(add), ctypes.c_int(n), dp(b))
    a, b = a.reshape(n, 5).T, b.reshape(n, 5).T
    ok = np.all(np.isfinite(a), axis=0)
    np.testing.assert_array_equal(np.all(np.isfinite(b), axis=0), ok)
    well = ok & (st[0] >= 4.0)
    for j in range(5):
        sc = np.abs(a[1:4]).max(axis=0) if 1 <= j <= 3 else np.abs(a[j])
        rel = np.abs(b[j] - a[j]) / sc
        assert np.max(rel[ok]) < 1e-11, j
        assert np.max(rel[well]) < 1e-13, j


def test_flux_pair_matches_lanes(phys, golden):
    """Flux summed as a warp pair does (multipoles 0..31 and 32..34 apart) and
    as four warps do (series parts times m-factor parts with the v_phi powers
    by squaring)."""
    g = golden["ham_rhs"]
    st, add = np.ascontiguousarray(g["state"]), np.ascontiguousarray(g["add"])
    n = st.shape[1]
    buf = np.zeros(3 * n)
    phys.phys_flux_pair(dp(st), dp(add), ctypes.c_int(n), dp(buf))
    out = buf[:2 * n].reshape(n, 2)
    quad = buf[2 * n:]
    ok = np.isfinite(out[:, 0])
    assert ok.sum() > 0.9 * n
    np.testing.assert_array_equal(np.isfinite(out[:, 1]), ok)
    assert np.max(np.abs(out[ok, 1] / out[ok, 0] - 1)) < 1e-13
    assert np.max(np.abs(quad[ok] / out[ok, 0] - 1)) < 1e-13


def test_eob_log_accuracy(phys):
    """Table-driven log of the hot path: within one ulp of an extended-precision
    log (mpmath) over the arguments the path uses (r >= 1, v in (0, 1)) and
    beyond, with the special values of log."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    rng = np.random.default_rng(3)
    x = np.concatenate([np.exp(rng.uniform(-9.0, 9.0, 4000)), 1.0 + rng.uniform(-1e-3, 1e-3, 1000),
                        1.0 + rng.uniform(-1e-10, 1e-10, 200), [1e-310, 5e-324, 1e300, 0.5, 2.0, 1.0]])
    y = np.zeros_like(x)
    phys.phys_log(dp(x), ctypes.c_int(len(x)), dp(y))
    worst = 0.0
    for xi, yi in zip(x, y):
        t = mpmath.log(mpmath.mpf(float(xi)))
        if t == 0:
            assert yi == 0.0
            continue
        worst = max(worst, abs(float((mpmath.mpf(float(yi)) - t) / np.spacing(abs(float(t))))))
    assert worst <= 1.0, worst
    sp = np.array([0.0, -1.0, np.inf, np.nan])
    ys = np.zeros_like(sp)
    phys.phys_log(dp(sp), ctypes.c_int(4), dp(ys))
    assert ys[0] == -np.inf and np.isnan(ys[1]) and ys[2] == np.inf and np.isnan(ys[3])


def test_rhs_vs_reference(phys, golden):
    g = golden["ham_rhs"]
    st, add = np.ascontiguousarray(g["state"]), np.ascontiguousarray(g["add"])
    n = st.shape[1]
    k = np.zeros(4 * n)
    phys.phys_rhs(dp(st), dp(add), ctypes.c_int(n), dp(k))
    k = k.reshape(4, n)
    ref = g["rhs"]
    ok = np.all(np.isfinite(ref), axis=0)
    np.testing.assert_array_equal(np.all(np.isfinite(k), axis=0), ok)
    assert np.max(np.abs(k[:, ok] - ref[:, ok]) / np.abs(ref[:, ok]).max(axis=0)) < 1e-12


def test_generic_flux_matches_specialised(phys, golden):
    g = golden["ham_rhs"]
    st, add = np.ascontiguousarray(g["state"]), np.ascontiguousarray(g["add"])
    n = st.shape[1]
    buf = np.zeros(4 * n)
    phys.phys_flux_both(dp(st), dp(add), ctypes.c_int(n), dp(buf))
    out = buf[:3 * n].reshape(n, 3)
    lanes = buf[3 * n:]
    ok = np.isfinite(out[:, 0])
    assert ok.sum() > 0.9 * n
    assert np.max(np.abs(out[ok, 1] / out[ok, 0] - 1)) < 1e-13
    assert np.max(np.abs(out[ok, 2] / out[ok, 0] - 1)) < 1e-13
    assert np.max(np.abs(lanes[ok] / out[ok, 0] - 1)) < 1e-13


def test_newton_prefixes(phys):
    from golden.make_golden import newton_prefixes
    for m1, m2 in ((0.6, 0.4), (0.5, 0.5), (0.9, 0.1)):
        pre = np.zeros(70)
        phys.phys_prefixes(ctypes.c_double(m1), ctypes.c_double(m2), dp(pre))
        ref = newton_prefixes(m1, m2)
        assert np.max(np.abs(pre[0::2] + 1j * pre[1::2] - ref)) < 1e-14 * np.abs(ref).max()
