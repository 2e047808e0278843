"""The reference-shaped entry points (eob.pyEOB, eob.pydopr853, eob.pytdinterp
mirrors) on the GPU against the reference's golden outputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _t(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def test_hamiltonian_entry_points(torch_cuda, golden):
    torch = torch_cuda
    from eobgpu_gb300.eob import pyEOB
    g = golden["ham_rhs"]
    st, add = g["state"], g["add"]
    n = st.shape[1]
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    pyEOB.evaluate_Ham_align_AD(out, _t(torch, st[0]), _t(torch, st[1]), _t(torch, st[2]), _t(torch, st[3]),
                                _t(torch, add[0]), _t(torch, add[1]), _t(torch, add[2]), _t(torch, add[3]),
                                0.0, 0.0, 0.0, 0.0, n)
    H = out.cpu().numpy()
    ok = np.isfinite(g["H"])
    # states down to r = 2 with |pr| up to 6 are included; there sqrt(A W) is nearly
    # singular and GPU FMA contraction / libm differences reach ~1e-12 in H and ~1e-10 in
    # its gradient.  Away from that corner (r >= 4) the agreement is held to 1e-11.
    well = ok & (st[0] >= 4.0)
    assert np.max(np.abs(H[ok] / g["H"][ok] - 1)) < 1e-11
    grad = torch.zeros(4 * n, dtype=torch.float64, device="cuda")
    pyEOB.grad_Ham_align_AD(_t(torch, st.ravel()), grad, _t(torch, add.ravel()), n)
    gr = grad.cpu().numpy().reshape(4, n)
    rel = np.abs(gr - g["grad"]) / np.abs(g["grad"]).max(axis=0)
    assert np.max(rel[:, ok]) < 1e-9
    assert np.max(rel[:, well]) < 1e-11
    hess = torch.zeros(16 * n, dtype=torch.float64, device="cuda")
    pyEOB.hessian_Ham_align_AD(_t(torch, st.ravel()), hess, _t(torch, add.ravel()), n)
    hs = hess.cpu().numpy().reshape(16, n)
    for q in range(1, 16):
        ref = g["hess"][q, ok]
        scale = np.maximum(np.abs(ref), 1e-6 * np.abs(g["hess"][15, ok]))
        assert np.max(np.abs(hs[q, ok] - ref) / scale) < 1e-8, q


def test_ode_and_force(torch_cuda, golden):
    torch = torch_cuda
    from eobgpu_gb300.eob import pyEOB
    g = golden["ham_rhs"]
    b = g["binary"]
    ns = g["state"].shape[1] // len(b)
    for bi in range(len(b)):
        sl = slice(bi * ns, (bi + 1) * ns)
        m1, m2, c1, c2 = b[bi]
        eta = m1 * m2 / (m1 + m2) ** 2
        chiS, chiA = (c1 + c2) / 2, (c1 - c2) / 2
        tpl = (1 - 2 * eta) * chiS + (m1 - m2) / (m1 + m2) * chiA
        cls = pyEOB.SEOBNRv5Class()
        one = lambda v: _t(torch, np.array([v]))
        cls.update_information(one(m1), one(m2), one(eta), one(tpl), one(chiS), one(chiA), 1, 1, None)
        st = _t(torch, g["state"][:, sl].ravel())
        add = _t(torch, g["add"][:, sl].ravel())
        idx = torch.zeros(ns, dtype=torch.int32, device="cuda")
        k = torch.zeros(4 * ns, dtype=torch.float64, device="cuda")
        cls.ODE_Ham_align_AD(torch.zeros(1, device="cuda", dtype=torch.float64), st, k, add, ns, idx)
        kk = k.cpu().numpy().reshape(4, ns)
        ref = g["rhs"][:, sl]
        ok = np.all(np.isfinite(ref), axis=0)
        # near-singular corner (r < 4 with large |pr|) as for the gradient above
        well = ok & (g["state"][0, sl] >= 4.0)
        rel = np.abs(kk - ref) / np.abs(ref).max(axis=0)
        assert np.max(rel[:, ok]) < 1e-9
        assert np.max(rel[:, well]) < 1e-11
        f = torch.zeros(2 * ns, dtype=torch.float64, device="cuda")
        gbuf = torch.zeros(4 * ns, dtype=torch.float64, device="cuda")
        cls.RR_force(f, gbuf, st, add, ns, idx)
        ff = f.cpu().numpy().reshape(2, ns)
        fr = g["force"][:, sl]
        relf = np.abs(ff - fr) / np.abs(fr).max(axis=0)
        assert np.max(relf[:, ok]) < 1e-9
        assert np.max(relf[:, well]) < 1e-11
        cls.deallocate_information()


def test_interpolate_td(torch_cuda, golden):
    torch = torch_cuda
    from eobgpu_gb300.eob import pytdinterp
    s = golden["spline"]
    L = len(s["x"])
    x = _t(torch, s["x"])
    y = _t(torch, s["y"].T.ravel())
    Bv, ud, dg, ld = (torch.zeros(2 * L, dtype=torch.float64, device="cuda") for _ in range(4))
    pytdinterp.interpolate_TD_wrap(x, y, Bv, ud, dg, ld, torch.tensor([L], dtype=torch.int32, device="cuda"), 1, 2)
    for ref, mine in ((s["c1"], ud), (s["c2"], dg), (s["c3"], ld)):
        m = mine.cpu().numpy().reshape(L, 2).T
        assert np.max(np.abs(m[:, :-1] - ref[:, :-1])) < 1e-11 * np.abs(ref[:, :-1]).max()
