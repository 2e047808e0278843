"""Every mode the reference's waveform class computes -- (2,2), (2,1), (3,3),
(4,4), (5,5) -- on the GPU against the reference's own outputs
(tests/golden/modes5.npz: the reference's EOBGetSpinFactorizedWaveform,
src/EOB.cu:1235-1677, on its own trajectories of the eight configuration-1
binaries, q = 1.4-3.0, with the five-mode strain and lnL):

* the reference-shaped entry point (eob_ctx_waveform, through the
  SEOBNRv5Class mirror) on the reference's rows and inputs, per mode;
* the fused FP64 path with all five modes on its own knots against the
  oracle replayed on those knots: strain within 1e-8 of its peak, phase at
  the peak within 1e-5 rad, relative lnL within 1e-9 (the oracle's modes are
  pinned to the reference's within 3e-14); and free-running against the
  reference (its own knots, the same row and sample counts);
* the mixed-precision synthesis with all five modes: mismatch <= 1e-6,
  |dlnL| <= 1e-3, phase at the peak within 1e-5 rad."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _t(torch, a, dtype=None):
    import torch as _torch
    return torch.tensor(np.ascontiguousarray(a), dtype=dtype or _torch.float64, device="cuda")


def test_ctx_waveform_every_mode(torch_cuda, golden):
    torch = torch_cuda
    from eobgpu_gb300.eob import pyEOB
    g = golden["modes5"]
    worst = 0.0
    for b in range(len(g["params"])):
        p = g["params"][b]
        m1, m2 = p[0] / (p[0] + p[1]), p[1] / (p[0] + p[1])
        eta = m1 * m2
        chiS, chiA = (p[2] + p[3]) / 2, (p[2] - p[3]) / 2
        tpl = (1 - 2 * eta) * chiS + (m1 - m2) * chiA
        cls = pyEOB.SEOBNRv5Class()
        one = lambda v: _t(torch, np.array([v]))
        cls.update_information(one(m1), one(m2), one(eta), one(tpl), one(chiS), one(chiA), 1, 1, None)
        n = int(g["nsteps"][b])
        y = g["traj_y"][b, :n]
        cols = [_t(torch, y[:, q]) for q in range(4)]
        v, H, vphi = (_t(torch, g[k][b, :n]) for k in ("v", "Hreal", "vPhi"))
        idx = torch.zeros(1, dtype=torch.int32, device="cuda")
        out = torch.zeros(2 * n, dtype=torch.float64, device="cuda")
        for k, (l, m) in enumerate(g["modes"]):
            pre = g["prefix"][b, k]
            cls.EOBGetSpinFactorizedWaveform(out, *cols, v, H, one(g["eta"][b]), vphi, int(l), int(m),
                                             _t(torch, [pre.real, pre.imag]), 0.0, 1, n, idx)
            got = out.cpu().numpy()
            mine = got[0::2] + 1j * got[1::2]
            ref = g["hlm"][b, k, :n]
            err = np.max(np.abs(mine - ref)) / np.max(np.abs(ref))
            worst = max(worst, err)
            assert err < 1e-12, (b, l, m, err)
        cls.deallocate_information()
    print(f"\nctx waveform, worst mode error of its peak: {worst:.2e}")


def _peak(h):
    k = int(np.argmax(np.abs(h)))
    return k, h[k]


@pytest.fixture(scope="module")
def five_mode_runs(torch_cuda, golden):
    torch = torch_cuda
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    g, c = golden["modes5"], golden["config1"]
    modes = [tuple(int(v) for v in lm) for lm in g["modes"]]
    P = _t(torch, g["params"])
    D = _t(torch, c["data"])
    N = int(c["N"])
    out = {}
    for prec in (0, 1):
        o = _lib.default_options()
        o.precision = prec
        wl = WaveformLikelihood(len(g["params"]), 4000, modes, N, options=o)
        lnl, st = wl.run(P, D, float(c["dt"]), float(c["amp"]))
        h, _ = wl.strain(P, float(c["dt"]), N)
        tr = wl.trajectories()
        out[prec] = (lnl.cpu().numpy(), st.cpu().numpy(), h.cpu().numpy(), wl.npts(), tr[0])
        if prec == 0:
            out["traj"] = tr[3]
    return out


def test_fused_five_modes_fp64_replay(five_mode_runs, golden, oracle):
    """The fused FP64 path with five modes against the oracle replayed on the
    GPU's own knots (the oracle's modes are pinned to the reference's within
    3e-14, tests/test_oracle_modes5.py): the FP64 tolerances per binary."""
    g, c = golden["modes5"], golden["config1"]
    lnl, st, h, npts, nsteps = five_mode_runs[0]
    trajs = five_mode_runs["traj"]
    modes = [tuple(int(v) for v in lm) for lm in g["modes"]]
    assert np.all(st == 0)
    worst = [0.0, 0.0, 0.0]
    for b in range(len(lnl)):
        r = oracle.lnl_one(g["params"][b], float(c["dt"]), int(c["N"]), modes, c["data"], float(c["amp"]),
                           want_detail=True, replay_t=trajs[b][0])
        assert r["status"] == 0 and r["npts"] == npts[b]
        n = int(npts[b])
        k, hk = _peak(r["h"][:n])
        e = [np.max(np.abs(h[b, :n] - r["h"][:n])) / abs(hk), abs(np.angle(h[b, k] / hk)), abs(lnl[b] / r["lnl"] - 1)]
        worst = [max(u, v) for u, v in zip(worst, e)]
        assert e[0] < 1e-8 and e[1] < 1e-5 and e[2] < 1e-9, (b, e)
    print(f"\nfive modes, replay: strain {worst[0]:.2e} of peak, phase {worst[1]:.2e} rad, lnL {worst[2]:.2e}")


def test_fused_five_modes_fp64_vs_reference(five_mode_runs, golden):
    """Free-running against the reference's own five-mode output: the same
    row and sample counts; the two runs sample the trajectory on knots that
    differ by ~1e-5 relative (adaptive steps), which moves the strain near the
    merger by up to ~2e-8 of its peak."""
    g = golden["modes5"]
    lnl, st, h, npts, nsteps = five_mode_runs[0]
    assert np.all(st == 0)
    np.testing.assert_array_equal(nsteps, g["nsteps"])
    np.testing.assert_array_equal(npts, g["npts"])
    rows = []
    for b in range(len(lnl)):
        hr = g[f"h_{b}"]
        n = int(g["npts"][b])
        k, hk = _peak(hr[:n])
        rows.append((np.max(np.abs(h[b, :n] - hr[:n])) / abs(hk), abs(np.angle(h[b, k] / hk)),
                     abs(lnl[b] / g["lnl"][b] - 1)))
    print("\nfive modes, free-running vs reference (strain of peak, phase at peak, rel lnL):")
    for b, e in enumerate(rows):
        print(b, " ".join(f"{v:.2e}" for v in e))
    for b, e in enumerate(rows):
        assert e[0] < 1e-7, (b, e)
        assert e[1] < 1e-5, (b, e)
        assert e[2] < 1e-8, (b, e)


def test_fused_five_modes_mixed_vs_reference(five_mode_runs, golden):
    g = golden["modes5"]
    lnl, st, h, npts, nsteps = five_mode_runs[1]
    assert np.all(st == 0)
    for b in range(len(lnl)):
        hr = g[f"h_{b}"]
        n = int(g["npts"][b])
        a, c = hr[:n], h[b, :n]
        ov = np.real(np.vdot(a, c)) / np.sqrt(np.real(np.vdot(a, a)) * np.real(np.vdot(c, c)))
        k, hk = _peak(a)
        assert 1 - ov <= 1e-6, (b, 1 - ov)
        assert abs(np.angle(c[k] / hk)) < 1e-5, b
        assert abs(lnl[b] - g["lnl"][b]) <= 1e-3, (b, lnl[b], g["lnl"][b])


def test_compute_hlms_every_mode(torch_cuda, golden):
    """SEOBNRv5Class.compute_hlms (the reference's kernel, src/EOB.cu:3147-3322,
    computes these modes but never stores them) on the reference's own rows of
    the eight configuration-1 binaries: H, v, omega_c and vPhi formed inside from
    additionalArgs, every mode against the reference's EOBGetSpinFactorizedWaveform
    output: within 1e-11 of the mode's peak on rows with r >= 4, within 1e-9 on
    every row (the plunge, where the gradients -- and so v and vPhi -- agree
    with the reference's to the bounds of the reference-shaped entry points)."""
    torch = torch_cuda
    from eobgpu_gb300.eob import pyEOB
    g = golden["modes5"]
    B = len(g["params"])
    p = g["params"]
    m1, m2 = p[:, 0] / (p[:, 0] + p[:, 1]), p[:, 1] / (p[:, 0] + p[:, 1])
    eta = m1 * m2
    chiS, chiA = (p[:, 2] + p[:, 3]) / 2, (p[:, 2] - p[:, 3]) / 2
    tpl = (1 - 2 * eta) * chiS + (m1 - m2) * chiA
    modes = [tuple(int(v) for v in lm) for lm in g["modes"]]
    K = len(modes)
    pre = np.ascontiguousarray(g["prefix"].T)  # [K][B] complex
    pre_d = torch.tensor(pre.view(np.float64).copy(), device="cuda")
    cls = pyEOB.SEOBNRv5Class()
    cls.update_information(_t(torch, m1), _t(torch, m2), _t(torch, eta), _t(torch, tpl), _t(torch, chiS),
                           _t(torch, chiA), 1, B, pre_d)
    L = g["traj_y"].shape[1]
    y = g["traj_y"]
    add = np.zeros((80, B))
    add[0], add[1], add[2], add[3] = m1, m2, p[:, 2], p[:, 3]
    hlms = torch.zeros(2 * B * K * L, dtype=torch.float64, device="cuda")
    cols = [_t(torch, y[:, :, q]) for q in range(4)]
    cls.compute_hlms(hlms, *cols, _t(torch, m1), _t(torch, m2), _t(torch, p[:, 2]), _t(torch, p[:, 3]),
                     _t(torch, g["nsteps"], torch.int32), L, _t(torch, [l for l, _ in modes], torch.int32),
                     _t(torch, [m for _, m in modes], torch.int32), K, B, _t(torch, add), 80)
    out = hlms.cpu().numpy().view(np.complex128).reshape(B, K, L)
    worst = 0.0
    for b in range(B):
        n = int(g["nsteps"][b])
        for k in range(K):
            ref = g["hlm"][b, k, :n]
            d = np.abs(out[b, k, :n] - ref) / np.max(np.abs(ref))
            far = y[b, :n, 0] >= 4.0
            worst = max(worst, float(d.max()))
            assert d[far].max() < 1e-11, (b, modes[k], d[far].max())
            assert d.max() < 1e-9, (b, modes[k], d.max())
    cls.deallocate_information()
    print(f"\ncompute_hlms, worst mode error of its peak: {worst:.2e}")
