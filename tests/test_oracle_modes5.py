"""Every mode the reference's waveform class computes -- (2,2), (2,1), (3,3),
(4,4), (5,5) -- against the reference's own outputs (tests/golden/modes5.npz,
made by tests/golden/make_golden.py from the reference's host-compiled
EOBGetSpinFactorizedWaveform, src/EOB.cu:1235-1677, on its own trajectories
of the eight configuration-1 binaries, q = 1.4-3.0).

These pin the oracle's higher modes: the complex log-Gamma phase of T_lm,
the delta_lm phases, f_lm and the odd-m Newtonian factors."""
import numpy as np
import pytest


def _ctx(oracle, p):
    m1, m2 = p[0] / (p[0] + p[1]), p[1] / (p[0] + p[1])
    return oracle.context(np.array([m1]), np.array([m2]), np.array([p[2]]), np.array([p[3]]))


@pytest.mark.parametrize("b", range(8))
def test_oracle_modes_on_reference_inputs(oracle, golden, b):
    """Same rows, same v, H_real and vPhi: every mode within 1e-12 of its
    largest value on the trajectory."""
    g = golden["modes5"]
    n = int(g["nsteps"][b])
    y = g["traj_y"][b, :n]
    ctx = _ctx(oracle, g["params"][b])
    for k, (l, m) in enumerate(g["modes"]):
        mine = ctx.waveform(y[:, 0], y[:, 1], y[:, 2], y[:, 3], g["v"][b, :n], g["Hreal"][b, :n], g["eta"][b],
                            g["vPhi"][b, :n], int(l), int(m), g["prefix"][b, k])
        ref = g["hlm"][b, k, :n]
        scale = np.max(np.abs(ref))
        assert scale > 0
        err = np.max(np.abs(mine - ref)) / scale
        assert err < 1e-12, (l, m, err)


@pytest.mark.parametrize("b", range(8))
def test_oracle_five_mode_path_on_reference_knots(oracle, golden, b):
    """The whole five-mode path (modes, splines, synthesis, lnL) replayed on
    the reference's knots: strain within 1e-9 of its peak, lnL within 1e-12."""
    g = golden["modes5"]
    c = golden["config1"]
    n = int(g["nsteps"][b])
    modes = [tuple(int(v) for v in lm) for lm in g["modes"]]
    r = oracle.lnl_one(g["params"][b], float(c["dt"]), int(c["N"]), modes, c["data"], float(c["amp"]),
                       want_detail=True, replay_t=g["traj_t"][b, :n])
    assert r["status"] == 0 and r["npts"] == g["npts"][b]
    hr = g[f"h_{b}"]
    m = min(len(hr), int(r["npts"]))
    assert np.max(np.abs(r["h"][:m] - hr[:m])) < 1e-9 * np.abs(hr).max()
    assert abs(r["lnl"] / g["lnl"][b] - 1) < 1e-12, (r["lnl"], g["lnl"][b])


def test_higher_modes_are_not_negligible(golden):
    """The fixture exercises the odd-m modes: unequal masses, so (2,1), (3,3)
    and (5,5) carry a visible share of the strain."""
    g = golden["modes5"]
    for b in range(8):
        n = int(g["nsteps"][b])
        peak = np.abs(g["hlm"][b, :, :n]).max(axis=1)
        assert np.all(peak[1:] > 1e-4 * peak[0]), peak
