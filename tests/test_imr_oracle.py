"""The merger-ringdown completion of the oracle (oracle/imr_oracle.py and the
fits of physics/imr_fits.h) against the reference's own functions
(tests/golden/imr.npz, made by tests/golden/make_imr_golden.py), and the
inputs the reference takes from lal and pesummary against closed forms and
known values: the Kerr ISCO, the final spin, and the QNM table against
Leaver's method solved directly."""
import importlib.util
import os

import numpy as np
import pytest

from oracle import imr_oracle as imr

HERE = os.path.dirname(os.path.abspath(__file__))
MODES = [(2, 2), (2, 1), (3, 3), (4, 4), (5, 5)]


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "golden", "imr.npz")))


@pytest.fixture(scope="module")
def leaver():
    path = os.path.join(HERE, "..", "eobgpu_gb300", "csrc", "physics", "gen_qnm_table.py")
    spec = importlib.util.spec_from_file_location("gen_qnm_table", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_nr_fits_match_the_reference(oracle, gold):
    g = gold
    for b in range(len(g["m1"])):
        for k, (l, m) in enumerate(MODES):
            f = imr.fits(oracle, l, m, g["m1"][b], g["m2"][b], g["chi1"][b], g["chi2"][b])
            mine = [f["amp"], f["adot"], f["addot"], f["omega"], f["omegadot"],
                    f["delta_t22"] + (10.0 if (l, m) == (5, 5) else 0.0)]
            np.testing.assert_allclose(mine, g["nr_fits"][:, k, b], rtol=1e-13, atol=1e-16, err_msg=f"{b} {l} {m}")
            np.testing.assert_allclose([f["c1f"], f["c2f"], f["d1f"], f["d2f"]], g["rd_free"][:, k, b], rtol=1e-13,
                                       atol=1e-15)
        f = imr.fits(oracle, 2, 2, g["m1"][b], g["m2"][b], g["chi1"][b], g["chi2"][b])
        assert f["delta_t22"] == pytest.approx(g["delta_t22"][b], rel=1e-14)
        assert f["final_mass"] == pytest.approx(g["final_mass"][b], rel=1e-14)


def test_nqc_factor_matches_the_reference(gold):
    g = gold
    c = {k: g["nqc_" + k] for k in ("a1", "a2", "a3", "b1", "b2")}
    np.testing.assert_allclose(imr.nqc_factor(g["nqc_r"], g["nqc_pr"], g["nqc_omega"], c), g["nqc_factor"],
                               rtol=1e-14)


def test_nqc_coefficients_match_the_reference(oracle, gold):
    """Splines over the window, their derivatives at the attachment time, the
    NR fits and both solves, for two binaries and five modes."""
    g = gold
    for b in range(2):
        for k, (l, m) in enumerate(MODES):
            t_nr = g["nqcw_tpeak"][b] - g["nqcw_dt"][b, k]
            c = imr.nqc_coefficients(oracle, g["nqcw_t"][b], g["nqcw_amp"][b, k], g["nqcw_phase"][b, k],
                                     g["nqcw_r"][b], g["nqcw_pr"][b], g["nqcw_omega"][b], g["nqcw_t"].shape[1], t_nr,
                                     l, m, g["nqcw_m1"][b], g["nqcw_m2"][b], g["nqcw_chi1"][b], g["nqcw_chi2"][b])
            for key in ("a1", "a2", "a3", "b1", "b2"):
                assert c[key] == pytest.approx(g["nqcw_" + key][b, k], rel=1e-9, abs=1e-12), (b, l, m, key)


def test_ringdown_matches_the_reference(oracle, gold):
    g = gold
    for b in range(2):
        for k, (l, m) in enumerate(MODES):
            m1, m2, c1, c2 = g["nqcw_m1"][b], g["nqcw_m2"][b], g["nqcw_chi1"][b], g["nqcw_chi2"][b]
            f = imr.fits(oracle, l, m, m1, m2, c1, c2)
            h = imr.ringdown(g["rd_t"][b], g["rd_tmatch"][b], g["rd_amp"][b, k], g["rd_damp"][b, k],
                             g["rd_omega"][b, k], g["rd_phimatch"][b, k], l, m, m1, m2, c1, c2, g["rd_qnm"][k], f)
            ref = g["rd_h"][b, k]
            assert np.max(np.abs(h - ref)) <= 1e-12 * np.max(np.abs(ref)), (b, l, m)


def test_spline_matches_the_reference_native_spline(golden):
    """The oracle's numpy not-a-knot spline against the reference's
    interpolate_TD output (tests/golden/spline.npz)."""
    s = golden["spline"]
    for q in range(2):
        sp = imr.Spline(s["x"], s["y"][q])
        sc = np.abs(s["c1"][q]).max()
        np.testing.assert_allclose(sp.c1[:-1], s["c1"][q][:-1], atol=1e-12 * sc)
        np.testing.assert_allclose(sp.c2[:-1], s["c2"][q][:-1], atol=1e-12 * np.abs(s["c2"][q]).max())
        np.testing.assert_allclose(sp.c3[:-1], s["c3"][q][:-1], atol=1e-12 * np.abs(s["c3"][q]).max())


def test_kerr_isco_and_remnant(oracle):
    """Schwarzschild and extremal ISCO radii; the final spin of an equal-mass
    non-spinning binary (NR: 0.6864) and the final mass of the same (NR:
    0.9516); both limits of the final spin fit."""
    f = imr.fits(oracle, 2, 2, 0.5, 0.5, 0.0, 0.0)
    assert f["final_spin"] == pytest.approx(0.6864, abs=2e-3)
    assert f["final_mass"] == pytest.approx(0.9516, abs=2e-3)
    # a test particle on a Kerr hole keeps the hole's spin
    g = imr.fits(oracle, 2, 2, 1.0, 1e-6, 0.7, 0.0)
    assert g["final_spin"] == pytest.approx(0.7, abs=1e-4)
    # aligned spins raise the final spin, anti-aligned lower it
    up = imr.fits(oracle, 2, 2, 0.5, 0.5, 0.8, 0.8)["final_spin"]
    dn = imr.fits(oracle, 2, 2, 0.5, 0.5, -0.8, -0.8)["final_spin"]
    assert dn < f["final_spin"] < up < 1.0


def test_qnm_table_against_leaver(oracle, leaver):
    """The device table (four-point interpolation between its nodes) against
    Leaver's method solved directly at random spins, and Schwarzschild
    values of the literature."""
    assert leaver.qnm_at(2, 2, 0.0) == pytest.approx(0.3736716844 - 0.0889623157j, abs=1e-9)
    assert leaver.qnm_at(3, 3, 0.0) == pytest.approx(0.5994432884 - 0.0927030479j, abs=1e-9)
    assert leaver.qnm_at(4, 4, 0.0) == pytest.approx(0.809178 - 0.094164j, abs=1e-6)
    rng = np.random.default_rng(2)
    for a in np.concatenate([rng.uniform(-0.98, 0.98, 3), [0.987, -0.9]]):
        for l, m in MODES:
            exact = leaver.qnm_at(l, m, a)
            tab = imr.qnm_table(oracle, l, m, a)
            assert abs(tab - exact) < 1e-8 * abs(exact), (a, l, m, tab, exact)
