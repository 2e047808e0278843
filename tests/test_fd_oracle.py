"""The numpy restatement of the frequency-domain likelihood flow
(oracle/td_oracle.py: detector response of eob/seobnrv4phm.py:597-634, the
two real FFTs of :736-744, the likelihood of :778-817) on closed forms: the
sidereal time, the antenna patterns of an L-shaped detector and the delay
from the geocenter."""
import numpy as np

from oracle import td_oracle as t

DX = 0.5 * (np.outer([1, 0, 0], [1, 0, 0]) - np.outer([0, 1, 0], [0, 1, 0]))


def test_gmst_at_j2000():
    """At 2000-01-01 12:00 UTC (GPS 630763213, 13 leap seconds) T = 0 and
    GMST = 67310.54841 s (18h 41m 50.54841s)."""
    assert abs(t.gmst_from_gps(630763213.0) - 67310.54841 / 86400 * 2 * np.pi) < 1e-12


def test_gmst_sidereal_day_and_leap_seconds():
    g0 = t.gmst_from_gps(1.2e9)
    g1 = t.gmst_from_gps(1.2e9 + 86164.0905)  # one sidereal day later
    assert abs((g1 - g0 + np.pi) % (2 * np.pi) - np.pi) < 1e-6
    # a leap second shifts UTC by one second: across 2017-01-01 the GPS
    # clock runs one second ahead of the sidereal rotation
    a, b = t.gmst_from_gps(1167264017.5), t.gmst_from_gps(1167264018.5)
    assert abs(b - a) < 1e-9 * 2 * np.pi


def test_antenna_patterns_of_an_l_shaped_detector():
    rng = np.random.default_rng(3)
    B = 64
    ra, dec = rng.uniform(0, 2 * np.pi, B), rng.uniform(-1.5, 1.5, B)
    psi, tm = rng.uniform(0, np.pi, B), rng.uniform(1e9, 1.3e9, B)
    R = 6.4e6
    Fp, Fx, tau = t.detector_information(ra, dec, tm, psi, DX[None], np.array([[R, 0.0, 0.0]]))
    ph = ra - np.fmod(t.gmst_from_gps(tm), 2 * np.pi)
    th = np.pi / 2 - dec
    # |F+|^2 + |Fx|^2 does not depend on the polarisation angle
    tot = 0.25 * (1 + np.cos(th) ** 2) ** 2 * np.cos(2 * ph) ** 2 + np.cos(th) ** 2 * np.sin(2 * ph) ** 2
    np.testing.assert_allclose(Fp[0] ** 2 + Fx[0] ** 2, tot, atol=1e-14)
    # rotating psi by pi/4 exchanges the patterns (up to sign)
    Fp2, Fx2, _ = t.detector_information(ra, dec, tm, psi + np.pi / 4, DX[None], np.array([[R, 0.0, 0.0]]))
    np.testing.assert_allclose(np.abs(Fp2[0]), np.abs(Fx[0]), atol=1e-13)
    # delay: the source direction projected on the vertex
    np.testing.assert_allclose(tau[0], np.sin(th) * np.cos(ph) * R / t.SPEED_OF_LIGHT, rtol=1e-14, atol=1e-20)


def test_fd_get_ll_of_the_data_itself_is_zero():
    """A template equal to the detector data (its projection at the same
    delay) has lnL = 0; a zero template gives -1/2 4 df sum |d|^2 / S."""
    rng = np.random.default_rng(5)
    N, fs = 256, 64.0
    h = rng.standard_normal((2, N)) + 1j * rng.standard_normal((2, N))
    D = np.stack([DX, 0.5 * (np.outer([0, 0, 1], [0, 0, 1]) - np.outer([1, 0, 0], [1, 0, 0]))])
    V = np.array([[6.4e6, 0, 0], [0, 6.4e6, 0]])
    ra, dec, psi, tm = np.array([0.3, 1.2]), np.array([0.1, -0.4]), np.array([0.2, 2.0]), np.array([1.1e9, 1.2e9])
    Fp, Fx, tau = t.detector_information(ra, dec, tm, psi, D, V)
    f = np.fft.rfftfreq(N, 1.0 / fs)
    hp, hc = np.fft.rfft(h.real, axis=-1), np.fft.rfft(h.imag, axis=-1)
    psd = rng.uniform(0.5, 2.0, (2, N // 2 + 1))
    for b in range(2):
        data = (Fp[:, b, None] * hp[b] + Fx[:, b, None] * hc[b]) * np.exp(-2j * np.pi * f * tau[:, b, None])
        ll = t.fd_get_ll(h, data, psd, ra, dec, psi, tm, D, V, fs)
        assert abs(ll[b]) < 1e-12 * np.sum(np.abs(data) ** 2 / psd)
    zero = t.fd_get_ll(np.zeros((1, N), complex), data, psd, ra[:1], dec[:1], psi[:1], tm[:1], D, V, fs)
    df = fs / N
    np.testing.assert_allclose(zero[0], -0.5 * 4 * df * np.sum(np.abs(data) ** 2 / psd), rtol=1e-13)
