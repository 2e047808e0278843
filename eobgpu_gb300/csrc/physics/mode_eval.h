// Factorized waveform multipole h_lm on a trajectory point.
//
// Restates EOBGetSpinFactorizedWaveform (src/EOB.cu:1235-1613):
//   h_lm = T_lm e^{i delta_lm} S_lm (rho_lm^l + f_lm) h^N_lm,
//   T_lm = Gamma(l + 1 - 2 i k) / l! e^{pi k} e^{2 i k log(4 m Omega / sqrt(e))},
//   k = m H_real Omega,  h^N_lm = n_lm vPhi^(l+eps) Y_{l-eps}^{-m}(pi/2, phi).
// The complex Gamma function is our own: an upward shift by the recurrence
// Gamma(z) = Gamma(z + n) / prod_{j<n} (z + j) (Abramowitz & Stegun 6.1.15)
// and the Stirling series for log Gamma (A&S 6.1.40) at Re(z + n) >= 16.
// Only exp() of the log is ever used, so the branch of the complex logarithm
// does not matter.  The reference's SciPy-derived loggamma is not used.
//
// With derotate = true the result is multiplied by e^{i m phi}: the
// e^{-i m phi} of the spherical harmonic is simply not applied, which is what
// the spline inputs of the synthesis need (eob/seobnrv4phm.py:2331).
#pragma once
#include "fac_coeffs.h"

namespace eob {

struct cdbl {
    double re, im;
};
EOB_HD cdbl cmul(cdbl a, cdbl b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// log Gamma(z) + log(prod shift) pieces: returns log|Gamma(z)| and arg Gamma(z) (mod 2 pi)
EOB_HD void cloggamma_shifted(double zr, double zi, double *lg_re, double *lg_im)
{
    // shift product P = prod (z + j) until Re(z) >= 16
    double pr = 1.0, pim = 0.0;
    while (zr < 16.0) {
        const double t = pr * zr - pim * zi;
        pim = pr * zi + pim * zr;
        pr = t;
        zr += 1.0;
    }
    // 1/w and 1/w^2
    const double den = 1.0 / (zr * zr + zi * zi);
    const double ir = zr * den, ii = -zi * den;
    const double i2r = ir * ir - ii * ii, i2i = 2.0 * ir * ii;
    // sum_k c_k w^{-(2k-1)}, c_k = B_2k / (2k (2k - 1)), k = 1..8, Horner in 1/w^2
    const double c[8] = {1.0 / 12.0, -1.0 / 360.0, 1.0 / 1260.0, -1.0 / 1680.0,
                         1.0 / 1188.0, -691.0 / 360360.0, 1.0 / 156.0, -3617.0 / 122400.0};
    double sr = c[7], si = 0.0;
    for (int k = 6; k >= 0; --k) {
        const double t = sr * i2r - si * i2i + c[k];
        si = sr * i2i + si * i2r;
        sr = t;
    }
    const double tr = sr * ir - si * ii;
    const double ti = sr * ii + si * ir;
    // (w - 1/2) log w - w + log(2 pi)/2
    const double lmod = 0.5 * log(zr * zr + zi * zi);
    const double larg = atan2(zi, zr);
    const double ar = zr - 0.5;
    double re = ar * lmod - zi * larg - zr + 0.91893853320467274178 + tr;
    double im = ar * larg + zi * lmod - zi + ti;
    // divide by P
    re -= 0.5 * log(pr * pr + pim * pim);
    im -= atan2(pim, pr);
    *lg_re = re;
    *lg_im = im;
}

// h_lm (or h_lm e^{i m phi} when derotate). i = lm_index(l, m).
EOB_HD cdbl mode_eval(const FacCoeffs &fc, int l, int m, double pre_re, double pre_im, double eta, double r, double phi,
                      double pphi, double v, double Hreal, double vPhiInput, double h22_calib, bool derotate)
{
    if (eta > 0.25 && eta < 0.25 + 1e-4) eta = 0.25;
    const int i = lm_index(l, m);
    const double v2 = v * v;
    const double Omega = v2 * v;
    const double vh3 = Hreal * Omega;
    const double vh = cbrt(vh3);
    const double eulerlog = kEulerGamma + log(2.0 * m * v);
    const double vPhi = r * cbrt(vPhiInput) * Omega;
    const int eps = (l + m) % 2;
    // |Y| part and Newtonian amplitude: n_lm vPhi^(l+eps) (-1)^m Y_{l-eps}^m(pi/2, 0)
    double vpow = 1.0;
    for (int q = 0; q < l + eps; ++q) vpow *= vPhi;
    const double y0 = ((m % 2) ? -1.0 : 1.0) * ylm_equator(l - eps, m);
    const double S = (eps == 0) ? (Hreal * Hreal - 1.0) / (2.0 * eta) + 1.0 : v * pphi;
    // delta_lm
    double delta = 0.0, p = 1.0;
    for (int k = 1; k < 10; ++k) { p *= vh; delta = fma(fc.dvh[i][k], p, delta); }
    p = 1.0;
    for (int k = 1; k < 9; ++k) { p *= v; delta = fma(fc.dv[i][k], p, delta); }
    // rho_lm^l + f_lm
    double rho = 0.0;
    for (int k = kRhoDeg; k >= 1; --k) rho = (rho + fma(fc.rhol[i][k], eulerlog, fc.rho[i][k])) * v;
    rho += 1.0;
    if (l == 2 && m == 2) {
        const double v4 = v2 * v2;
        rho = fma(h22_calib, v4 * v4 * v4, rho);
    }
    double rpl = rho;
    for (int q = 1; q < l; ++q) rpl *= rho;
    double fr = 0.0;
    p = 1.0;
    for (int k = 1; k < 8; ++k) { p *= v; fr = fma(fc.fre[i][k], p, fr); }
    const double fi = fc.fim_vh6[i] * vh3 * vh3;
    cdbl rf = {rpl + fr, fi};
    if (eta == 0.25 && (m % 2)) rf = {fr, fi};
    // T_lm
    const double k = m * Omega;
    const double hk = Hreal * k;
    double lgr, lgi;
    cloggamma_shifted(l + 1.0, -2.0 * hk, &lgr, &lgi);
    double lfact = 0.0;
    for (int q = 2; q <= l; ++q) lfact += log((double)q);
    const double tmod = kPi * hk + lgr - lfact;
    double phase = 2.0 * hk * log(4.0 * k / 1.6487212707001281468) + lgi + delta;  // sqrt(e)
    if (!derotate) phase -= m * phi;
    double sp, cp;
    sincos(phase, &sp, &cp);
    const double amp = exp(tmod) * S * vpow * y0;
    const cdbl e = {amp * cp, amp * sp};
    return cmul(cmul(e, rf), cdbl{pre_re, pre_im});
}

}  // namespace eob
