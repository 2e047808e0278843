// Radiation-reaction flux and force from per-binary tables, written for FP64
// issue rate.
//
// Restates EOBSpinFactorizedFlux / EOBFluxGetSpinFactorizedWaveform /
// RR_force (src/EOB.cu:2505-2642, 1705-1943): F = omega^2/(8 pi)
// sum_{l<=8, 1<=m<=l} m^2 |h_lm|^2 with the flux multipoles' truncated
// rho_lm.  Only |h_lm|^2 is needed, so every factor is squared in place:
//   |T_lm|^2 = (4 pi k)/(1 - exp(-4 pi k)) / (l!)^2 * prod_{j<=l} (4 k^2 + j^2),
//   k = m H_real omega,
// the same closed form the reference uses for its flux (src/EOB.cu:1740-1748).
// Shared pieces are computed once per call: one exp(-4 pi H omega) raised to
// the m-th power, one log(v) for every eulerlog_m, the products over j
// accumulated across l for each m, powers of vPhi^2 by multiplication.
#pragma once
#include "fac_coeffs.h"
#include "ham_eval.h"
#include "ham_jets.h"

namespace eob {

struct FluxTable {
    double rho[kNumLM][11];   // flux rho_lm: 1 + sum_{k=1..10} (rho[k] + rhol[k] eulerlog_m) v^k
    double rhol[kNumLM][11];
    double f1[kNumLM], f3[kNumLM];  // f_lm = f1 v + f3 v^3
    double nabs2[kNumLM];     // |Newtonian prefix|^2 Y_{l-eps}^m(pi/2)^2
    double h22calib;          // h22 calibration: rho_22 += h22calib v^12
    double eta;               // clamped symmetric mass ratio used by S_lm
    double equal_mass;        // 1.0 when eta == 0.25 (odd m use f_lm alone)
    double elog[kLMax + 1];   // gamma + log(2 m), m = 1..8: eulerlog_m(v) = elog[m] + log v
    double gmul[kNumLM];      // m^2 nabs2 / (l!)^2 (lane-group evaluator)
    double inv2eta;           // 1 / (2 eta) (lane-group evaluator)
    double fo_scale;          // inv2eta / (4 pi): F / omega = S omega fo_scale

    EOB_HD double c_rho(int i, int k) const { return rho[i][k]; }
    EOB_HD double c_rhol(int i, int k) const { return rhol[i][k]; }
    EOB_HD double c_f1(int i) const { return f1[i]; }
    EOB_HD double c_f3(int i) const { return f3[i]; }
    EOB_HD double c_nabs2(int i, int, int) const { return nabs2[i]; }
    EOB_HD double c_elog(int m) const { return elog[m]; }
    EOB_HD double c_eta() const { return eta; }
    EOB_HD double c_equal() const { return equal_mass; }
    EOB_HD double c_h22() const { return h22calib; }
    EOB_HD double c_gmul(int i, int, int) const { return gmul[i]; }
    EOB_HD double c_inv2eta() const { return inv2eta; }
    EOB_HD double c_fo_scale() const { return fo_scale; }
};

// The same flux inputs read straight from a FacCoeffs table and
// reference-layout prefixes (additionalArgs rows 10.., stride n); used by the
// reference-shaped entry points, which receive coefficients and prefixes
// separately (src/EOB.cu:2505-2561).
struct FacFluxView {
    const FacCoeffs *fc;
    const double *add;  // additionalArgs + system index
    int n;              // row stride of additionalArgs
    double eta, equal_mass, h22;
    EOB_HD double c_rho(int i, int k) const { return fc->rho[i][k]; }
    EOB_HD double c_rhol(int i, int k) const { return fc->rhol[i][k]; }
    EOB_HD double c_f1(int i) const { return fc->fre[i][1]; }
    EOB_HD double c_f3(int i) const { return fc->fre[i][3]; }
    EOB_HD double c_nabs2(int i, int l, int m) const
    {
        const double re = add[(size_t)(10 + 2 * i) * n], im = add[(size_t)(11 + 2 * i) * n];
        const double y = ylm_equator(l - (l + m) % 2, m);
        return (re * re + im * im) * y * y;
    }
    EOB_HD double c_elog(int m) const { return kEulerGamma + log(2.0 * m); }
    EOB_HD double c_eta() const { return eta; }
    EOB_HD double c_equal() const { return equal_mass; }
    EOB_HD double c_h22() const { return h22; }
    EOB_HD double c_gmul(int i, int l, int m) const
    {
        double f = 1.0;
        for (int j = 2; j <= l; ++j) f *= (double)j;
        return (double)(m * m) * c_nabs2(i, l, m) / (f * f);
    }
    EOB_HD double c_inv2eta() const { return 0.5 / eta; }
    EOB_HD double c_fo_scale() const { return c_inv2eta() * (0.25 / kPi); }
};

EOB_HD void flux_table_build(FluxTable *t, const FacCoeffs &fc, const double *prefix_re, const double *prefix_im,
                             double h22calib, double nu)
{
    for (int l = 2; l <= kLMax; ++l)
        for (int m = 1; m <= l; ++m) {
            const int i = lm_index(l, m);
            const int kmax = flux_rho_maxdeg(l, m);
            for (int k = 0; k <= 10; ++k) {
                t->rho[i][k] = (k >= 1 && k <= kmax) ? fc.rho[i][k] : 0.0;
                t->rhol[i][k] = (k >= 1 && flux_keeps_rhol(l, m, k)) ? fc.rhol[i][k] : 0.0;
            }
            t->f1[i] = flux_keeps_f(l, m, 1) ? fc.fre[i][1] : 0.0;
            t->f3[i] = flux_keeps_f(l, m, 3) ? fc.fre[i][3] : 0.0;
            const int eps = (l + m) % 2;
            const double y = ylm_equator(l - eps, m);
            t->nabs2[i] = (prefix_re[i] * prefix_re[i] + prefix_im[i] * prefix_im[i]) * y * y;
            double lf = 1.0;
            for (int j = 2; j <= l; ++j) lf *= (double)j;
            t->gmul[i] = (double)(m * m) * t->nabs2[i] / (lf * lf);
        }
    t->h22calib = h22calib;
    double eta = nu;
    if (eta > 0.25 && eta < 0.25 + 1e-4) eta = 0.25;
    t->eta = eta;
    t->inv2eta = 0.5 / eta;
    t->fo_scale = t->inv2eta * (0.25 / kPi);
    t->equal_mass = (eta == 0.25) ? 1.0 : 0.0;
    t->elog[0] = 0.0;
    for (int m = 1; m <= kLMax; ++m) t->elog[m] = kEulerGamma + log(2.0 * m);
}

// (l)!^2 for l = 0..8
EOB_HD constexpr double fact2_sq(int l)
{
    return l <= 1 ? 1.0 : (double)l * (double)l * fact2_sq(l - 1);
}

struct FluxShared {
    double v, lv, vphi2, Se, Sodd, x, omega, E1;
    double v12, S2e, S2o;  // v^12, S_even^2, S_odd^2 (one-lane flux)
};

// x^N for a compile-time N >= 1 by squaring
template <int N>
EOB_HD double ipow(double x)
{
    if constexpr (N == 1) return x;
    else if constexpr (N % 2 == 0) {
        const double h = ipow<N / 2>(x);
        return h * h;
    } else {
        return x * ipow<N - 1>(x);
    }
}

// prod_{j=1..l} (x + j^2) = sum_i kTprod[l][i] x^i (exact integers)
#define EOB_TPROD_INIT                                                                                       \
    {{1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},                                                          \
     {1.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},                                                          \
     {4.0, 5.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0},                                                          \
     {36.0, 49.0, 14.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0},                                                       \
     {576.0, 820.0, 273.0, 30.0, 1.0, 0.0, 0.0, 0.0, 0.0},                                                   \
     {14400.0, 21076.0, 7645.0, 1023.0, 55.0, 1.0, 0.0, 0.0, 0.0},                                           \
     {518400.0, 773136.0, 296296.0, 44473.0, 3003.0, 91.0, 1.0, 0.0, 0.0},                                   \
     {25401600.0, 38402064.0, 15291640.0, 2475473.0, 191620.0, 7462.0, 140.0, 1.0, 0.0},                    \
     {1625702400.0, 2483133696.0, 1017067024.0, 173721912.0, 14739153.0, 669188.0, 16422.0, 204.0, 1.0}}
static constexpr double kTprodH[kLMax + 1][kLMax + 1] = EOB_TPROD_INIT;
#ifdef __CUDACC__
__device__ const double kTprodD[kLMax + 1][kLMax + 1] = EOB_TPROD_INIT;
#endif

EOB_HD const double *tprod_row(int l)
{
#ifdef __CUDA_ARCH__
    return kTprodD[l];
#else
    return kTprodH[l];
#endif
}

// prod_{j=1..L} (x + j^2) for a compile-time L by Horner on the table's exact
// integer coefficients (leading coefficient 1): L FP64 instructions
template <int L, int Q>
struct TprodHorner {
    static EOB_HD double eval(double x, double p)
    {
        constexpr double c = kTprodH[L][Q];
        return TprodHorner<L, Q - 1>::eval(x, fma(p, x, c));
    }
};
template <int L>
struct TprodHorner<L, -1> {
    static EOB_HD double eval(double, double p) { return p; }
};
template <int L>
EOB_HD double tprod_poly(double x)
{
    constexpr double c = kTprodH[L][L - 1];
    return TprodHorner<L, L - 2>::eval(x, x + c);
}

// contribution m^2 |h_lm|^2 / (omega^2) of one (l, m) without the factors
// its m and parity share: P = prod_{j<=l} (4k^2 + j^2) times the constant
// m^2 |h^N_lm|^2 / (l!)^2 from the table, rho^2l and v_phi^(2 (l + eps));
// flux_m multiplies the even- and odd-parity sums by S_e^2 and S_o^2 and the
// whole by (m x)/(1 - e^{-m x}).  rho_lm by fma Horner, rho^l by squaring.
template <int l, int m, class Tab>
EOB_HD double flux_term(const Tab &t, const FluxShared &s, double P, const double *vp2)
{
    constexpr int i = (l - 2) * (l + 1) / 2 + (m - 1);
    constexpr int eps = (l + m) % 2;
    constexpr int kmax = (l == 2) ? 10 : (l == 3) ? 8 : (l == 4) ? 6 : (l == 5) ? ((m == 5) ? 6 : (m == 3 || m == 1) ? 5 : 4)
                                   : (l == 6) ? ((m % 2 == 0) ? 4 : 3) : (l == 7) ? ((m % 2 == 1) ? 3 : 2) : 2;
    constexpr bool has_log = (l <= 4);
    // eulerlog_m = gamma + log(2 m v); c_k = rho_k + rhol_k eulerlog_m
    const double elm = t.c_elog(m) + s.lv;
    auto ck = [&](int k) {
        double c = t.c_rho(i, k);
        if (has_log && (k == 6 || k == 7 || k == 8 || k == 10)) c = fma(t.c_rhol(i, k), elm, c);
        return c;
    };
    // rho = 1 + v (c_1 + v (c_2 + ... + v c_kmax))
    double acc = ck(kmax);
#pragma unroll
    for (int k = kmax - 1; k >= 1; --k) acc = fma(acc, s.v, ck(k));
    double rho = fma(acc, s.v, 1.0);
    if (l == 2 && m == 2) rho = fma(t.c_h22(), s.v12, rho);
    double rpl = ipow<l>(rho);
    const bool has_f = (l == 2 && m == 1) || (l == 3 && (m == 3 || m == 1)) || (l == 4 && (m == 3 || m == 1));
    if (has_f) {
        const double v2 = s.v * s.v;
        const double aux = s.v * fma(t.c_f3(i), v2, t.c_f1(i));
        rpl = (m % 2 == 1 && t.c_equal() != 0.0) ? aux : rpl + aux;
    } else if (m % 2 == 1) {
        rpl = (t.c_equal() != 0.0) ? 0.0 : rpl;
    }
    return t.c_gmul(i, l, m) * P * (rpl * rpl) * vp2[l + eps];
}

// Accumulate l = lmin..8 for one m into the even- and odd-parity sums; on
// entry P = prod_{j<=l} (4 k^2 + j^2), carried across l; HE, HO: a term of
// that parity is already in.
template <int m, int l, bool HE, bool HO, class Tab>
EOB_HD void flux_m_l(const Tab &t, const FluxShared &s, double P, double k2x4, const double *vp2, double &se,
                     double &so)
{
    constexpr bool even = ((l + m) % 2 == 0);
    const double v = flux_term<l, m, Tab>(t, s, P, vp2);
    if constexpr (even) se = HE ? se + v : v;
    else so = HO ? so + v : v;
    if constexpr (l < kLMax)
        flux_m_l<m, l + 1, HE || even, HO || !even, Tab>(t, s, P * (k2x4 + (double)((l + 1) * (l + 1))), k2x4, vp2,
                                                          se, so);
}

template <int m, class Tab>
EOB_HD double flux_m(const Tab &t, const FluxShared &s, double Em, double hw, const double *vp2)
{
    const double mx = m * s.x;
    const double Tpre = mx * eob_rcp(1.0 - Em);  // (4 pi k)/(1 - exp(-4 pi k)), k = m H omega
    const double km = m * hw;
    const double k2x4 = 4.0 * km * km;
    constexpr int lmin = (m > 2) ? m : 2;
    double se = 0.0, so = 0.0;
    flux_m_l<m, lmin, false, false, Tab>(t, s, tprod_poly<lmin>(k2x4), k2x4, vp2, se, so);
    return Tpre * fma(s.S2e, se, s.S2o * so);
}

// Radiation-reaction flux (before the division by nu of RR_force).
// omega: orbital frequency in the flux (dH/dpphi at the state); Hreal = nu H;
// omega_c: circular frequency (dH/dpphi at p_r = 0).
// flux_sum() is the multipole sum S with flux = S omega^2 / (8 pi).
template <class Tab>
EOB_HD double flux_sum(const Tab &t, double r, double pphi, double omega, double Hreal, double omega_c)
{
    FluxShared s;
    s.omega = omega;
    const double ro = eob_rcbrt(omega);
    s.v = omega * (ro * ro);  // omega^(1/3)
    s.lv = eob_log(s.v);
    // v_phi = r (omega_c^2 r^3)^(-1/3) omega = omega omega_c^(-2/3)
    (void)r;
    const double rc = eob_rcbrt(omega_c);
    const double vphi = omega * (rc * rc);
    s.vphi2 = vphi * vphi;
    s.Se = fma(Hreal * Hreal - 1.0, t.c_inv2eta(), 1.0);
    s.Sodd = s.v * pphi;
    const double v2 = s.v * s.v, v4 = v2 * v2;
    s.v12 = v4 * v4 * v4;
    s.S2e = s.Se * s.Se;
    s.S2o = s.Sodd * s.Sodd;
    s.x = 4.0 * kPi * Hreal * omega;
    double vp2[10];
    vp2[0] = 1.0;
#pragma unroll
    for (int q = 1; q < 10; ++q) vp2[q] = vp2[q - 1] * s.vphi2;
    const double E1 = exp(-s.x);
    const double hw = Hreal * omega;
    const double E2 = E1 * E1, E3 = E2 * E1, E4 = E2 * E2, E5 = E4 * E1, E6 = E3 * E3, E7 = E6 * E1, E8 = E4 * E4;
    double sum = flux_m<1, Tab>(t, s, E1, hw, vp2);
    sum += flux_m<2, Tab>(t, s, E2, hw, vp2);
    sum += flux_m<3, Tab>(t, s, E3, hw, vp2);
    sum += flux_m<4, Tab>(t, s, E4, hw, vp2);
    sum += flux_m<5, Tab>(t, s, E5, hw, vp2);
    sum += flux_m<6, Tab>(t, s, E6, hw, vp2);
    sum += flux_m<7, Tab>(t, s, E7, hw, vp2);
    sum += flux_m<8, Tab>(t, s, E8, hw, vp2);
    return sum;
}

template <class Tab>
EOB_HD double flux_eval(const Tab &t, double r, double pphi, double omega, double Hreal, double omega_c)
{
    return flux_sum(t, r, pphi, omega, Hreal, omega_c) * omega * omega / (8.0 * kPi);
}

// F / omega with F = flux / nu, from the multipole sum S: S omega / (8 pi nu)
// = S omega inv2eta / (4 pi) -- the reference's flux / nu / omega
// (src/EOB.cu:3046-3145) without its two divisions
template <class Tab>
EOB_HD double flux_over_omega(const Tab &t, double S, double omega)
{
    return (S * omega) * t.c_fo_scale();
}

// ODE right-hand side (src/EOB.cu:3046-3145): k = (dH/dpr, dH/dpphi,
// -dH/dr + F_r, F_phi), F = flux/nu, F_r = -pr/pphi F/omega, F_phi = -F/omega.
template <class Tab>
EOB_HD void eob_rhs(const HamCoeffs &h, const Tab &t, const double y[4], double k[4])
{
    HamEval e;
    ham_eval(h, y[0], y[2], y[3], &e);
    const double omega = e.dHdL;
    const double fo = flux_over_omega(t, flux_sum(t, y[0], y[3], omega, e.Hreal, e.omega_c), omega);
    k[0] = e.dHdpr;
    k[1] = omega;
    k[2] = -fma(y[2] * eob_rcp(y[3]), fo, e.dHdr);
    k[3] = -fo;
}

EOB_HD void lm_of_index(int i, int *l, int *m)
{
    int ll = 2;
    while (i >= ll) { i -= ll; ++ll; }
    *l = ll;
    *m = i + 1;
}

// Shared pieces of the lane-group flux from v = omega^(1/3) and
// w = omega_c^(1/3): vPhi = r (omega_c^2 r^3)^(-1/3) omega = omega / w^2
// (the reference's v_phi, src/EOB.cu:2610-2618, with the r's cancelled).
EOB_HD FluxShared flux_shared_make_rv(const FluxTable &t, double pphi, double omega, double Hreal, double v,
                                      double vphi)
{
    FluxShared s;
    s.omega = omega;
    s.v = v;
    s.lv = eob_log(v);
    s.vphi2 = vphi * vphi;
    s.Se = fma(Hreal * Hreal - 1.0, t.inv2eta, 1.0);
    s.Sodd = v * pphi;
    s.x = 4.0 * kPi * Hreal * omega;
    s.E1 = exp(-s.x);
    return s;
}

EOB_HD FluxShared flux_shared_make(const FluxTable &t, double pphi, double omega, double Hreal, double v, double w)
{
    return flux_shared_make_rv(t, pphi, omega, Hreal, v, omega / (w * w));
}

// one multipole of the flux, l and m at run time: m^2 |h_lm|^2 / omega^2
template <int KMAX>
EOB_HD double flux_mode_generic(const FluxTable &t, int i, const FluxShared &s, double hw)
{
    int l, m;
    lm_of_index(i, &l, &m);
    const int eps = (l + m) & 1;
    const double elm = t.elog[m] + s.lv;
    double rho = 0.0;
#pragma unroll
    for (int k = KMAX; k >= 1; --k) {
        double ck = t.rho[i][k];
        if (k == 6 || k == 7 || k == 8 || k == 10) ck = fma(t.rhol[i][k], elm, ck);
        rho = (rho + ck) * s.v;
    }
    rho += 1.0;
    if (i == lm_index(2, 2)) {
        const double v4 = (s.v * s.v) * (s.v * s.v);
        rho = fma(t.h22calib, v4 * v4 * v4, rho);
    }
    // rho^l by squaring (l = 2..8)
    const double r2 = rho * rho, r4 = r2 * r2;
    double rpl = (l & 4) ? r4 : 1.0;
    if (l & 2) rpl *= r2;
    if (l & 1) rpl *= rho;
    if (l == 8) rpl = r4 * r4;
    const double v2 = s.v * s.v;
    const double aux = s.v * fma(t.f3[i], v2, t.f1[i]);
    rpl = ((m & 1) && t.equal_mass != 0.0) ? aux : rpl + aux;
    const double S = eps ? s.Sodd : s.Se;
    // vphi^(2 (l + eps)) by squaring
    const int e = l + eps;
    const double p2 = s.vphi2 * s.vphi2, p4 = p2 * p2, p8 = p4 * p4;
    double vpw = (e & 8) ? p8 : 1.0;
    if (e & 4) vpw *= p4;
    if (e & 2) vpw *= p2;
    if (e & 1) vpw *= s.vphi2;
    // |T_lm|^2 (l!)^2 = (m x)/(1 - e^{-m x}) prod_{j<=l} (4 k^2 + j^2), k = m H omega
    const double km = m * hw;
    const double k4 = 4.0 * km * km;
    double P = 1.0;
#pragma unroll
    for (int j = 1; j <= kLMax; ++j) P *= (j <= l) ? (k4 + (double)(j * j)) : 1.0;
    // e^{-m x} from e^{-x} by squaring (m = 1..8)
    const double e2 = s.E1 * s.E1, e4 = e2 * e2;
    double Em = (m & 4) ? e4 : 1.0;
    if (m & 2) Em *= e2;
    if (m & 1) Em *= s.E1;
    if (m == 8) Em = e4 * e4;
    const double mx = m * s.x;
    const double T2 = mx * eob_rcp(1.0 - Em) * P;
    return t.gmul[i] * T2 * (S * S) * (rpl * rpl) * vpw;
}


// ---------------------------------------------------------------------------
// Multipole evaluation for lane groups of 8 or more lanes.  The factors that
// depend on m only are computed once per call on lanes 0..7 of the group (one
// exp(-m x) and one division per lane, in one instruction stream) and read by
// shuffles, the Gamma products prod_{j<=l} (4 k^2 + j^2) of every l among
// them (a running product on lane m - 1); powers of v_phi^2 are precomputed
// and selected.  (The warp pair and the four-warp group evaluate the Gamma
// product as a polynomial in 4 k^2 from a table, flux_mode_b_l.)


// per-call pieces shared by every multipole of one lane group
struct FluxLane {
    double v, v2, lv, v12, Se, Sodd;
    double vp[8];  // vphi^(2 e), e = 2..9
    double S2e, S2o;  // Se^2, Sodd^2
};

// the shared pieces from v and v_phi = omega / omega_c^(2/3), with log v
// given (a warp pair computes it as log(omega) / 3 on the other warp)
EOB_HD FluxLane flux_lane_make_rv(const FluxTable &t, double pphi, double omega, double Hreal, double v, double vphi,
                                  double lv)
{
    FluxLane f;
    f.v = v;
    f.lv = lv;
    const double v2 = v * v, v4 = v2 * v2;
    f.v2 = v2;
    f.v12 = v4 * v4 * v4;
    const double p1 = vphi * vphi;
    const double p2 = p1 * p1, p3 = p2 * p1, p4 = p2 * p2;
    f.vp[0] = p2;
    f.vp[1] = p3;
    f.vp[2] = p4;
    f.vp[3] = p4 * p1;
    f.vp[4] = p3 * p3;
    f.vp[5] = p3 * p4;
    f.vp[6] = p4 * p4;
    f.vp[7] = p4 * p4 * p1;
    f.Se = fma(Hreal * Hreal - 1.0, t.inv2eta, 1.0);
    f.Sodd = v * pphi;
    f.S2e = f.Se * f.Se;
    f.S2o = f.Sodd * f.Sodd;
    return f;
}

EOB_HD FluxLane flux_lane_make_lv(const FluxTable &t, double pphi, double omega, double Hreal, double v, double w,
                                  double lv)
{
    return flux_lane_make_rv(t, pphi, omega, Hreal, v, omega / (w * w), lv);
}

EOB_HD FluxLane flux_lane_make(const FluxTable &t, double pphi, double omega, double Hreal, double v, double w)
{
    return flux_lane_make_lv(t, pphi, omega, Hreal, v, w, eob_log(v));
}

// m x / (1 - e^{-m x}) and 4 k^2 = 4 (m H omega)^2 for one m (md = m as a
// double); 1 - e^{-m x} from eob_expm1_neg, without the cancellation of
// 1 - exp(-m x) at small m x
EOB_HD double flux_m_factor_T(double md, double x)
{
    const double xm = md * x;
    return xm * eob_rcp(-eob_expm1_neg(xm));
}

EOB_HD double flux_m_factor_k4(double md, double hw)
{
    const double km = md * hw;
    return 4.0 * km * km;
}

EOB_HD void flux_m_factors(int m, double x, double hw, double *T, double *k4)
{
    *T = flux_m_factor_T((double)m, x);
    *k4 = flux_m_factor_k4((double)m, hw);
}

// l and m of lm_index i, packed (l << 4) | m
#define EOB_LM_INIT                                                                                          \
    {0x21, 0x22, 0x31, 0x32, 0x33, 0x41, 0x42, 0x43, 0x44, 0x51, 0x52, 0x53, 0x54, 0x55, 0x61, 0x62, 0x63, 0x64, \
     0x65, 0x66, 0x71, 0x72, 0x73, 0x74, 0x75, 0x76, 0x77, 0x81, 0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88}

static constexpr unsigned char kLMH[kNumLM] = EOB_LM_INIT;
#ifdef __CUDACC__
__device__ const unsigned char kLMD[kNumLM] = EOB_LM_INIT;
#endif

EOB_HD int lm_packed(int i)
{
#ifdef __CUDA_ARCH__
    return kLMD[i];
#else
    return kLMH[i];
#endif
}

// m^2 |h_lm|^2 / omega^2 of multipole i as a product of two factors that
// separate warps can evaluate: flux_mode_a (rho_lm^l with the f_lm term, S^2
// and v_phi^(2 (l + eps)): the series in v) and flux_mode_b (m^2 |h^N_lm|^2 /
// (l!)^2 times (m x)/(1 - e^{-m x}) prod_{j<=l} (4 k^2 + j^2): the m factors).
// KMAX bounds the rho_lm series of the modes evaluated together.
// the series part without the v_phi power: S^2 (rho_lm^l + f_lm)^2
// the series part from rho_lm's sum: S^2 (rho_lm^l + f_lm)^2 with the h22
// calibration term
// a flag of the table (0.0 or 1.0) as a bool; on the device by its bits (a
// comparison of doubles takes an FP64 issue slot)
EOB_HD bool table_flag(double x)
{
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x) != 0;
#else
    return x != 0.0;
#endif
}

// lm: lm_packed(i), passed by callers that keep it in a register.  LMAX,
// LMIN: bounds on l of the multipoles evaluated together, so that what no
// multipole in that range needs is not formed: the powers of rho above
// LMAX; the h22 calibration term (the (2,2) multipole only) when LMIN > 2;
// and f_lm = f1 v + f3 v^3 when LMIN > 4 (it is zero from l = 5 on,
// flux_keeps_f), where rho^l + 0 is rho^l and f_lm alone (odd m at equal
// mass) is 0
template <int LMAX = kLMax, int LMIN = 2>
EOB_HD double flux_mode_s_rho_lm(const FluxTable &t, int i, int lm, const FluxLane &f, double rho)
{
    const int l = lm >> 4, m = lm & 15;
    const int eps = (l + m) & 1;
    if constexpr (LMIN <= 2) rho = fma((i == lm_index(2, 2)) ? t.h22calib : 0.0, f.v12, rho);
    // rho^l by squaring (l = 2..8)
    const double r2 = rho * rho, r4 = r2 * r2;
    double rpl = (LMAX >= 4 && (l & 4)) ? r4 : 1.0;
    if (l & 2) rpl *= r2;
    if (l & 1) rpl *= rho;
    if (LMAX >= 8 && l == 8) rpl = r4 * r4;
    if constexpr (LMIN <= 4) {
        const double aux = f.v * fma(t.f3[i], f.v2, t.f1[i]);
        rpl = ((m & 1) && table_flag(t.equal_mass)) ? aux : rpl + aux;
    } else {
        rpl = ((m & 1) && table_flag(t.equal_mass)) ? 0.0 : rpl;
    }
    const double S2 = eps ? f.S2o : f.S2e;
    return S2 * (rpl * rpl);
}

EOB_HD double flux_mode_s_rho(const FluxTable &t, int i, const FluxLane &f, double rho)
{
    return flux_mode_s_rho_lm(t, i, lm_packed(i), f, rho);
}

// elm = eulerlog_m(v) = elog[m] + log v, passed by callers that form it once per m
template <int KMAX, int LMAX = kLMax, int LMIN = 2>
EOB_HD double flux_mode_s_e(const FluxTable &t, int i, int lm, double elm, const FluxLane &f)
{
    // rho = 1 + v (c1 + v (c2 + ... + v cK)), c_k = rho_k + rhol_k eulerlog_m
    double acc = t.rho[i][KMAX];
    if (KMAX == 6 || KMAX == 7 || KMAX == 8 || KMAX == 10) acc = fma(t.rhol[i][KMAX], elm, acc);
#pragma unroll
    for (int k = KMAX - 1; k >= 1; --k) {
        double ck = t.rho[i][k];
        if (k == 6 || k == 7 || k == 8 || k == 10) ck = fma(t.rhol[i][k], elm, ck);
        acc = fma(acc, f.v, ck);
    }
    return flux_mode_s_rho_lm<LMAX, LMIN>(t, i, lm, f, fma(acc, f.v, 1.0));
}

template <int KMAX, int LMAX = kLMax, int LMIN = 2>
EOB_HD double flux_mode_s_lm(const FluxTable &t, int i, int lm, const FluxLane &f)
{
    return flux_mode_s_e<KMAX, LMAX, LMIN>(t, i, lm, t.elog[lm & 15] + f.lv, f);
}

template <int KMAX, int LMAX = kLMax, int LMIN = 2>
EOB_HD double flux_mode_s(const FluxTable &t, int i, const FluxLane &f)
{
    return flux_mode_s_lm<KMAX, LMAX, LMIN>(t, i, lm_packed(i), f);
}

// rho_lm's series (degree <= 10) in two halves for two lanes: half 0 gives
// c_1 + c_2 v + ... + c_5 v^4 and half 1 gives c_6 + c_7 v + ... + c_10 v^4,
// c_k = rho_k + rhol_k eulerlog_m (rhol_k is zero where the series has no
// log term); then rho = 1 + v (half 0 + v^5 half 1)
EOB_HD double flux_rho_half_e(const FluxTable &t, int i, double elm, const FluxLane &f, int half)
{
    const double *rh = t.rho[i] + (half ? 6 : 1), *rl = t.rhol[i] + (half ? 6 : 1);
    double acc = fma(rl[4], elm, rh[4]);
#pragma unroll
    for (int k = 3; k >= 0; --k) acc = fma(acc, f.v, fma(rl[k], elm, rh[k]));
    return acc;
}

EOB_HD double flux_rho_half(const FluxTable &t, int i, const FluxLane &f, int half)
{
    return flux_rho_half_e(t, i, t.elog[lm_packed(i) & 15] + f.lv, f, half);
}

// vphi^(2 (l + eps)) of multipole i selected from the precomputed powers
EOB_HD double flux_mode_vp(int i, const FluxLane &f)
{
    const int lm = lm_packed(i);
    const int l = lm >> 4, m = lm & 15;
    const int e = l + ((l + m) & 1) - 2;
    double vpw = f.vp[0];
#pragma unroll
    for (int q = 1; q < 8; ++q) vpw = (e == q) ? f.vp[q] : vpw;
    return vpw;
}

template <int KMAX, int LMAX = kLMax, int LMIN = 2>
EOB_HD double flux_mode_a(const FluxTable &t, int i, const FluxLane &f)
{
    return flux_mode_s<KMAX, LMAX, LMIN>(t, i, f) * flux_mode_vp(i, f);
}

// vphi^(2 (l + eps)) of multipole i from vphi^2 by squaring (l + eps = 2..9)
EOB_HD double flux_mode_vp_sq_lm(int lm, double vphi2)
{
    const int e = (lm >> 4) + (((lm >> 4) + (lm & 15)) & 1);
    const double p2 = vphi2 * vphi2, p4 = p2 * p2;
    double r = (e & 1) ? vphi2 : 1.0;
    if (e & 2) r *= p2;
    if (e & 4) r *= p4;
    if (e & 8) r *= p4 * p4;
    return r;
}

EOB_HD double flux_mode_vp_sq(int i, double vphi2) { return flux_mode_vp_sq_lm(lm_packed(i), vphi2); }

// LD: an upper bound on l of the multipoles evaluated together (the table's
// coefficients above l are zero)
template <int LD = kLMax>
EOB_HD double flux_mode_b_l(const FluxTable &t, int i, int l, double T, double k4)
{
    // prod_{j<=l} (4 k^2 + j^2)
    const double *c = tprod_row(l);
    double P = c[LD];
#pragma unroll
    for (int q = LD - 1; q >= 0; --q) P = fma(P, k4, c[q]);
    return t.gmul[i] * T * P;
}

template <int LD = kLMax>
EOB_HD double flux_mode_b(const FluxTable &t, int i, double T, double k4)
{
    return flux_mode_b_l<LD>(t, i, lm_packed(i) >> 4, T, k4);
}

template <int KMAX, int LD = kLMax, int LMIN = 2>
EOB_HD double flux_mode_lane(const FluxTable &t, int i, const FluxLane &f, double T, double k4)
{
    return flux_mode_b<LD>(t, i, T, k4) * flux_mode_a<KMAX, LD, LMIN>(t, i, f);
}

// Sequential use of the lane-group pieces (host tests)
EOB_HD double flux_eval_lanes(const FluxTable &t, double pphi, double omega, double Hreal, double omega_c)
{
    const FluxLane f = flux_lane_make(t, pphi, omega, Hreal, cbrt(omega), cbrt(omega_c));
    const double x = 4.0 * kPi * Hreal * omega, hw = Hreal * omega;
    double T[kLMax + 1], k4[kLMax + 1];
    for (int m = 1; m <= kLMax; ++m) flux_m_factors(m, x, hw, &T[m], &k4[m]);
    double sum = 0.0;
    for (int i = 0; i < kNumLM; ++i) {
        const int m = lm_packed(i) & 15;
        sum += flux_mode_lane<10>(t, i, f, T[m], k4[m]);
    }
    return sum * omega * omega / (8.0 * kPi);
}

#ifdef __CUDACC__
// ---------------------------------------------------------------------------
// The same flux with the 35 multipoles spread over a group of G lanes that
// carry the same binary (G = 2 .. 32).  Every lane runs one generic mode
// evaluation per round, with the mode picked by its position in the group, so
// the lanes never diverge; modes are ordered by the length of their rho_lm
// series so that each round's Horner loop is as short as its longest member.
// The partial sums are combined with butterfly shuffles inside the group.

// slot (lm_index) of the modes ordered by flux rho degree, longest first
// (global memory, not __constant__: the lanes of a warp read different entries)
__device__ const signed char kFluxOrder[kNumLM] = {
    0, 1,                                  // (2,1) (2,2): degree 10
    4, 3, 2,                               // (3,3) (3,2) (3,1): 8
    8, 7, 6, 5, 13,                        // (4,4..1) (5,5): 6
    11, 9,                                 // (5,3) (5,1): 5
    12, 10, 19, 17, 15,                    // (5,4) (5,2) (6,6) (6,4) (6,2): 4
    18, 16, 14, 26, 24, 22, 20,            // (6,5) (6,3) (6,1) (7,7) (7,5) (7,3) (7,1): 3
    25, 23, 21, 34, 33, 32, 31, 30, 29, 28, 27};  // (7,6) (7,4) (7,2) (8,8..1): 2
constexpr int kFluxDegSorted[kNumLM] = {10, 10, 8, 8, 8, 6, 6, 6, 6, 6, 5, 5, 4, 4, 4, 4, 4, 3,
                                        3,  3,  3, 3, 3, 3, 3, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2};

template <int G, int R>
__device__ __forceinline__ double flux_rounds(const FluxTable &t, const FluxShared &s, double hw, int sub)
{
    constexpr int first = R * G;
    if constexpr (first >= kNumLM) {
        return 0.0;
    } else {
        constexpr int KM = kFluxDegSorted[first];
        const int pos = first + sub;
        double here = 0.0;
        if (pos < kNumLM) here = flux_mode_generic<KM>(t, kFluxOrder[pos], s, hw);
        return here + flux_rounds<G, R + 1>(t, s, hw, sub);
    }
}

// l of the multipoles at the sorted positions of kFluxOrder, and the largest
// l among positions [first, first + n)
constexpr int kFluxLSorted[kNumLM] = {2, 2, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 5, 6, 6, 6, 6,
                                      6, 6, 7, 7, 7, 7, 7, 7, 7, 8, 8, 8, 8, 8, 8, 8, 8};
EOB_HD constexpr int flux_lmax(int first, int n)
{
    int m = 0;
    for (int p = first; p < first + n && p < kNumLM; ++p) m = kFluxLSorted[p] > m ? kFluxLSorted[p] : m;
    return m;
}

// the smallest l among positions [first, first + n)
EOB_HD constexpr int flux_lmin(int first, int n)
{
    int m = kLMax;
    for (int p = first; p < first + n && p < kNumLM; ++p) m = kFluxLSorted[p] < m ? kFluxLSorted[p] : m;
    return m;
}

// gp: on lane m - 1 of the group, prod_{j<=l} (4 k^2 + j^2) of that m for
// l = 2..8 (gp[l - 2]); each round reads only the l of its own range
template <int G, int R>
__device__ __forceinline__ double flux_rounds_lane(const FluxTable &t, const FluxLane &f, double Tm,
                                                   const double (&gp)[kLMax - 1], int sub)
{
    constexpr int first = R * G;
    if constexpr (first >= kNumLM) {
        return 0.0;
    } else {
        constexpr int KM = kFluxDegSorted[first];
        constexpr int LD = flux_lmax(first, G);
        constexpr int LN = flux_lmin(first, G);
        const int pos = first + sub;
        const int i = kFluxOrder[pos < kNumLM ? pos : kNumLM - 1];
        const int lm = lm_packed(i), l = lm >> 4, m = lm & 15;
        // the m factors live on lanes m-1 of the group
        const double T = __shfl_sync(0xffffffffu, Tm, m - 1, G);
        double P = 0.0;
#pragma unroll
        for (int q = LN; q <= LD; ++q) {
            const double pq = __shfl_sync(0xffffffffu, gp[q - 2], m - 1, G);
            P = (l == q) ? pq : P;
        }
        double here = (t.gmul[i] * T * P) * flux_mode_a<KM, LD, LN>(t, i, f);
        if (pos >= kNumLM) here = 0.0;
        return here + flux_rounds_lane<G, R + 1>(t, f, Tm, gp, sub);
    }
}

// the multipole sum S (flux = S omega^2 / (8 pi)) over a group of G lanes
template <int G>
__device__ double flux_sum_group(const FluxTable &t, double pphi, double omega, double Hreal, double omega_c, int sub)
{
    // reciprocal cube roots of omega (even lanes) and omega_c (odd lanes) in
    // one instruction stream: v = omega r_omega^2, v_phi = omega r_c^2
    const double rc = eob_rcbrt((sub & 1) ? omega_c : omega);
    const double r0 = __shfl_sync(0xffffffffu, rc, 0, G), r1 = __shfl_sync(0xffffffffu, rc, 1, G);
    const double v = omega * (r0 * r0), vphi = omega * (r1 * r1);
    double part;
    if constexpr (G >= 8) {
        const FluxLane f = flux_lane_make_rv(t, pphi, omega, Hreal, v, vphi, eob_log(v));
        double Tm, k4m;
        flux_m_factors((sub & 7) + 1, 4.0 * kPi * Hreal * omega, Hreal * omega, &Tm, &k4m);
        // the Gamma products of this lane's m for every l, by a running
        // product (an add and a multiply per l) instead of a Horner sum of
        // degree l in every round
        double gp[kLMax - 1];
        double p = k4m + 1.0;
#pragma unroll
        for (int l = 2; l <= kLMax; ++l) {
            p *= k4m + (double)(l * l);
            gp[l - 2] = p;
        }
        part = flux_rounds_lane<G, 0>(t, f, Tm, gp, sub);
    } else {
        const FluxShared s = flux_shared_make_rv(t, pphi, omega, Hreal, v, vphi);
        part = flux_rounds<G, 0>(t, s, Hreal * omega, sub);
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    return part;
}

template <int G>
__device__ void eob_rhs_group(const HamJets &h, const FluxTable &t, const double y[4], double k[4], int sub)
{
    HamEval e;
    ham_eval_group<G>(h, y[0], y[2], y[3], sub, &e);
    const double omega = e.dHdL;
    const double fo = flux_over_omega(t, flux_sum_group<G>(t, y[3], omega, e.Hreal, e.omega_c, sub), omega);
    k[0] = e.dHdpr;
    k[1] = omega;
    k[2] = -fma(y[2] * eob_rcp(y[3]), fo, e.dHdr);
    k[3] = -fo;
}
#endif

}  // namespace eob
