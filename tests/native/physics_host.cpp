// Host build of the product's device physics (eobgpu_gb300/csrc/physics/)
// for CPU tests: the same headers the CUDA kernels compile, exercised
// through a small extern "C" surface and compared with the oracle.
#include "../../eobgpu_gb300/csrc/physics/fac_coeffs.h"
#include "../../eobgpu_gb300/csrc/physics/ham_coeffs.h"
#include "../../eobgpu_gb300/csrc/physics/ham_eval.h"
#include "../../eobgpu_gb300/csrc/physics/ham_jets.h"
#include "../../eobgpu_gb300/csrc/physics/flux_eval.h"

extern "C" {

// state[4][n], add[80][n] (reference layout); out: H, dHdr, dHdpr, dHdL, omega_c per point
void phys_ham(const double *st, const double *add, int n, double *out)
{
    for (int i = 0; i < n; ++i) {
        eob::HamCoeffs h;
        eob::ham_coeffs_build(&h, add[i], add[n + i], add[2 * n + i], add[3 * n + i], add[5 * n + i], add[6 * n + i],
                              add[7 * n + i], add[8 * n + i]);
        eob::HamEval e;
        eob::ham_eval(h, st[i], st[2 * n + i], st[3 * n + i], &e);
        out[5 * i + 0] = e.H; out[5 * i + 1] = e.dHdr; out[5 * i + 2] = e.dHdpr; out[5 * i + 3] = e.dHdL;
        out[5 * i + 4] = e.omega_c;
    }
}

// the same through the 16-jet form used by lane groups (ham_jets.h)
void phys_ham_jets(const double *st, const double *add, int n, double *out)
{
    for (int i = 0; i < n; ++i) {
        eob::HamCoeffs h;
        eob::ham_coeffs_build(&h, add[i], add[n + i], add[2 * n + i], add[3 * n + i], add[5 * n + i], add[6 * n + i],
                              add[7 * n + i], add[8 * n + i]);
        eob::HamJets J;
        eob::ham_jets_build(h, &J);
        eob::HamEval e;
        eob::ham_eval_jets(J, st[i], st[2 * n + i], st[3 * n + i], &e);
        out[5 * i + 0] = e.H; out[5 * i + 1] = e.dHdr; out[5 * i + 2] = e.dHdpr; out[5 * i + 3] = e.dHdL;
        out[5 * i + 4] = e.omega_c;
    }
}

// the same through the pieces two warps of a pair evaluate side by side
// (jet halves + log part, comb_a/comb_b, comb_even/comb_odd, comb_final)
void phys_ham_pair(const double *st, const double *add, int n, double *out)
{
    for (int i = 0; i < n; ++i) {
        eob::HamCoeffs h;
        eob::ham_coeffs_build(&h, add[i], add[n + i], add[2 * n + i], add[3 * n + i], add[5 * n + i], add[6 * n + i],
                              add[7 * n + i], add[8 * n + i]);
        eob::HamJets J;
        eob::ham_jets_build(h, &J);
        const double r = st[i], L = st[3 * n + i];
        const double u = 1.0 / r, lr = eob::eob_log(r), su = sqrt(u);
        eob::Jet jt[eob::kNumJets];
        for (int j = 0; j < eob::kNumJets; ++j) {
            const eob::Jet a = eob::jet_half(J, j, false, u, r, 1.0), b = eob::jet_half(J, j, true, u, r, su);
            const eob::Jet l = eob::jet_part_l(J, j, u, r, lr);
            jt[j].v = (a.v + b.v) + l.v;
            jt[j].d = (a.d + b.d) + l.d;
        }
        double res[2][5];
        for (int z = 0; z < 2; ++z) {
            const double pr = z ? 0.0 : st[2 * n + i];
            const eob::CombA ca = eob::comb_a(J, jt, u);
            const eob::CombB cb = eob::comb_b(jt, pr * pr);
            const eob::HeffPart ev = eob::comb_even(jt, ca, cb, pr, L);
            const eob::HeffPart od = eob::comb_odd(J, jt, u, 1.0 / jt[eob::J_DC].v, pr, L);
            const eob::HamPart hp = eob::comb_final(J, u, ev, od);
            res[z][0] = hp.H; res[z][1] = hp.dHdr; res[z][2] = hp.dHdpr; res[z][3] = hp.dHdL; res[z][4] = hp.Hreal;
        }
        out[5 * i + 0] = res[0][0]; out[5 * i + 1] = res[0][1]; out[5 * i + 2] = res[0][2];
        out[5 * i + 3] = res[0][3]; out[5 * i + 4] = res[1][3];
    }
}

// the same through the pieces four warps evaluate: polynomial, sqrt(u) and
// log polynomials joined with sqrt(u) and log r (jet_join_s), then comb_A, comb_C,
// comb_W_b + comb_Wp_q, comb_N, the even and odd parts and comb_final
void phys_ham_quad(const double *st, const double *add, int n, double *out)
{
    for (int i = 0; i < n; ++i) {
        eob::HamCoeffs h;
        eob::ham_coeffs_build(&h, add[i], add[n + i], add[2 * n + i], add[3 * n + i], add[5 * n + i], add[6 * n + i],
                              add[7 * n + i], add[8 * n + i]);
        eob::HamJets J;
        eob::ham_jets_build(h, &J);
        const double r = st[i], L = st[3 * n + i];
        const double u = 1.0 / r, lr = eob::eob_log(r), su = eob::eob_rsqrt(r);
        eob::Jet jt[eob::kNumJets];
        for (int j = 0; j < eob::kNumJets; ++j)
            jt[j] = eob::jet_join_s(eob::jet_half(J, j, false, u, r, 1.0), eob::jet_poly_s(J, j, eob::upow(u)),
                                    eob::jet_poly_l(J, j, eob::upow(u)), su, 0.5 * r * su, lr, r);
        const double idc = 1.0 / jt[eob::J_DC].v;
        double res[2][5];
        for (int z = 0; z < 2; ++z) {
            const double pr = z ? 0.0 : st[2 * n + i];
            const eob::PartA a = eob::comb_A(jt, idc);
            const eob::PartC c = eob::comb_C(J, jt, u, idc);
            eob::PartW w = eob::comb_W_b(eob::comb_b(jt, pr * pr), pr);
            w.Wp = w.Wp + eob::comb_Wp_q(jt, pr);
            const eob::PartN nn = eob::comb_N(J, jt, pr * pr);
            const eob::HeffPart ev = eob::comb_even_parts(a, c, w, L);
            const eob::HeffPart od = eob::comb_odd_parts(jt, u, idc, nn, pr, L);
            const eob::HamPart hp = eob::comb_final(J, u, ev, od);
            res[z][0] = hp.H; res[z][1] = hp.dHdr; res[z][2] = hp.dHdpr; res[z][3] = hp.dHdL; res[z][4] = hp.Hreal;
        }
        out[5 * i + 0] = res[0][0]; out[5 * i + 1] = res[0][1]; out[5 * i + 2] = res[0][2];
        out[5 * i + 3] = res[0][3]; out[5 * i + 4] = res[1][3];
    }
}

// flux as a warp pair sums it: multipoles at sorted positions 0..31 (one
// warp) and 32..34 (the other), m factors per m, shared pieces from the two
// cube roots
static double flux_pair_host(const eob::FluxTable &t, double pphi, double omega, double Hreal, double omega_c)
{
    const double r0 = 1.0 / cbrt(omega), r1 = 1.0 / cbrt(omega_c);
    const eob::FluxLane f = eob::flux_lane_make_rv(t, pphi, omega, Hreal, omega * (r0 * r0), omega * (r1 * r1),
                                                   eob::eob_log(omega) * (1.0 / 3.0));
    double T[8], k4[8];
    for (int m = 1; m <= 8; ++m)
        eob::flux_m_factors(m, 4.0 * eob::kPi * Hreal * omega, Hreal * omega, &T[m - 1], &k4[m - 1]);
    static const signed char order[35] = {0, 1, 4, 3, 2, 8, 7, 6, 5, 13, 11, 9, 12, 10, 19, 17, 15, 18,
                                          16, 14, 26, 24, 22, 20, 25, 23, 21, 34, 33, 32, 31, 30, 29, 28, 27};
    double part[2] = {0.0, 0.0};
    for (int pos = 0; pos < 35; ++pos) {
        const int idx = order[pos];
        const int m = eob::lm_packed(idx) & 15;
        part[pos >= 32] += eob::flux_mode_lane<10>(t, idx, f, T[m - 1], k4[m - 1]);
    }
    return (part[0] + part[1]) * omega * omega / (8.0 * eob::kPi);
}

// flux as four warps sum it: series parts S^2 (rho^l + f)^2 times m-factor
// parts with v_phi^(2 (l + eps)) from v_phi^2 by squaring
static double flux_quad_host(const eob::FluxTable &t, double pphi, double omega, double Hreal, double omega_c)
{
    const double r0 = 1.0 / cbrt(omega), r1 = 1.0 / cbrt(omega_c);
    const double vphi = omega * (r1 * r1);
    const eob::FluxLane f = eob::flux_lane_make_rv(t, pphi, omega, Hreal, omega * (r0 * r0), vphi,
                                                   eob::eob_log(omega) * (1.0 / 3.0));
    double T[8], k4[8];
    for (int m = 1; m <= 8; ++m)
        eob::flux_m_factors(m, 4.0 * eob::kPi * Hreal * omega, Hreal * omega, &T[m - 1], &k4[m - 1]);
    // sorted positions 0..15 from the two halves of rho's series, the rest whole
    static const signed char order[35] = {0, 1, 4, 3, 2, 8, 7, 6, 5, 13, 11, 9, 12, 10, 19, 17, 15, 18,
                                          16, 14, 26, 24, 22, 20, 25, 23, 21, 34, 33, 32, 31, 30, 29, 28, 27};
    const double v5 = f.v2 * f.v2 * f.v;
    double sum = 0.0;
    for (int pos = 0; pos < 35; ++pos) {
        const int i = order[pos];
        const int m = eob::lm_packed(i) & 15;
        double s;
        if (pos < 16) {
            const double lo = eob::flux_rho_half(t, i, f, 0), hi = eob::flux_rho_half(t, i, f, 1);
            s = eob::flux_mode_s_rho(t, i, f, fma(fma(v5, hi, lo), f.v, 1.0));
        } else {
            s = eob::flux_mode_s<10>(t, i, f);
        }
        sum += (eob::flux_mode_b(t, i, T[m - 1], k4[m - 1]) * eob::flux_mode_vp_sq(i, vphi * vphi)) * s;
    }
    return sum * omega * omega / (8.0 * eob::kPi);
}

void phys_flux_pair(const double *st, const double *add, int n, double *out)
{
    for (int i = 0; i < n; ++i) {
        const double m1 = add[i], m2 = add[n + i], c1 = add[2 * n + i], c2 = add[3 * n + i];
        eob::HamCoeffs h;
        eob::ham_coeffs_build(&h, m1, m2, c1, c2, 0, 0, 0, 0);
        const double eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
        const double chiS = 0.5 * (c1 + c2), chiA = 0.5 * (c1 - c2);
        const double tpl = (1.0 - 2.0 * eta) * chiS + (m1 - m2) / (m1 + m2) * chiA;
        static eob::FacCoeffs fc;
        eob::fac_coeffs_build(&fc, 1, m1, m2, eta, tpl, chiS, chiA);
        double pre_re[35], pre_im[35];
        for (int j = 0; j < 35; ++j) { pre_re[j] = add[(10 + 2 * j) * n + i]; pre_im[j] = add[(11 + 2 * j) * n + i]; }
        static eob::FluxTable t;
        eob::flux_table_build(&t, fc, pre_re, pre_im, 0.0, h.nu);
        eob::HamEval e;
        eob::ham_eval(h, st[i], st[2 * n + i], st[3 * n + i], &e);
        out[2 * i] = eob::flux_eval_lanes(t, st[3 * n + i], e.dHdL, e.Hreal, e.omega_c);
        out[2 * i + 1] = flux_pair_host(t, st[3 * n + i], e.dHdL, e.Hreal, e.omega_c);
        out[2 * n + i] = flux_quad_host(t, st[3 * n + i], e.dHdL, e.Hreal, e.omega_c);
    }
}

// the hot path's logarithm
void phys_log(const double *x, int n, double *out)
{
    for (int i = 0; i < n; ++i) out[i] = eob::eob_log(x[i]);
}

// ODE right-hand side with coefficient tables built for each point's binary
void phys_rhs(const double *st, const double *add, int n, double *k)
{
    for (int i = 0; i < n; ++i) {
        const double m1 = add[i], m2 = add[n + i], c1 = add[2 * n + i], c2 = add[3 * n + i];
        eob::HamCoeffs h;
        eob::ham_coeffs_build(&h, m1, m2, c1, c2, add[5 * n + i], add[6 * n + i], add[7 * n + i], add[8 * n + i]);
        const double eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
        const double chiS = 0.5 * (c1 + c2), chiA = 0.5 * (c1 - c2);
        const double tpl = (1.0 - 2.0 * eta) * chiS + (m1 - m2) / (m1 + m2) * chiA;
        static eob::FacCoeffs fc;
        eob::fac_coeffs_build(&fc, 1, m1, m2, eta, tpl, chiS, chiA);
        double pre_re[35], pre_im[35];
        for (int j = 0; j < 35; ++j) { pre_re[j] = add[(10 + 2 * j) * n + i]; pre_im[j] = add[(11 + 2 * j) * n + i]; }
        static eob::FluxTable t;
        eob::flux_table_build(&t, fc, pre_re, pre_im, add[9 * n + i], h.nu);
        const double y[4] = {st[i], st[n + i], st[2 * n + i], st[3 * n + i]};
        double kk[4];
        eob::eob_rhs(h, t, y, kk);
        for (int q = 0; q < 4; ++q) k[q * n + i] = kk[q];
    }
}

// flux four ways: specialised per-mode code, the generic lane-group mode
// evaluator, the same with the lane-group shared pieces (out[3i .. 3i+2]),
// and the evaluator of groups of 8 or more lanes (out[3n + i])
void phys_flux_both(const double *st, const double *add, int n, double *out)
{
    for (int i = 0; i < n; ++i) {
        const double m1 = add[i], m2 = add[n + i], c1 = add[2 * n + i], c2 = add[3 * n + i];
        eob::HamCoeffs h;
        eob::ham_coeffs_build(&h, m1, m2, c1, c2, 0, 0, 0, 0);
        const double eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
        const double chiS = 0.5 * (c1 + c2), chiA = 0.5 * (c1 - c2);
        const double tpl = (1.0 - 2.0 * eta) * chiS + (m1 - m2) / (m1 + m2) * chiA;
        static eob::FacCoeffs fc;
        eob::fac_coeffs_build(&fc, 1, m1, m2, eta, tpl, chiS, chiA);
        double pre_re[35], pre_im[35];
        for (int j = 0; j < 35; ++j) { pre_re[j] = add[(10 + 2 * j) * n + i]; pre_im[j] = add[(11 + 2 * j) * n + i]; }
        static eob::FluxTable t;
        eob::flux_table_build(&t, fc, pre_re, pre_im, 0.0, h.nu);
        eob::HamEval e;
        eob::ham_eval(h, st[i], st[2 * n + i], st[3 * n + i], &e);
        const double omega = e.dHdL;
        out[3 * i] = eob::flux_eval(t, st[i], st[3 * n + i], omega, e.Hreal, e.omega_c);
        eob::FluxShared s;
        s.omega = omega;
        s.v = cbrt(omega);
        s.lv = log(s.v);
        const double vphi = st[i] * cbrt(1.0 / (e.omega_c * e.omega_c * st[i] * st[i] * st[i])) * omega;
        s.vphi2 = vphi * vphi;
        s.Se = (e.Hreal * e.Hreal - 1.0) / (2.0 * t.eta) + 1.0;
        s.Sodd = s.v * st[3 * n + i];
        s.x = 4.0 * eob::kPi * e.Hreal * omega;
        s.E1 = exp(-s.x);
        double sum = 0.0;
        for (int j = 0; j < 35; ++j) sum += eob::flux_mode_generic<10>(t, j, s, e.Hreal * omega);
        out[3 * i + 1] = sum * omega * omega / (8.0 * eob::kPi);
        // the lane-group form: shared pieces from the two cube roots
        const eob::FluxShared s2 = eob::flux_shared_make(t, st[3 * n + i], omega, e.Hreal, cbrt(omega), cbrt(e.omega_c));
        double sum2 = 0.0;
        for (int j = 0; j < 35; ++j) sum2 += eob::flux_mode_generic<10>(t, j, s2, e.Hreal * omega);
        out[3 * i + 2] = sum2 * omega * omega / (8.0 * eob::kPi);
        // lanes of 8 or more: m factors computed per m, table Gamma products
        out[3 * n + i] = eob::flux_eval_lanes(t, st[3 * n + i], omega, e.Hreal, e.omega_c);
    }
}

// Newtonian prefixes of one binary, interleaved (re, im) x 35
void phys_prefixes(double m1, double m2, double *out)
{
    for (int l = 2; l <= 8; ++l)
        for (int m = 1; m <= l; ++m) {
            const int i = eob::lm_index(l, m);
            eob::newton_prefix(m1, m2, l, m, &out[2 * i], &out[2 * i + 1]);
        }
}
}
