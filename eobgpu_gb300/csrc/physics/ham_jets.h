// The Hamiltonian of ham_eval.h rearranged for a group of lanes that carry one
// binary: every function of r it needs is one of 16 "jets"
//
//   J(u) = sum_k c[k] u^k + log(r) sum_k l[k] u^k + sqrt(u) sum_k s[k] u^k,  k = 0..6,
//
// with value and d/du, so that the lanes of a group evaluate different jets
// with the same instruction stream (no divergence: only the coefficients
// differ).  The jets are then exchanged by shuffles and every lane runs the
// combination (A, Bnp, W, the odd part, the square roots).  Lanes of odd index
// run the combination at p_r = 0, which gives dH/dp_phi at p_r = 0 -- the
// circular frequency of the flux (src/EOB.cu:2611-2616) -- in the same
// instructions as the full state on the even lanes.
//
// The algebra is that of ham_eval() (same tables, same formulas); only the
// grouping of the polynomial evaluations differs.
#pragma once
#include "ham_eval.h"

namespace eob {

constexpr int kNumJets = 16;
constexpr int kJetTerms = 7;

enum JetId : int {
    J_AK0 = 0,  // AK0(u) with its log r and u^6 sqrt(u) terms
    J_AKA,      // AKa(u)
    J_FA,       // Fa(u) = 1 + fa1 u + fa2 u^2
    J_AS,       // AS(u) = 1 + as4 u^4 + as5 u^5 + as6 u^6
    J_DC,       // Dc(u) = 1 + ap2 u^2 + 2 ap2 u^3
    J_DB,       // Dbpm(u) with its log r and u^5 sqrt(u) terms
    J_G,        // 1 + kb u
    J_BX,       // bs3 u^3 + bs4 u^4 - 1 + ap2 u^2
    J_BNN,      // -(u^2 + 2 u^3): numerator of Bnpa
    J_Q4,
    J_Q6,
    J_Q8,
    J_N0,
    J_N1,
    J_N2,
    J_N3,
};

struct HamJets {
    double c[kNumJets][kJetTerms], l[kNumJets][kJetTerms], s[kNumJets][kJetTerms];
    double n4, apsq, nu, M;
    double inv8pinu;  // 1 / (8 pi nu): the flux's factor omega / (8 pi nu)
    double inv_nu;    // 1 / nu: H = H_real / nu without a division
    double two_nu;    // 2 nu (exact): s^2 = 1 + 2 nu (H_eff - 1)
    double M2;        // M^2 (the same product the right-hand sides formed per call)
    // The log r and sqrt(u) polynomials have one or two adjacent terms per
    // jet: L = u^k (a + b u) with k = lk (3..5) and lc = {a, b, k a, (k+1) b};
    // S = s u^k with k = sk (2..6) and sc = {s, k s} (zero where a jet has no
    // such part), evaluated from powers of u instead of degree-6 Horner sums.
    double lc[kNumJets][4], sc[kNumJets][2];
    signed char lk[kNumJets], sk[kNumJets];
};

EOB_HD void ham_jets_build(const HamCoeffs &h, HamJets *J)
{
    for (int j = 0; j < kNumJets; ++j)
        for (int k = 0; k < kJetTerms; ++k) J->c[j][k] = J->l[j][k] = J->s[j][k] = 0.0;
    for (int k = 0; k < 7; ++k) {
        J->c[J_AK0][k] = h.ak0[k];
        J->c[J_AKA][k] = h.aka[k];
    }
    J->l[J_AK0][5] = h.ak0l[5];
    J->l[J_AK0][6] = h.ak0l[6];
    J->s[J_AK0][6] = h.ak0h;
    J->c[J_FA][0] = 1.0;
    J->c[J_FA][1] = h.fa1;
    J->c[J_FA][2] = h.fa2;
    J->c[J_AS][0] = 1.0;
    J->c[J_AS][4] = h.as4;
    J->c[J_AS][5] = h.as5;
    J->c[J_AS][6] = h.as6;
    J->c[J_DC][0] = 1.0;
    J->c[J_DC][2] = h.ap2;
    J->c[J_DC][3] = 2.0 * h.ap2;
    for (int k = 0; k < 6; ++k) J->c[J_DB][k] = h.db[k];
    J->l[J_DB][4] = h.dbl[4];
    J->l[J_DB][5] = h.dbl[5];
    J->s[J_DB][5] = h.dbh;
    J->c[J_G][0] = 1.0;
    J->c[J_G][1] = h.kb;
    J->c[J_BX][0] = -1.0;
    J->c[J_BX][2] = h.ap2;
    J->c[J_BX][3] = h.bs3;
    J->c[J_BX][4] = h.bs4;
    J->c[J_BNN][2] = -1.0;
    J->c[J_BNN][3] = -2.0;
    for (int k = 2; k <= 4; ++k) J->c[J_Q4][k] = h.q4c[k];
    J->l[J_Q4][4] = h.q4l;
    J->s[J_Q4][4] = h.q4h;
    J->c[J_Q6][2] = h.q6c[2];
    J->c[J_Q6][3] = h.q6c[3];
    J->s[J_Q6][3] = h.q6h;
    J->c[J_Q8][1] = h.q8c[1];
    J->c[J_Q8][2] = h.q8c[2];
    J->s[J_Q8][2] = h.q8h;
    for (int k = 0; k <= 4; ++k) J->c[J_N0][k] = h.nc[0][k];
    J->l[J_N0][4] = h.ncl[0][4];
    for (int k = 0; k <= 3; ++k) J->c[J_N1][k] = h.nc[1][k];
    J->l[J_N1][3] = h.ncl[1][3];
    for (int k = 0; k <= 2; ++k) J->c[J_N2][k] = h.nc[2][k];
    for (int k = 0; k <= 1; ++k) J->c[J_N3][k] = h.nc[3][k];
    // sparse forms: the lowest log term (the tables above set at most two
    // adjacent ones, at k = 3..6) and the single sqrt(u) term (k = 2..6)
    for (int j = 0; j < kNumJets; ++j) {
        int kl = 3, ks = 2;
        for (int k = kJetTerms - 1; k >= 2; --k) {
            if (J->l[j][k] != 0.0) kl = k;
            if (J->s[j][k] != 0.0) ks = k;
        }
        if (kl > 5) kl = 5;
        const double a = J->l[j][kl], b = J->l[j][kl + 1];
        J->lk[j] = (signed char)kl;
        J->lc[j][0] = a;
        J->lc[j][1] = b;
        J->lc[j][2] = kl * a;
        J->lc[j][3] = (kl + 1) * b;
        J->sk[j] = (signed char)ks;
        J->sc[j][0] = J->s[j][ks];
        J->sc[j][1] = ks * J->s[j][ks];
    }
    J->n4 = h.nc[4][0];
    J->apsq = h.apsq;
    J->nu = h.nu;
    J->M = h.M;
    J->inv8pinu = 1.0 / (8.0 * kPi * h.nu);
    J->inv_nu = 1.0 / h.nu;
    J->two_nu = 2.0 * h.nu;
    J->M2 = h.M * h.M;
}

// powers of u for the sparse log r and sqrt(u) polynomials
struct UPow {
    double u, u2, u3, u4, u5;
};

EOB_HD UPow upow(double u)
{
    UPow p;
    p.u = u;
    p.u2 = u * u;
    p.u3 = p.u2 * u;
    p.u4 = p.u2 * p.u2;
    p.u5 = p.u4 * u;
    return p;
}

// u^k, k = 1..5 (selects, no arithmetic)
EOB_HD double upow_sel(const UPow &p, int k)
{
    return k == 1 ? p.u : k == 2 ? p.u2 : k == 3 ? p.u3 : k == 4 ? p.u4 : p.u5;
}

// the log(r) polynomial itself (L, dL/du), without the factor log r: four
// warps evaluate it beside log r and join the pieces afterwards (jet_join_s)
EOB_HD Jet jet_poly_l(const HamJets &J, int j, const UPow &p)
{
    const double *c = J.lc[j];
    const int k1 = J.lk[j] - 1;  // 2..4 (ham_jets_build keeps lk in 3..5)
    const double pk = (k1 == 2) ? p.u2 : ((k1 == 3) ? p.u3 : p.u4);  // u^(k-1)
    return {(pk * p.u) * fma(c[1], p.u, c[0]), pk * fma(c[3], p.u, c[2])};
}

// the sqrt(u) polynomial itself (S, dS/du), without the factor sqrt(u)
EOB_HD Jet jet_poly_s(const HamJets &J, int j, const UPow &p)
{
    const double pk = upow_sel(p, J.sk[j] - 1);  // u^(k-1)
    return {(pk * p.u) * J.sc[j][0], pk * J.sc[j][1]};
}

// the sqrt(u) polynomial with d/du (sqrt(u) S) / sqrt(u) = S' + r S / 2 in
// place of S', so that the join needs sqrt(u) alone (d sqrt(u)/du =
// sqrt(u) r / 2)
EOB_HD Jet jet_poly_s_t(const HamJets &J, int j, const UPow &p, double r)
{
    const Jet s = jet_poly_s(J, j, p);
    return {s.v, fma(0.5 * r, s.v, s.d)};
}

// value and d/du of jet j at u (r = 1/u, lr = log r, su = sqrt(u)): the
// polynomial part by Horner, the log r and sqrt(u) parts from their sparse
// forms; d(log r)/du = -r, d(sqrt u)/du = sqrt(u) r / 2
EOB_HD Jet jet_eval(const HamJets &J, int j, double u, double r, double lr, double su)
{
    const double *c = J.c[j];
    double cv = c[6], cd = 0.0;
#pragma unroll
    for (int k = 5; k >= 0; --k) {
        cd = fma(cd, u, cv);
        cv = fma(cv, u, c[k]);
    }
    const UPow p = upow(u);
    const Jet l = jet_poly_l(J, j, p), sq = jet_poly_s(J, j, p);
    Jet out;
    out.v = fma(su, sq.v, fma(lr, l.v, cv));
    out.d = fma(su, fma(0.5 * r, sq.v, sq.d), fma(lr, l.d, fma(-r, l.v, cd)));
    return out;
}

// H and its first derivatives at (r, pr, L) from the 16 jets
struct HamPart {
    double H, Hreal, dHdr, dHdpr, dHdL;
};

// The combination in pieces, so that the warps carrying one binary can
// evaluate them side by side: a warp pair runs comb_a with comb_b, then
// comb_even with comb_odd; four warps split them finer (comb_A, comb_C,
// comb_W, comb_N, then comb_even_parts with comb_odd_parts).  ham_combine()
// runs them in sequence.  Every path composes the same pieces.

// A(u) = S Fa As / Dc and its u-derivative, given 1 / Dc
struct PartA {
    double Av, Ad;
};

EOB_HD PartA comb_A(const Jet *jt, double idc)
{
    const Jet ak0 = jt[J_AK0], aka = jt[J_AKA], fa = jt[J_FA], as = jt[J_AS], dc = jt[J_DC];
    const double Sv = ak0.v + aka.v, Sd = ak0.d + aka.d;
    const double sf = Sv * fa.v;
    const double na = sf * as.v;
    const double dna = fma(Sd * fa.v + Sv * fa.d, as.v, sf * as.d);
    PartA o;
    o.Av = na * idc;
    o.Ad = fma(-o.Av, dc.d, dna) * idc;
    return o;
}

// the centrifugal coefficient c(u) = u^2 (1 + a^2 Bnpa), Bnpa = -(u^2 + 2 u^3) / Dc
struct PartC {
    double cuv, cud;
};

EOB_HD PartC comb_C(const HamJets &J, const Jet *jt, double u, double idc)
{
    const Jet dc = jt[J_DC], bnn = jt[J_BNN];
    const double u2 = u * u;
    const double bnpa = bnn.v * idc;
    const double dbnpa = fma(-bnpa, dc.d, bnn.d) * idc;
    const double cf = fma(J.apsq, bnpa, 1.0);
    PartC o;
    o.cuv = u2 * cf;
    o.cud = fma(2.0 * u, cf, u2 * J.apsq * dbnpa);
    return o;
}

struct CombA {
    double idc, Av, Ad, cuv, cud;
};

EOB_HD CombA comb_a(const HamJets &J, const Jet *jt, double u)
{
    CombA o;
    o.idc = eob_rcp(jt[J_DC].v);
    const PartA pa = comb_A(jt, o.idc);
    const PartC pc = comb_C(J, jt, u, o.idc);
    o.Av = pa.Av;
    o.Ad = pa.Ad;
    o.cuv = pc.cuv;
    o.cud = pc.cud;
    return o;
}

// B_np(u) and the p_r^4 coefficient q(u, p_r^2)
struct CombB {
    double bnpv, bnpd, qa, qad;
};

EOB_HD CombB comb_b(const Jet *jt, double p2)
{
    const Jet ak0 = jt[J_AK0], db = jt[J_DB], g = jt[J_G], bx = jt[J_BX], q4 = jt[J_Q4], q6 = jt[J_Q6],
              q8 = jt[J_Q8];
    CombB o;
    const double ad = ak0.v * db.v;
    o.bnpv = fma(ad, g.v, bx.v);
    o.bnpd = fma(fma(ak0.d, db.v, ak0.v * db.d), g.v, fma(ad, g.d, bx.d));
    o.qa = fma(p2, fma(p2, q8.v, q6.v), q4.v);
    o.qad = fma(p2, fma(p2, q8.d, q6.d), q4.d);
    return o;
}

// the part of W = 1 + p_r^2 (1 + B_np) + L^2 c + p_r^4 q that does not need c:
// W - L^2 c, its u-derivative minus L^2 c', and dW/dp_r
struct PartW {
    double W, Wu, Wp;
};

EOB_HD PartW comb_W(const Jet *jt, const CombB &b, double pr)
{
    const Jet q4 = jt[J_Q4], q6 = jt[J_Q6], q8 = jt[J_Q8];
    const double p2 = pr * pr;
    PartW o;
    o.W = fma(p2 * p2, b.qa, fma(p2, 1.0 + b.bnpv, 1.0));
    o.Wu = fma(p2 * p2, b.qad, p2 * b.bnpd);
    o.Wp = 2.0 * pr * ((1.0 + b.bnpv) + p2 * fma(p2, fma(4.0 * p2, q8.v, 3.0 * q6.v), 2.0 * q4.v));
    return o;
}

// comb_W with dW/dp_r cut in two, for four warps: comb_W_b keeps its B_np
// part 2 p_r (1 + B_np) and comb_Wp_q gives the rest,
// 2 p_r p_r^2 (2 q_4 + 3 p_r^2 q_6 + 4 p_r^4 q_8), from the jets alone
EOB_HD PartW comb_W_b_p2(const CombB &b, double pr, double p2)
{
    PartW o;
    o.W = fma(p2 * p2, b.qa, fma(p2, 1.0 + b.bnpv, 1.0));
    o.Wu = fma(p2 * p2, b.qad, p2 * b.bnpd);
    o.Wp = 2.0 * pr * (1.0 + b.bnpv);
    return o;
}

EOB_HD PartW comb_W_b(const CombB &b, double pr) { return comb_W_b_p2(b, pr, pr * pr); }

EOB_HD double comb_Wp_q_p2(const Jet *jt, double pr, double p2)
{
    return 2.0 * pr * (p2 * fma(p2, fma(4.0 * p2, jt[J_Q8].v, 3.0 * jt[J_Q6].v), 2.0 * jt[J_Q4].v));
}

EOB_HD double comb_Wp_q(const Jet *jt, double pr) { return comb_Wp_q_p2(jt, pr, pr * pr); }

// a piece of H_eff with its derivatives in u, p_r and L
struct HeffPart {
    double v, du, dp, dL;
};

// even part sqrt(A W)
EOB_HD HeffPart comb_even_parts(const PartA &a, const PartC &c, const PartW &w, double L)
{
    const double L2 = L * L;
    const double W = fma(L2, c.cuv, w.W);
    const double Wu = fma(L2, c.cud, w.Wu);
    // sqrt and the reciprocal from one reciprocal square root
    const double AW = a.Av * W;
    const double rAW = eob_rsqrt(AW);
    const double ih2 = 0.5 * rAW;
    HeffPart o;
    o.v = AW * rAW;
    o.du = fma(a.Ad, W, a.Av * Wu) * ih2;
    o.dp = a.Av * w.Wp * ih2;
    o.dL = (a.Av * L) * (c.cuv * rAW);  // A W_L / (2 sqrt(A W)), W_L = 2 L c
    return o;
}

EOB_HD HeffPart comb_even(const Jet *jt, const CombA &a, const CombB &b, double pr, double L)
{
    return comb_even_parts({a.Av, a.Ad}, {a.cuv, a.cud}, comb_W(jt, b, pr), L);
}

// N(u, p_r^2) = sum_j p_r^(2j) N_j(u) with its u- and p_r^2-derivatives
struct PartN {
    double Nv, Nu, Np;
};

EOB_HD PartN comb_N(const HamJets &J, const Jet *jt, double p2)
{
    const Jet n0 = jt[J_N0], n1 = jt[J_N1], n2 = jt[J_N2], n3 = jt[J_N3];
    const double n4 = J.n4;
    PartN o;
    o.Nv = n0.v + p2 * (n1.v + p2 * (n2.v + p2 * (n3.v + p2 * n4)));
    o.Nu = n0.d + p2 * (n1.d + p2 * (n2.d + p2 * n3.d));
    o.Np = n1.v + p2 * (2.0 * n2.v + p2 * (3.0 * n3.v + p2 * 4.0 * n4));
    return o;
}

// odd part L u^3 N / Dc
EOB_HD HeffPart comb_odd_parts(const Jet *jt, double u, double idc, const PartN &n, double pr, double L)
{
    const Jet dc = jt[J_DC];
    const double u2 = u * u, u3 = u2 * u;
    const double u3i = u3 * idc;
    HeffPart o;
    o.v = L * u3i * n.Nv;
    o.du = L * idc * (3.0 * u2 * n.Nv + u3 * n.Nu - u3 * n.Nv * idc * dc.d);
    o.dp = (L * u3i * n.Np) * (2.0 * pr);  // the same bits: both products by 2 are exact
    o.dL = u3i * n.Nv;
    return o;
}

EOB_HD HeffPart comb_odd(const HamJets &J, const Jet *jt, double u, double idc, double pr, double L)
{
    return comb_odd_parts(jt, u, idc, comb_N(J, jt, pr * pr), pr, L);
}

// H = M sqrt(1 + 2 nu (H_eff - 1)) / nu and its derivatives
EOB_HD HamPart comb_final(const HamJets &J, double u, const HeffPart &ev, const HeffPart &od)
{
    const double heff = ev.v + od.v;
    const double M = J.M;
    const double s2 = fma(J.two_nu, heff - 1.0, 1.0);
    const double rs = eob_rsqrt(s2);
    const double s = s2 * rs;
    const double f = M * rs;
    HamPart o;
    o.H = (M * s) * J.inv_nu;
    o.Hreal = M * s;
    o.dHdr = -(u * u) * f * (ev.du + od.du);
    o.dHdpr = f * (ev.dp + od.dp);
    o.dHdL = f * (ev.dL + od.dL);
    return o;
}

// comb_final from s^2 = 1 + 2 nu (H_eff - 1) and 1/s computed elsewhere
// (the four-warp group takes them from the warp that forms H_eff)
EOB_HD HamPart comb_final_s(const HamJets &J, double u, const HeffPart &ev, const HeffPart &od, double s2,
                            double rs)
{
    const double nu = J.nu, M = J.M;
    const double s = s2 * rs;
    const double f = M * rs;
    HamPart o;
    o.H = (M * s) * J.inv_nu;
    o.Hreal = M * s;
    o.dHdr = -(u * u) * f * (ev.du + od.du);
    o.dHdpr = f * (ev.dp + od.dp);
    o.dHdL = f * (ev.dL + od.dL);
    return o;
}

EOB_HD HamPart ham_combine(const HamJets &J, const Jet *jt, double u, double pr, double L)
{
    const CombA a = comb_a(J, jt, u);
    const CombB b = comb_b(jt, pr * pr);
    const HeffPart ev = comb_even(jt, a, b, pr, L);
    const HeffPart od = comb_odd(J, jt, u, a.idc, pr, L);
    return comb_final(J, u, ev, od);
}

// A jet split in pieces that the two warps of a pair evaluate: the
// polynomial part (P, dP/du) and the sqrt(u) part (su S, su (dS/du + r S / 2))
// -- jet_half(.., sq = false / true) -- and the log(r) part jet_part_l().
// poly + sqrt + log, added in that order, is jet_eval().
EOB_HD Jet jet_half(const HamJets &J, int j, bool sq, double u, double r, double su)
{
    const double *c = sq ? J.s[j] : J.c[j];
    double pv = c[6], pd = 0.0;
#pragma unroll
    for (int k = 5; k >= 0; --k) {
        pd = fma(pd, u, pv);
        pv = fma(pv, u, c[k]);
    }
    Jet out;
    out.v = su * pv;
    out.d = su * (sq ? fma(0.5 * r, pv, pd) : pd);
    return out;
}

EOB_HD Jet jet_part_l(const HamJets &J, int j, double u, double r, double lr)
{
    const Jet l = jet_poly_l(J, j, upow(u));
    Jet out;
    out.v = lr * l.v;
    out.d = fma(lr, l.d, -r * l.v);
    return out;
}

// a jet from its polynomial part p, the sqrt(u) and log polynomials s and l,
// su = sqrt(u), hs = r su / 2 = d sqrt(u) / du and lr = log r:
// value P + su S + lr L, d/du = P' + su S' + hs S - r L + lr L'
// the same from jet_poly_s_t's sqrt part (st.d = S' + r S / 2): one fma less
EOB_HD Jet jet_join_t(const Jet &p, const Jet &st, const Jet &l, double su, double lr, double r)
{
    Jet out;
    out.v = fma(lr, l.v, fma(su, st.v, p.v));
    out.d = fma(lr, l.d, fma(-r, l.v, fma(su, st.d, p.d)));
    return out;
}

EOB_HD Jet jet_join_s(const Jet &p, const Jet &s, const Jet &l, double su, double hs, double lr, double r)
{
    Jet out;
    out.v = fma(lr, l.v, fma(su, s.v, p.v));
    out.d = fma(lr, l.d, fma(-r, l.v, fma(hs, s.v, fma(su, s.d, p.d))));
    return out;
}

// Sequential use of the same pieces (host tests, and one-lane callers)
EOB_HD void ham_eval_jets(const HamJets &J, double r, double pr, double L, HamEval *out)
{
    const double u = eob_rcp(r), lr = eob_log(r), su = eob_rsqrt(r);
    Jet jt[kNumJets];
    for (int j = 0; j < kNumJets; ++j) jt[j] = jet_eval(J, j, u, r, lr, su);
    const HamPart a = ham_combine(J, jt, u, pr, L);
    const HamPart c = ham_combine(J, jt, u, 0.0, L);
    out->H = a.H;
    out->Hreal = a.Hreal;
    out->dHdr = a.dHdr;
    out->dHdpr = a.dHdpr;
    out->dHdL = a.dHdL;
    out->omega_c = c.dHdL;
}

#ifdef __CUDACC__
// Lane groups evaluate the jets in rounds, the seven jets with log r or
// sqrt(u) parts first (AK0, Dbpm, q4, q6, q8, N0, N1), so that rounds past
// them evaluate the polynomial part alone: with 8 lanes per binary the second
// round costs 12 FP64 instructions instead of jet_eval's 40.
constexpr int kJetsWithParts = 7;
__device__ const signed char kJetOrderD[kNumJets] = {J_AK0, J_DB, J_Q4, J_Q6, J_Q8, J_N0, J_N1, J_AKA,
                                                     J_FA,  J_AS, J_DC, J_G,  J_BX, J_BNN, J_N2, J_N3};

// position of jet j in that order
EOB_HD constexpr int jet_pos(int j)
{
    return j == J_AK0 ? 0 : j == J_DB ? 1 : j == J_Q4 ? 2 : j == J_Q6 ? 3 : j == J_Q8 ? 4 : j == J_N0 ? 5
         : j == J_N1 ? 6 : j == J_AKA ? 7 : j == J_FA ? 8 : j == J_AS ? 9 : j == J_DC ? 10 : j == J_G ? 11
         : j == J_BX ? 12 : j == J_BNN ? 13 : j == J_N2 ? 14 : 15;
}

// G lanes (2 .. 32, power of two) of one binary: jets split over the lanes,
// full state on even lanes and p_r = 0 on odd lanes; every lane returns the
// same result.  All 32 lanes of the warp must call it together.
template <int G>
__device__ __forceinline__ void ham_eval_group(const HamJets &J, double r, double pr, double L, int sub,
                                               HamEval *out)
{
    static_assert(G >= 2 && G <= 32 && (G & (G - 1)) == 0, "group size");
    const double u = eob_rcp(r), lr = eob_log(r), su = eob_rsqrt(r);
    constexpr int R = (kNumJets + G - 1) / G;
    double mv[R], md[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
        const int j = kJetOrderD[(q * G + sub) & (kNumJets - 1)];
        const Jet t = (q * G < kJetsWithParts) ? jet_eval(J, j, u, r, lr, su) : jet_half(J, j, false, u, r, 1.0);
        mv[q] = t.v;
        md[q] = t.d;
    }
    Jet jt[kNumJets];
#pragma unroll
    for (int j = 0; j < kNumJets; ++j) {
        const int p = jet_pos(j);
        jt[j].v = __shfl_sync(0xffffffffu, mv[p / G], p % G, G);
        jt[j].d = __shfl_sync(0xffffffffu, md[p / G], p % G, G);
    }
    const HamPart p = ham_combine(J, jt, u, (sub & 1) ? 0.0 : pr, L);
    out->H = __shfl_sync(0xffffffffu, p.H, 0, G);
    out->Hreal = __shfl_sync(0xffffffffu, p.Hreal, 0, G);
    out->dHdr = __shfl_sync(0xffffffffu, p.dHdr, 0, G);
    out->dHdpr = __shfl_sync(0xffffffffu, p.dHdpr, 0, G);
    out->dHdL = __shfl_sync(0xffffffffu, p.dHdL, 0, G);
    out->omega_c = __shfl_sync(0xffffffffu, p.dHdL, 1, G);
}
#endif

}  // namespace eob
