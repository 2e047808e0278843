// Hamiltonian, its first derivatives and the circular-orbit frequency from the
// per-binary tables of ham_coeffs.h, written for FP64 issue rate.
//
// Replaces the reference's generated derivative expressions
// (src/EOB.cu:139-222, grad_Ham_align_AD_single) and its second gradient
// evaluation at p_r = 0 (src/EOB.cu:2611-2616).  Every function of r is
// carried as a jet (value, d/du) in u = 1/r; the only transcendental calls
// are one log (eob_log, fastlog.h), a square root, reciprocals and reciprocal square roots.
// No pow() anywhere: on GB300 one FP64 pow costs about 100 DFMA slots.
#pragma once
#include "ham_coeffs.h"
#include "fastlog.h"

namespace eob {

// 1/sqrt(x): the device's reciprocal square root (one instruction sequence
// instead of a square root and a division); on the host 1/sqrt(x)
EOB_HD double eob_rsqrt(double x)
{
#ifdef __CUDA_ARCH__
    return rsqrt(x);
#else
    return 1.0 / sqrt(x);
#endif
}

// Reciprocal and reciprocal cube root on the FP64 critical path.  A
// dependent FP64 instruction costs one issue slot of its SM sub-partition
// (64 cycles on GB300); the general-purpose division and rcbrt() take about
// 6 and 18 of them.  Both here start from a hardware seed and take one
// third-order Newton step (the truncated binomial series of (1 - e)^(-1/p)
// for the seed's relative residual e), which cubes the seed's relative error:
//
//   1/x:       y0 = rcp.approx.ftz.f64(x) (rel. error < 2^-19),
//              e = 1 - x y0,      y = y0 (1 + e + e^2)
//   x^(-1/3):  y0 = x^(-1/3) in single precision (rel. error ~2^-22),
//              e = 1 - x y0^3,    y = y0 (1 + e/3 + 2 e^2 / 9)
//
// Measured against the device's division and rcbrt() and extended-precision
// references over 10^6 arguments in [1e-6, 1e6]: within 0.51 and 0.77 ulp.
// Arguments are finite, nonzero and of normal range on the hot path (r >= 1,
// D_c ~ 1, 1 - e^(-m x) in (0, 1), omega in (0, 1)); x = 0 or x = inf give
// NaN, which the integrator's finiteness checks report, and the cube root's
// single-precision seed needs |x| within the float range (1e-38 .. 3e38;
// orbital frequencies are above 1e-6).  Host: 1/x and 1/cbrt(x).
EOB_HD double eob_rcp(double x)
{
#ifdef __CUDA_ARCH__
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
#else
    return 1.0 / x;
#endif
}

EOB_HD double eob_rcbrt(double x)
{
#ifdef __CUDA_ARCH__
    const double y = (double)rcbrtf((float)x);
    const double e = fma(-x, y * y * y, 1.0);
    return fma(y * e, fma(e, 2.0 / 9.0, 1.0 / 3.0), y);
#else
    return 1.0 / cbrt(x);
#endif
}

// x^(-1/8) (the step-size controller's err^(-1/8)) without pow(): a
// single-precision seed (FP32 pipe) refined by one third-order step for
// y^-8 = x, e = 1 - x y^8, y <- y (1 + e/8 + 9 e^2/128): 7 FP64 instructions
// instead of a reciprocal square root and two square roots (about 24).  x is
// first clamped to [1e-30, 1e30] (NaN passes through): the controller clamps
// the resulting scale to [1/3, 6], which every x outside that range reaches
// anyway.  Host: 1/sqrt(sqrt(sqrt(x))) of the clamped x.
EOB_HD double eob_inv_eighth_root(double x)
{
    x = (x < 1e-30) ? 1e-30 : ((x > 1e30) ? 1e30 : x);
#ifdef __CUDA_ARCH__
    const double y = (double)rsqrtf(sqrtf(sqrtf((float)x)));
    const double y2 = y * y, y4 = y2 * y2;
    const double e = fma(-x, y4 * y4, 1.0);
    return fma(y * e, fma(e, 9.0 / 128.0, 0.125), y);
#else
    return 1.0 / sqrt(sqrt(sqrt(x)));
#endif
}

struct HamEval {
    double H;        // H_real / nu  (reference evaluate_Ham_align_AD)
    double dHdr, dHdpr, dHdL;
    double Hreal;    // nu * H = M sqrt(1 + 2 nu (Heff - 1))
    double omega_c;  // dH/dpphi at p_r = 0
};

struct Jet {
    double v, d;
};

// f = sum_{k=0..n-1} c[k] u^k and df/du, Horner.
template <int N>
EOB_HD Jet poly_jet(const double *c, double u)
{
    double v = c[N - 1], d = 0.0;
#pragma unroll
    for (int k = N - 2; k >= 0; --k) {
        d = fma(d, u, v);
        v = fma(v, u, c[k]);
    }
    return {v, d};
}

EOB_HD void ham_eval(const HamCoeffs &h, double r, double pr, double L, HamEval *out)
{
    const double u = eob_rcp(r);
    const double lr = eob_log(r);
    const double su = eob_rsqrt(r);  // sqrt(u)
    const double u2 = u * u, u3 = u2 * u, u4 = u3 * u, u5 = u4 * u;

    // AK0 = P(u) + lr (l5 u^5 + l6 u^6) + h u^6 sqrt(u);  d(lr)/du = -1/u
    Jet ak0 = poly_jet<7>(h.ak0, u);
    {
        const double pl = u5 * fma(h.ak0l[6], u, h.ak0l[5]);
        const double dpl = u4 * fma(6.0 * h.ak0l[6], u, 5.0 * h.ak0l[5]);
        const double hv = h.ak0h * u5 * u * su;
        ak0.v += fma(lr, pl, hv);
        ak0.d += fma(lr, dpl, fma(6.5 * h.ak0h, u5 * su, -pl * r));
    }
    const Jet aka = poly_jet<7>(h.aka, u);
    const Jet S = {ak0.v + aka.v, ak0.d + aka.d};
    const Jet fa = {fma(fma(h.fa2, u, h.fa1), u, 1.0), fma(2.0 * h.fa2, u, h.fa1)};
    const Jet as = {1.0 + u4 * fma(fma(h.as6, u, h.as5), u, h.as4),
                    u3 * fma(fma(6.0 * h.as6, u, 5.0 * h.as5), u, 4.0 * h.as4)};
    const double ap2 = h.ap2;
    const Jet dc = {1.0 + ap2 * u2 * (1.0 + 2.0 * u), ap2 * u * (2.0 + 6.0 * u)};
    const double idc = eob_rcp(dc.v);
    const double sf = S.v * fa.v;
    const double na = sf * as.v;
    const double dna = (S.d * fa.v + S.v * fa.d) * as.v + sf * as.d;
    const Jet A = {na * idc, (dna - na * idc * dc.d) * idc};

    // Dbpm = Q(u) + lr (l4 u^4 + l5 u^5) + h u^5 sqrt(u)
    Jet db = poly_jet<6>(h.db, u);
    {
        const double pl = u4 * fma(h.dbl[5], u, h.dbl[4]);
        const double dpl = u3 * fma(5.0 * h.dbl[5], u, 4.0 * h.dbl[4]);
        const double hv = h.dbh * u5 * su;
        db.v += fma(lr, pl, hv);
        db.d += fma(lr, dpl, fma(5.5 * h.dbh, u4 * su, -pl * r));
    }
    const double g = fma(h.kb, u, 1.0);
    const double ad = ak0.v * db.v;
    Jet bnp;
    bnp.v = ad * g + u3 * fma(h.bs4, u, h.bs3) - 1.0 + ap2 * u2;
    bnp.d = (ak0.d * db.v + ak0.v * db.d) * g + ad * h.kb + u2 * fma(4.0 * h.bs4, u, 3.0 * h.bs3) + 2.0 * ap2 * u;
    // Bnpa = -(u^2 + 2 u^3) / Dc ;  c = u^2 (1 + apsq Bnpa)
    const double bnpa = -(u2 + 2.0 * u3) * idc;
    const double dbnpa = (-(2.0 * u + 6.0 * u2) - bnpa * dc.d) * idc;
    const double cf = fma(h.apsq, bnpa, 1.0);
    const Jet cu = {u2 * cf, 2.0 * u * cf + u2 * h.apsq * dbnpa};

    // q4, q6, q8
    const Jet q4 = {u2 * fma(fma(h.q4c[4], u, h.q4c[3]), u, h.q4c[2]) + u4 * fma(h.q4l, lr, h.q4h * su),
                    u * fma(fma(4.0 * h.q4c[4], u, 3.0 * h.q4c[3]), u, 2.0 * h.q4c[2]) +
                        u3 * fma(h.q4l, 4.0 * lr - 1.0, 4.5 * h.q4h * su)};
    const Jet q6 = {u2 * fma(h.q6h * su + h.q6c[3], u, h.q6c[2]),
                    u * fma(fma(3.5 * h.q6h, su, 3.0 * h.q6c[3]), u, 2.0 * h.q6c[2])};
    const Jet q8 = {u * fma(h.q8h * su + h.q8c[2], u, h.q8c[1]),
                    fma(fma(2.5 * h.q8h, su, 2.0 * h.q8c[2]), u, h.q8c[1])};

    const double p2 = pr * pr, L2 = L * L;
    const double qa = fma(p2, fma(p2, q8.v, q6.v), q4.v);
    const double qad = fma(p2, fma(p2, q8.d, q6.d), q4.d);
    const double W = 1.0 + p2 * (1.0 + bnp.v) + L2 * cu.v + p2 * p2 * qa;
    const double Wu = p2 * bnp.d + L2 * cu.d + p2 * p2 * qad;
    const double Wp = 2.0 * pr * ((1.0 + bnp.v) + p2 * fma(p2, fma(4.0 * p2, q8.v, 3.0 * q6.v), 2.0 * q4.v));
    const double WL = 2.0 * L * cu.v;

    const double AW = A.v * W;
    const double rAW = eob_rsqrt(AW);
    const double heven = AW * rAW;
    const double ih2 = 0.5 * rAW;
    const double hev_u = (A.d * W + A.v * Wu) * ih2;
    const double hev_p = A.v * Wp * ih2;
    const double hev_L = A.v * WL * ih2;

    // odd part: N = sum_j p2^j N_j(u), N_j triangular in u (k <= 4 - j)
    const double(*nc)[5] = h.nc;
    const Jet n0 = {nc[0][0] + u * (nc[0][1] + u * (nc[0][2] + u * (nc[0][3] + u * nc[0][4]))) + h.ncl[0][4] * u4 * lr,
                    nc[0][1] + u * (2.0 * nc[0][2] + u * (3.0 * nc[0][3] + u * 4.0 * nc[0][4])) +
                        h.ncl[0][4] * u3 * (4.0 * lr - 1.0)};
    const Jet n1 = {nc[1][0] + u * (nc[1][1] + u * (nc[1][2] + u * nc[1][3])) + h.ncl[1][3] * u3 * lr,
                    nc[1][1] + u * (2.0 * nc[1][2] + u * 3.0 * nc[1][3]) + h.ncl[1][3] * u2 * (3.0 * lr - 1.0)};
    const Jet n2 = {nc[2][0] + u * (nc[2][1] + u * nc[2][2]), nc[2][1] + 2.0 * u * nc[2][2]};
    const Jet n3 = {nc[3][0] + u * nc[3][1], nc[3][1]};
    const double n4 = nc[4][0];
    const double Nv = n0.v + p2 * (n1.v + p2 * (n2.v + p2 * (n3.v + p2 * n4)));
    const double Nu = n0.d + p2 * (n1.d + p2 * (n2.d + p2 * n3.d));
    const double Np = n1.v + p2 * (2.0 * n2.v + p2 * (3.0 * n3.v + p2 * 4.0 * n4));
    const double u3i = u3 * idc;
    const double hodd = L * u3i * Nv;
    const double hodd_u = L * idc * (3.0 * u2 * Nv + u3 * Nu - u3 * Nv * idc * dc.d);
    const double hodd_p = L * u3i * Np * 2.0 * pr;
    const double hodd_L = u3i * Nv;

    const double heff = heven + hodd;
    const double nu = h.nu, M = h.M;
    const double s2 = fma(2.0 * nu, heff - 1.0, 1.0);
    const double rs = eob_rsqrt(s2);
    const double s = s2 * rs;
    const double H = M * s / nu;
    const double f = M * rs;  // M^2 / (nu H)
    out->H = H;
    out->Hreal = M * s;
    out->dHdr = -u2 * f * (hev_u + hodd_u);
    out->dHdpr = f * (hev_p + hodd_p);
    out->dHdL = f * (hev_L + hodd_L);

    // circular frequency: dH/dL at p_r = 0
    const double W0 = 1.0 + L2 * cu.v;
    const double AW0 = A.v * W0;
    const double r0 = eob_rsqrt(AW0);
    const double hodd0 = L * u3i * n0.v;
    const double rs0 = eob_rsqrt(fma(2.0 * nu, fma(AW0, r0, hodd0) - 1.0, 1.0));
    out->omega_c = (M * rs0) * fma(A.v * L * cu.v, r0, u3i * n0.v);
}

}  // namespace eob
