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

#ifdef __CUDA_ARCH__
// Conversions between double and float by integer operations.  On GB300 a
// conversion instruction (F64 <-> F32) has the latency of a DFMA (about 65
// cycles); these take a few integer instructions.  Both are
// for positive normal floats, 2^-126 <= x < 2^128: the exponent is rebiased
// (1023 - 127 = 896) and the mantissa shifted by 29 bits, truncating x to 24
// significant bits (a seed's argument) or extending f exactly.
__device__ __forceinline__ float f32_from_pos(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    return __uint_as_float(((hi - (896u << 20)) << 3) | (lo >> 29));
}

__device__ __forceinline__ double f64_from_pos(float f)
{
    const unsigned fb = __float_as_uint(f);
    return __hiloint2double((int)((fb >> 3) + (896u << 20)), (int)(fb << 29));
}

// x^p (p = -1/3, -1/8) of a positive float from the special-function unit:
// 2^(p log2 x), relative error about 2^-21 (a seed, never a result)
__device__ __forceinline__ float f32_pow_seed(float x, float p)
{
    float l, y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(l) : "f"(x));
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(p * l));
    return y;
}
#endif

// Reciprocal, reciprocal square root, reciprocal cube root and the step
// controller's x^(-1/8) on the FP64 critical path.  A dependent FP64
// instruction costs one issue slot of its SM sub-partition (64 cycles on
// GB300); the general-purpose division, rsqrt() and rcbrt() take about 6, 6
// and 18 of them.  Each here starts from a seed and takes one third-order
// Newton step (the truncated binomial series of (1 - e)^(-1/p) for the seed's
// relative residual e), which cubes the seed's relative error:
//
//   1/x:        y0 = rcp.approx.ftz.f64(x)   (rel. error < 2^-19),
//               e = 1 - x y0,      y = y0 (1 + e + e^2)
//   1/sqrt(x):  y0 = rsqrt.approx.ftz.f64(x),
//               e = 1 - x y0^2,    y = y0 (1 + e/2 + 3 e^2/8)
//   x^(-1/3):   y0 = 2^(-log2(x)/3) in single precision,
//               e = 1 - x y0^3,    y = y0 (1 + e/3 + 2 e^2/9)
//   x^(-1/8):   y0 = 2^(-log2(x)/8) in single precision,
//               e = 1 - x y0^8,    y = y0 (1 + e/8 + 9 e^2/128)
//
// The two FP64 seeds carry about 20 significant bits (their low words are
// zero), so y0^2 is exact and e is formed with a single rounding.  Measured
// against extended-precision references over 2.6e5 arguments in [1e-6, 1e6]
// (tests/test_gpu_math.py): within one ulp each.  Arguments are positive and
// of normal range on the hot path (r >= 1, D_c ~ 1, A W ~ 1, 1 - e^(-m x) in
// (0, 1), omega in (0, 1)); x = 0 or x = inf give NaN or inf, which the
// integrator's finiteness checks report, and the single-precision seeds need
// 2^-126 <= x < 2^128 (orbital frequencies are above 1e-6).  Host: the
// library's 1/x, 1/sqrt(x), 1/cbrt(x).
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

EOB_HD double eob_rsqrt(double x)
{
#ifdef __CUDA_ARCH__
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y * y, 1.0);
    return fma(y * e, fma(e, 0.375, 0.5), y);
#else
    return 1.0 / sqrt(x);
#endif
}

EOB_HD double eob_rcbrt(double x)
{
#ifdef __CUDA_ARCH__
    const double y = f64_from_pos(f32_pow_seed(f32_from_pos(x), -1.0f / 3.0f));
    const double e = fma(-x, y * y * y, 1.0);
    return fma(y * e, fma(e, 2.0 / 9.0, 1.0 / 3.0), y);
#else
    return 1.0 / cbrt(x);
#endif
}

// x^(-1/8) without pow(): 7 FP64 instructions instead of a reciprocal square
// root and two square roots (about 24).  x is first clamped to [1e-30, 1e30]
// (NaN passes through), by integer comparisons of its bits (a comparison of
// doubles takes an FP64 issue slot): the controller clamps the resulting
// scale to [1/3, 6], which every x outside that range reaches anyway.  Host:
// 1/sqrt(sqrt(sqrt(x))) of the clamped x.
EOB_HD double eob_inv_eighth_root(double x)
{
#ifdef __CUDA_ARCH__
    const long long b = __double_as_longlong(x);
    constexpr long long kLo = 0x39b4484bfeebc2a0LL;  // bits of 1e-30
    constexpr long long kHi = 0x46293e5939a08ceaLL;  // bits of 1e30
    constexpr long long kInf = 0x7ff0000000000000LL;
    // b < kLo: below 1e-30 or negative (or a NaN with the sign bit set,
    // which makes the scale finite; the caller ends the pass on err's NaN)
    x = (b < kLo) ? 1e-30 : ((b > kHi && b <= kInf) ? 1e30 : x);
    const double y = f64_from_pos(f32_pow_seed(f32_from_pos(x), -0.125f));
    const double y2 = y * y, y4 = y2 * y2;
    const double e = fma(-x, y4 * y4, 1.0);
    return fma(y * e, fma(e, 9.0 / 128.0, 0.125), y);
#else
    x = (x < 1e-30) ? 1e-30 : ((x > 1e30) ? 1e30 : x);
    return 1.0 / sqrt(sqrt(sqrt(x)));
#endif
}

// e^(-y) - 1 for 0 <= y < 700 (the m factors' arguments 4 pi m H omega lie
// in (0, 40)) by the table-driven method of P. T. P. Tang (ACM TOMS 15, 144
// (1989)): -y = (32 n + j) ln2/32 + r with |r| <= ln2/64, so that
// e^(-y) = 2^n 2^(j/32) e^r, e^r - 1 by its Taylor polynomial of degree 7
// (truncation below 5e-17 relative), the 32 values 2^(j/32) from a table
// (correctly rounded).  For n = j = 0 the polynomial is the result (S = 1
// below), with no cancellation in e^(-y) - 1; otherwise the result is within
// about 1.4e-16 in absolute terms (6e-15 relative to 1 - e^(-y) >= 0.0107:
// the table entry's rounding, that of S - 1 and of the last fma).  12 FP64
// instructions; exp() measures about 1150 cycles on GB300, 18 FP64 issue
// slots.  Host: expm1(-y).
#define EOB_EXP2_32_INIT                                                                                         \
    {0x1.0000000000000p+0, 0x1.059b0d3158574p+0, 0x1.0b5586cf9890fp+0, 0x1.11301d0125b51p+0, 0x1.172b83c7d517bp+0, \
     0x1.1d4873168b9aap+0, 0x1.2387a6e756238p+0, 0x1.29e9df51fdee1p+0, 0x1.306fe0a31b715p+0, 0x1.371a7373aa9cbp+0, \
     0x1.3dea64c123422p+0, 0x1.44e086061892dp+0, 0x1.4bfdad5362a27p+0, 0x1.5342b569d4f82p+0, 0x1.5ab07dd485429p+0, \
     0x1.6247eb03a5585p+0, 0x1.6a09e667f3bcdp+0, 0x1.71f75e8ec5f74p+0, 0x1.7a11473eb0187p+0, 0x1.82589994cce13p+0, \
     0x1.8ace5422aa0dbp+0, 0x1.93737b0cdc5e5p+0, 0x1.9c49182a3f090p+0, 0x1.a5503b23e255dp+0, 0x1.ae89f995ad3adp+0, \
     0x1.b7f76f2fb5e47p+0, 0x1.c199bdd85529cp+0, 0x1.cb720dcef9069p+0, 0x1.d5818dcfba487p+0, 0x1.dfc97337b9b5fp+0, \
     0x1.ea4afa2a490dap+0, 0x1.f50765b6e4540p+0}
#ifdef __CUDACC__
__device__ const double kExp2_32[32] = EOB_EXP2_32_INIT;
#endif

EOB_HD double eob_expm1_neg(double y)
{
#ifdef __CUDA_ARCH__
    constexpr double kShift = 6755399441055744.0;        // 1.5 2^52: round to integer in the low bits
    constexpr double kInvL = 0x1.71547652b82fep+5;       // 32 / ln 2
    constexpr double kLHi = 0x1.62e42fefa2000p-6;        // ln2/32, 40 significant bits
    constexpr double kLLo = 0x1.9ef35793c7673p-46;       // ln2/32 - kLHi
    const double t = fma(-y, kInvL, kShift);
    const double nd = t - kShift;                        // N = round(-y 32 / ln 2)
    const double r = fma(nd, -kLLo, fma(nd, -kLHi, -y));
    const int N = (int)__double2loint(t);                // two's complement N in the low word
    double q = fma(r, 1.0 / 5040.0, 1.0 / 720.0);
    q = fma(q, r, 1.0 / 120.0);
    q = fma(q, r, 1.0 / 24.0);
    q = fma(q, r, 1.0 / 6.0);
    q = fma(q, r, 0.5);
    const double p = fma(r * r, q, r);                   // e^r - 1 to degree 7
    // 2^n 2^(j/32) by adding n to the table entry's exponent field
    const double S = __longlong_as_double(__double_as_longlong(kExp2_32[N & 31]) + ((long long)(N >> 5) << 52));
    return fma(S, p, S - 1.0);                           // p itself when N = 0 (S = 1)
#else
    return expm1(-y);
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
        const double dpl = u4 * fma(h.d.ak0l6, u, h.d.ak0l5);
        const double hv = h.ak0h * u5 * u * su;
        ak0.v += fma(lr, pl, hv);
        ak0.d += fma(lr, dpl, fma(h.d.ak0h, u5 * su, -pl * r));
    }
    const Jet aka = poly_jet<7>(h.aka, u);
    const Jet S = {ak0.v + aka.v, ak0.d + aka.d};
    const Jet fa = {fma(fma(h.fa2, u, h.fa1), u, 1.0), fma(h.d.fa2, u, h.fa1)};
    const Jet as = {1.0 + u4 * fma(fma(h.as6, u, h.as5), u, h.as4),
                    u3 * fma(fma(h.d.as6, u, h.d.as5), u, h.d.as4)};
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
        const double dpl = u3 * fma(h.d.dbl5, u, h.d.dbl4);
        const double hv = h.dbh * u5 * su;
        db.v += fma(lr, pl, hv);
        db.d += fma(lr, dpl, fma(h.d.dbh, u4 * su, -pl * r));
    }
    const double g = fma(h.kb, u, 1.0);
    const double ad = ak0.v * db.v;
    Jet bnp;
    bnp.v = ad * g + u3 * fma(h.bs4, u, h.bs3) - 1.0 + ap2 * u2;
    bnp.d = (ak0.d * db.v + ak0.v * db.d) * g + ad * h.kb + u2 * fma(h.d.bs4, u, h.d.bs3) + h.d.two_ap2 * u;
    // Bnpa = -(u^2 + 2 u^3) / Dc ;  c = u^2 (1 + apsq Bnpa)
    const double bnpa = -(u2 + 2.0 * u3) * idc;
    const double dbnpa = (-(2.0 * u + 6.0 * u2) - bnpa * dc.d) * idc;
    const double cf = fma(h.apsq, bnpa, 1.0);
    const Jet cu = {u2 * cf, 2.0 * u * cf + u2 * h.apsq * dbnpa};

    // q4, q6, q8
    const Jet q4 = {u2 * fma(fma(h.q4c[4], u, h.q4c[3]), u, h.q4c[2]) + u4 * fma(h.q4l, lr, h.q4h * su),
                    u * fma(fma(h.d.q4c4, u, h.d.q4c3), u, h.d.q4c2) +
                        u3 * fma(h.q4l, 4.0 * lr - 1.0, h.d.q4h * su)};
    const Jet q6 = {u2 * fma(h.q6h * su + h.q6c[3], u, h.q6c[2]),
                    u * fma(fma(h.d.q6h, su, h.d.q6c3), u, h.d.q6c2)};
    const Jet q8 = {u * fma(h.q8h * su + h.q8c[2], u, h.q8c[1]),
                    fma(fma(h.d.q8h, su, h.d.q8c2), u, h.q8c[1])};

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
                    nc[0][1] + u * (h.d.nc02 + u * (h.d.nc03 + u * h.d.nc04)) +
                        h.ncl[0][4] * u3 * (4.0 * lr - 1.0)};
    const Jet n1 = {nc[1][0] + u * (nc[1][1] + u * (nc[1][2] + u * nc[1][3])) + h.ncl[1][3] * u3 * lr,
                    nc[1][1] + u * (h.d.nc12 + u * 3.0 * nc[1][3]) + h.ncl[1][3] * u2 * (3.0 * lr - 1.0)};
    const Jet n2 = {nc[2][0] + u * (nc[2][1] + u * nc[2][2]), nc[2][1] + 2.0 * u * nc[2][2]};
    const Jet n3 = {nc[3][0] + u * nc[3][1], nc[3][1]};
    const double n4 = nc[4][0];
    const double Nv = n0.v + p2 * (n1.v + p2 * (n2.v + p2 * (n3.v + p2 * n4)));
    const double Nu = n0.d + p2 * (n1.d + p2 * (n2.d + p2 * n3.d));
    const double Np = n1.v + p2 * (2.0 * n2.v + p2 * (3.0 * n3.v + p2 * h.d.four_n4));
    const double u3i = u3 * idc;
    const double hodd = L * u3i * Nv;
    const double hodd_u = L * idc * (3.0 * u2 * Nv + u3 * Nu - u3 * Nv * idc * dc.d);
    const double hodd_p = (L * u3i * Np) * (2.0 * pr);  // the same bits: the products by 2 are exact
    const double hodd_L = u3i * Nv;

    const double heff = heven + hodd;
    const double nu = h.nu, M = h.M;
    const double s2 = fma(h.d.two_nu, heff - 1.0, 1.0);
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
    const double rs0 = eob_rsqrt(fma(h.d.two_nu, fma(AW0, r0, hodd0) - 1.0, 1.0));
    out->omega_c = (M * rs0) * fma(A.v * L * cu.v, r0, u3i * n0.v);
}

}  // namespace eob
