// Natural logarithm for the FP64 hot path: Tang's table-driven method
// (P. T. P. Tang, "Table-driven implementation of the logarithm function in
// IEEE floating-point arithmetic", ACM TOMS 16(4), 1990, 378-400).
//
// On GB300 every FP64 instruction of a lane group's critical path costs one
// FP64 issue slot of its SM sub-partition (64 cycles), and a general-purpose
// FP64 log takes about 36 of them.  Here the range reduction is integer work
// (exponent and the top mantissa bits select a breakpoint) and the FP64 part
// is 13 instructions:
//
//   x = 2^e m,  m in [1, 2),  j = round(128 (m - 1)),  F_j = 1 + j/128
//   z = m inv_j - 1        (one fma; inv_j = RN(1/F_j), |z| <= 2^-8)
//   log x = e ln2 + T_j + log1p(z),   T_j = -log(inv_j) (exact for the rounded inv_j)
//   log1p(z) = z + z^2 q(z),  q = -1/2 + z/3 - ... + z^5/7   (truncation < 2^-67)
//
// T_j and ln2 are split into a 40-bit head and a tail, so e ln2_hi + T_hi is
// exact; the result is within about one ulp of log x (checked against
// extended-precision references on the host and against the device's log on
// the GPU).  Non-positive, non-finite and subnormal arguments are handled
// without a table lookup in a branch the hot path never takes.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include "log_table.h"

#ifndef EOB_HD
#ifdef __CUDACC__
#define EOB_HD __host__ __device__ __forceinline__
#else
#define EOB_HD inline
#endif
#endif

namespace eob {

#ifndef __CUDA_ARCH__
using std::fma;
#endif

struct LogEntry {
    double inv, thi, tlo;
};

static constexpr LogEntry kLogTabH[129] = EOB_LOGTAB_INIT;
#ifdef __CUDACC__
__device__ const LogEntry kLogTabD[129] = EOB_LOGTAB_INIT;
#endif

EOB_HD const LogEntry &log_entry(int j)
{
#ifdef __CUDA_ARCH__
    return kLogTabD[j];
#else
    return kLogTabH[j];
#endif
}

EOB_HD int64_t dbl_bits(double x)
{
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    int64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

EOB_HD double bits_dbl(int64_t b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double(b);
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

// log(x) for finite x >= 2^-1022 (the caller's arguments: r >= 1 and
// v = omega^(1/3) in (0, 1)); other arguments go through eob_log below.
EOB_HD double eob_log_normal(int64_t bits)
{
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    const int64_t frac = bits & 0xfffffffffffffLL;
    const int j = (int)((frac + (1LL << 44)) >> 45);  // round(128 (m - 1)), 0..128
    const double m = bits_dbl(frac | 0x3ff0000000000000LL);
    const LogEntry &t = log_entry(j);
    const double z = fma(m, t.inv, -1.0);
    double q = 1.0 / 7.0;
    q = fma(q, z, -1.0 / 6.0);
    q = fma(q, z, 1.0 / 5.0);
    q = fma(q, z, -0.25);
    q = fma(q, z, 1.0 / 3.0);
    q = fma(q, z, -0.5);
    const double p = fma(z * z, q, z);
    const double de = (double)e;
    const double hi = fma(de, EOB_LN2_HI, t.thi);  // exact
    const double lo = fma(de, EOB_LN2_LO, t.tlo);
    return hi + (lo + p);
}

// arguments outside the normal positive range (NaN, negative, zero, +inf,
// subnormal): kept out of line on the device, so that every inlined log
// carries only the normal path (the kernels that inline it are large, and
// their instruction fetch is part of the critical path)
#ifdef __CUDACC__
static __host__ __device__ __noinline__
#else
inline
#endif
double eob_log_special(double x)
{
    const int64_t bits = dbl_bits(x);
    if (x != x || x < 0.0) return bits_dbl(0x7ff8000000000000LL);  // NaN
    if (x == 0.0) return -bits_dbl(0x7ff0000000000000LL);           // -inf
    if (bits == 0x7ff0000000000000LL) return x;                      // +inf
    // subnormal: scale by 2^54
    return eob_log_normal(dbl_bits(x * 18014398509481984.0)) - 54.0 * EOB_LN2_HI - 54.0 * EOB_LN2_LO;
}

EOB_HD double eob_log(double x)
{
    const int64_t bits = dbl_bits(x);
    // normal, positive, finite: exponent field in [1, 2046], sign clear
    if ((uint64_t)bits - 0x0010000000000000ULL < 0x7fe0000000000000ULL) return eob_log_normal(bits);
    return eob_log_special(x);
}

}  // namespace eob
