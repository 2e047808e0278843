// Measurement and test hooks (no counterpart in the reference; not part of
// the waveform path):
//   eob_fp64_probe        the device's FP64 issue rate, the denominator of the
//                         integrator's roofline, measured where it runs;
//   eob_math_probe        the hot path's reciprocal, roots and logarithm next to
//                         the device library's, for accuracy tests;
//   eob_sync_expiry_hook  the multi-warp integrator's group barrier
//                         (pair_sync_limit, rhs_pair.cuh) with one warp of the
//                         chosen groups leaving early, so that a test can watch
//                         a bounded wait run out and the others finish normally.
#include "eob_device.cuh"
#include "rhs_pair.cuh"

namespace {
__global__ void k_fp64_probe(double *out, int iters)
{
    double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const double x = 1.0000001, y = 1e-9;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, x, y); a1 = fma(a1, x, y); a2 = fma(a2, x, y); a3 = fma(a3, x, y);
        a4 = fma(a4, x, y); a5 = fma(a5, x, y); a6 = fma(a6, x, y); a7 = fma(a7, x, y);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// out[10 i + 0..9] = eob_rcp, 1/x, eob_rcbrt, rcbrt, eob_log, log, eob_rsqrt,
// eob_inv_eighth_root, eob_expm1_neg (of min(x, 600)), expm1(-min(x, 600)) of x[i].
__global__ void k_math_probe(const double *x, int n, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    double *o = out + 10 * (size_t)i;
    o[0] = eob::eob_rcp(v);
    o[1] = 1.0 / v;
    o[2] = eob::eob_rcbrt(v);
    o[3] = rcbrt(v);
    o[4] = eob::eob_log(v);
    o[5] = log(v);
    o[6] = eob::eob_rsqrt(v);
    o[7] = eob::eob_inv_eighth_root(v);
    const double y = v < 600.0 ? v : 600.0;
    o[8] = eob::eob_expm1_neg(y);
    o[9] = expm1(-y);
}

constexpr int kHookThreads = 256;  // 8 warps: 4 pairs or 2 four-warp groups per block

// Groups of GW warps (2: a pair, 4: a four-warp group) pass `rounds` group
// barriers.  In every round each warp publishes round * 8 + its index in the
// group to shared memory (double-buffered by round parity) before it arrives,
// and after the barrier checks every value of its group.  In a group chosen by
// skip_mask (bit g for global group g < 32), warp skip_warp leaves the loop at
// round skip_round without arriving -- a partner that stopped answering --
// so the group's other warps wait at that barrier until limit_ns runs out.
// Per warp w: out[4 w + 0] = 1 if none of its waits ran out, [1] = barriers
// passed, [2] = values read back wrong, [3] = microseconds spent in the wait
// that ran out (0 if none).
template <int GW>
__global__ void k_sync_expiry(int rounds, unsigned skip_mask, int skip_round, int skip_warp,
                              unsigned long long limit_ns, int *out)
{
    constexpr int kGroups = kHookThreads / (32 * GW);
    __shared__ unsigned long long bars[kGroups];
    __shared__ int val[2][kGroups][GW];
    eob::group_init(bars, kGroups, 32 * GW);
    const int warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
    const int grp = warp / GW, role = warp % GW;
    const int ggrp = (int)blockIdx.x * kGroups + grp;
    const bool skipped = ggrp < 32 && ((skip_mask >> ggrp) & 1u);
    eob::PairSync ps{(unsigned)__cvta_generic_to_shared(&bars[grp]), 0u, true};
    int passed = 0, bad = 0;
    unsigned long long waited = 0;
    for (int r = 0; r < rounds; ++r) {
        if (skipped && role == skip_warp && r == skip_round) break;
        if (lane == 0) val[r & 1][grp][role] = r * 8 + role;
        const unsigned long long t0 = eob::global_ns();
        eob::pair_sync_limit(ps, limit_ns);
        if (!ps.ok) {
            waited = eob::global_ns() - t0;
            break;
        }
        ++passed;
        bool wrong = false;
        for (int j = 0; j < GW; ++j) wrong |= (val[r & 1][grp][j] != r * 8 + j);
        bad += __popc(__ballot_sync(0xffffffffu, wrong));
    }
    if (lane == 0) {
        int *o = out + 4 * ((size_t)blockIdx.x * (kHookThreads / 32) + warp);
        o[0] = ps.ok ? 1 : 0;
        o[1] = passed;
        o[2] = bad;
        o[3] = (int)(waited / 1000ull);
    }
}
}  // namespace

extern "C" int eob_math_probe(const double *x, int n, double *out, cudaStream_t stream)
{
    if (!x || !out || n < 1) return EOB_E_ARG;
    k_math_probe<<<(n + 255) / 256, 256, 0, stream>>>(x, n, out);
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

extern "C" int eob_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t stream)
{
    if (!out || blocks < 1 || threads < 1 || threads > 1024 || iters < 1) return EOB_E_ARG;
    k_fp64_probe<<<blocks, threads, 0, stream>>>(out, iters);
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

extern "C" int eob_sync_expiry_hook(int group_warps, int rounds, unsigned skip_mask, int skip_round, int skip_warp,
                                    long long limit_ns, int *out, int blocks, cudaStream_t stream)
{
    if (!out || (group_warps != 2 && group_warps != 4) || rounds < 1 || rounds > 4096 || skip_round < 0 ||
        skip_round >= rounds || skip_warp < 0 || skip_warp >= group_warps || limit_ns < 1000 ||
        limit_ns > 2000000000ll || blocks < 1 || blocks > 1024)
        return EOB_E_ARG;
    const unsigned long long lim = (unsigned long long)limit_ns;
    if (group_warps == 2)
        k_sync_expiry<2><<<blocks, kHookThreads, 0, stream>>>(rounds, skip_mask, skip_round, skip_warp, lim, out);
    else
        k_sync_expiry<4><<<blocks, kHookThreads, 0, stream>>>(rounds, skip_mask, skip_round, skip_warp, lim, out);
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}
