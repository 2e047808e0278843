// FP64 issue-rate probe used by the benchmark to measure the denominator of
// the integrator's roofline on the device it runs on.
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
}  // namespace

// Component timing: every thread evaluates one piece of the right-hand side
// `iters` times on binary 0 of a prepared workspace (states varied slightly
// so nothing is hoisted).  With one warp per SM sub-partition the FP64 pipe
// sets the pace, so time / iters / 64 cycles = FP64 instructions per call.
template <int WHICH>
__global__ void k_component(const eob::BinaryRec *bins, int iters, double *out)
{
    const eob::BinaryRec &b = bins[0];
    const int lane = threadIdx.x & 31;
    double r = 12.0 + 1e-3 * threadIdx.x, pr = -1e-3, L = 3.9, acc = 0.0;
    for (int i = 0; i < iters; ++i) {
        r += 1e-9;
        if (WHICH == 0) {
            eob::HamEval e;
            eob::ham_eval(b.ham, r, pr, L, &e);
            acc += e.dHdr + e.dHdpr + e.dHdL + e.omega_c + e.Hreal;
        } else if (WHICH == 1) {
            acc += eob::flux_eval(b.flux, r, L, 0.0227 + 1e-12 * i, 0.987, 0.0226);
        } else if (WHICH == 2) {
            const double y[4] = {r, 0.0, pr, L};
            double k[4];
            eob::eob_rhs(b.ham, b.flux, y, k);
            acc += k[0] + k[1] + k[2] + k[3];
        } else if (WHICH == 3) {
            const double y[4] = {r, 0.0, pr, L};
            double k[4];
            eob::eob_rhs_group<16>(b.jets, b.flux, y, k, lane & 15);
            acc += k[0] + k[1] + k[2] + k[3];
        } else if (WHICH == 4) {
            acc += eob::flux_eval_group<16>(b.flux, L, 0.0227 + 1e-12 * i, 0.987, 0.0226, lane & 15);
        } else if (WHICH == 5) {
            acc += eob::flux_eval_group<32>(b.flux, L, 0.0227 + 1e-12 * i, 0.987, 0.0226, lane);
        } else if (WHICH == 6 || WHICH == 7) {
            eob::HamEval e;
            if (WHICH == 6) eob::ham_eval_group<16>(b.jets, r, pr, L, lane & 15, &e);
            else eob::ham_eval_group<32>(b.jets, r, pr, L, lane, &e);
            acc += e.dHdr + e.dHdpr + e.dHdL + e.omega_c + e.Hreal;
        } else if (WHICH == 8) {
            const double y[4] = {r, 0.0, pr, L};
            double k[4];
            eob::eob_rhs_group<32>(b.jets, b.flux, y, k, lane);
            acc += k[0] + k[1] + k[2] + k[3];
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// Round trip of the warp-pair barrier: every pair of the block passes `iters`
// barriers back to back (mode 0: suspending try_wait, as the integrator; mode
// 1: spinning test_wait); out[pair] = 1 if every wait completed in time.
__global__ void k_pair_sync_probe(int iters, int mode, int *out)
{
    __shared__ unsigned long long bars[eob::kPairMax];
    eob::pair_init(bars, (int)(blockDim.x / 64));
    const int pair = (int)(threadIdx.x >> 6);
    eob::PairSync ps{(unsigned)__cvta_generic_to_shared(&bars[pair]), 0u, true};
    for (int i = 0; i < iters; ++i) {
        if (mode == 0) eob::pair_sync(ps);
        else eob::pair_sync_spin(ps);
    }
    if ((threadIdx.x & 63) == 0) out[blockIdx.x * eob::kPairMax + pair] = ps.ok ? 1 : 0;
}

// Warp-pair right-hand side alone: each pair evaluates it `iters` times on
// binary 0 of a prepared workspace (state varied slightly), out[pair] = sum.
__global__ void k_pair_rhs_probe(const eob::BinaryRec *bins, int iters, double *out)
{
    __shared__ eob::PairXchg xch[eob::kPairMax];
    __shared__ unsigned long long bars[eob::kPairMax];
    eob::pair_init(bars, (int)(blockDim.x / 64));
    const int pair = (int)(threadIdx.x >> 6), role = (int)((threadIdx.x >> 5) & 1), lane = threadIdx.x & 31;
    eob::PairSync ps{(unsigned)__cvta_generic_to_shared(&bars[pair]), 0u, true};
    const eob::BinaryRec &b = bins[0];
    double r = 12.0 + 1e-3 * pair, acc = 0.0;
    for (int i = 0; i < iters; ++i) {
        r += 1e-9;
        const double y[4] = {r, 0.0, -1e-3, 3.9};
        double k[4];
        eob::eob_rhs_pair(b.jets, b.flux, y, k, lane, role, xch[pair], ps);
        acc += k[0] + k[1] + k[2] + k[3];
    }
    if ((threadIdx.x & 63) == 0) out[blockIdx.x * eob::kPairMax + pair] = ps.ok ? acc : 0.0;
}

extern "C" int eob_pair_probe(const void *bins, int which, int iters, void *out, int blocks, int threads,
                              cudaStream_t stream)
{
    if (!out || blocks < 1 || threads < 64 || threads > 64 * eob::kPairMax || threads % 64 || iters < 1)
        return EOB_E_ARG;
    if (which == 0 || which == 1) k_pair_sync_probe<<<blocks, threads, 0, stream>>>(iters, which, (int *)out);
    else if (which == 2 && bins) k_pair_rhs_probe<<<blocks, threads, 0, stream>>>((const eob::BinaryRec *)bins, iters, (double *)out);
    else return EOB_E_ARG;
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

extern "C" int eob_component_probe(const void *bins, int which, int iters, double *out, int blocks, int threads,
                                   cudaStream_t stream)
{
    if (!bins || !out || blocks < 1 || threads < 32 || threads > 1024 || iters < 1) return EOB_E_ARG;
    const eob::BinaryRec *b = (const eob::BinaryRec *)bins;
    switch (which) {
        case 0: k_component<0><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 1: k_component<1><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 2: k_component<2><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 3: k_component<3><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 4: k_component<4><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 5: k_component<5><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 6: k_component<6><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 7: k_component<7><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        case 8: k_component<8><<<blocks, threads, 0, stream>>>(b, iters, out); break;
        default: return EOB_E_ARG;
    }
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

// The hot path's own reciprocal, reciprocal cube root, logarithm and
// reciprocal square root next to the device library's, for accuracy tests:
// out[8 i + 0..7] = eob_rcp, 1/x, eob_rcbrt, rcbrt, eob_log, log, eob_rsqrt,
// eob_inv_eighth_root of x[i].
__global__ void k_math_probe(const double *x, int n, double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    double *o = out + 8 * (size_t)i;
    o[0] = eob::eob_rcp(v);
    o[1] = 1.0 / v;
    o[2] = eob::eob_rcbrt(v);
    o[3] = rcbrt(v);
    o[4] = eob::eob_log(v);
    o[5] = log(v);
    o[6] = eob::eob_rsqrt(v);
    o[7] = eob::eob_inv_eighth_root(v);
}

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
