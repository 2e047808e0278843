// Reference-shaped synthesis and likelihood entry points of src/tdinterp.pyx:
//
//   eob_tdinterp2              TDInterp_wrap2 -> TD2 (src/interpolate.cu:441-549)
//   eob_tdinterp               TDInterp_wrap  -> TD  (src/interpolate.cu:323-438)
//   eob_all_in_one_likelihood  all_in_one_likelihood (src/interpolate.cu:553-627)
//
// The first two evaluate per-mode cubic splines (y + c1 x + c2 x^2 + c3 x^3,
// the reference's expression) on a caller time grid, rotate each mode by
// e^{-i m phi} with phi the orbital-phase spline and sum the modes; the third
// forms the frequency-domain residual d - (F+ h+ + Fx hx) e^{-2 pi i f tau}
// and sums |r|^2 / S_n per 1024-bin block of frequencies, one partial per
// (block, binary, channel) in the reference's layout.  Layouts, index
// arithmetic and argument meaning are the reference's, including TD2's sub-
// series stride old_lengths[b] inside a slot of old_length rows; knot indices
// are clamped into the binary's rows (the reference reads whatever memory an
// out-of-range index points at).  Complex
// arrays are interleaved (re, im) doubles.  All three are grid-stride
// streaming kernels: one thread per output sample (per frequency bin for the
// likelihood, four bins per thread), coalesced over samples.
#include "eob_device.cuh"

namespace {

constexpr int kMaxTdModes = 20;  // src/interpolate.cu:320 (MAX_EOB_MODES)
constexpr int kSumBins = 1024;   // frequency bins per likelihood partial (NUM_THREADS_SUM)
constexpr int kSumThreads = 256;

__device__ __forceinline__ double cubic(const double *y, const double *c1, const double *c2, const double *c3, size_t j,
                                        double x, double x2, double x3)
{
    return y[j] + c1[j] * x + c2[j] * x2 + c3[j] * x3;
}

// sum_k (re_k + i im_k) e^{-i m_k phi} of one sample; sub-series k of a
// binary's block start at base + k * stride.  One mode: sincos(m phi) as the
// reference.  Several modes: e^{i q phi} for q = 1 .. max m by complex
// products of e^{i phi} (one FP64 sincos per sample instead of one per mode;
// the powers agree with direct evaluation to ~q ulp), each mode taken at its
// own q; modes with m outside 1..8 use their own sincos.
__device__ __forceinline__ double2 mode_sum(const double *y, const double *c1, const double *c2, const double *c3,
                                            size_t base, size_t stride, int ind, double x, int K, const int *ms,
                                            int mmax)
{
    const double x2 = x * x, x3 = x * x2;
    const double phi = cubic(y, c1, c2, c3, base + 2 * (size_t)K * stride + ind, x, x2, x3);
    double hr = 0.0, hi = 0.0;
    auto add = [&](int k, double c, double s) {
        const double re = cubic(y, c1, c2, c3, base + (size_t)k * stride + ind, x, x2, x3);
        const double im = cubic(y, c1, c2, c3, base + (size_t)(K + k) * stride + ind, x, x2, x3);
        // (re + i im)(c - i s)
        hr += re * c + im * s;
        hi += im * c - re * s;
    };
    if (K == 1) {
        double s, c;
        sincos(ms[0] * phi, &s, &c);
        add(0, c, s);
        return make_double2(hr, hi);
    }
    double s1, cp1;
    sincos(phi, &s1, &cp1);
    double pc = 1.0, ps = 0.0;
    for (int q = 1; q <= mmax; ++q) {
        const double cn = pc * cp1 - ps * s1;
        ps = fma(ps, cp1, pc * s1);
        pc = cn;
        for (int k = 0; k < K; ++k)
            if (ms[k] == q) add(k, pc, ps);
    }
    for (int k = 0; k < K; ++k) {
        if (ms[k] < 1 || ms[k] > 8) {
            double s, c;
            sincos(ms[k] * phi, &s, &c);
            add(k, c, s);
        }
    }
    return make_double2(hr, hi);
}

// largest m in 1..8 among the modes (shared, after ms is loaded)
__device__ __forceinline__ int max_m(const int *ms, int K)
{
    int mm = 0;
    for (int k = 0; k < K; ++k)
        if (ms[k] >= 1 && ms[k] <= 8 && ms[k] > mm) mm = ms[k];
    return mm;
}

__global__ void k_td2(double2 *out, const double *dataTime, const double *ts, const double *y, const double *c1,
                      const double *c2, const double *c3, int old_length, const int *old_lengths, int data_length,
                      int B, int K, const int *ms_in, const int *inds, const int *lengths, int max_length)
{
    __shared__ int ms[kMaxTdModes];
    for (int k = threadIdx.x; k < K; k += blockDim.x) ms[k] = ms_in[k];
    __syncthreads();
    const int mmax = max_m(ms, K);
    for (int b = blockIdx.y; b < B; b += gridDim.y) {
        // a binary's samples stop at max_length and its knot indices stay
        // inside its slot (the reference trusts its caller for both)
        const int n = min(lengths[b], max_length);
        const int olh = min(old_lengths[b], old_length);
        const size_t base = (size_t)b * (2 * K + 1) * (size_t)old_length;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
            const int ind = min(max(inds[(size_t)max_length * b + i], 0), old_length - 1);
            const double x = dataTime[i] - ts[(size_t)b * old_length + ind];
            out[(size_t)b * data_length + i] = mode_sum(y, c1, c2, c3, base, (size_t)olh, ind, x, K, ms, mmax);
        }
    }
}

// one binary of TDInterp: its own arrays, samples ind_start .. ind_start + n of
// the time grid, written from element data_length of its output (the
// reference's templateChannels[data_length + i])
__global__ void k_td1(double2 *out, const double *dataTime, const double *ts, const double *y, const double *c1,
                      const double *c2, const double *c3, int old_length, int data_length, int K, const int *ms_in,
                      const int *inds, int ind_start, int n)
{
    __shared__ int ms[kMaxTdModes];
    for (int k = threadIdx.x; k < K; k += blockDim.x) ms[k] = ms_in[k];
    __syncthreads();
    const int mmax = max_m(ms, K);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
        const int ind = min(max(inds[i], 0), old_length - 1);
        const double x = dataTime[i + ind_start] - ts[ind];
        out[(size_t)data_length + i] = mode_sum(y, c1, c2, c3, 0, (size_t)old_length, ind, x, K, ms, mmax);
    }
}

// |d - h|^2 / S_n summed over one block of kSumBins frequencies for one
// (binary, channel): blockIdx.x = frequency block, y = binary, z = channel
__global__ void __launch_bounds__(kSumThreads) k_fd_lnl(double2 *temp_sum, const double2 *hp, const double2 *hc,
                                                        const double2 *data, const double *psd, const double *Fplus,
                                                        const double *Fcross, const double *tshift, double df, int B,
                                                        int nch, int N)
{
    __shared__ double warp_sum[kSumThreads / 32];
    for (int b = blockIdx.y; b < B; b += gridDim.y) {
        for (int ch = blockIdx.z; ch < nch; ch += gridDim.z) {
            const double fp = Fplus[(size_t)ch * B + b], fc = Fcross[(size_t)ch * B + b];
            const double tau = tshift[(size_t)ch * B + b];
            // the thread's bins are kSumThreads apart: e^{-2 pi i f tau} at the
            // first one, then rotations by e^{-2 pi i df kSumThreads tau}
            const int i0 = blockIdx.x * kSumBins + threadIdx.x;
            double s, co, sd, cd;
            sincos(2.0 * eob::kPi * (df * i0) * tau, &s, &co);
            sincos(2.0 * eob::kPi * (df * kSumThreads) * tau, &sd, &cd);
            double acc = 0.0;
#pragma unroll
            for (int q = 0; q < kSumBins / kSumThreads; ++q) {
                const int i = i0 + q * kSumThreads;
                if (q > 0) {
                    const double cn = co * cd - s * sd;
                    s = fma(s, cd, co * sd);
                    co = cn;
                }
                if (i < N) {
                    const double2 p = hp[(size_t)b * N + i], c = hc[(size_t)b * N + i];
                    const double2 d = data[(size_t)ch * N + i];
                    // (F+ h+ + Fx hx) (co - i s)
                    const double gr = fp * p.x + fc * c.x, gi = fp * p.y + fc * c.y;
                    const double rr = d.x - (gr * co + gi * s);
                    const double ri = d.y - (gi * co - gr * s);
                    // reciprocal (seed + one Newton step, 3 FP64 instructions)
                    // and a product instead of a division (about 6)
                    acc = fma(fma(rr, rr, ri * ri), eob::eob_rcp(psd[(size_t)ch * N + i]), acc);
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
            if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = acc;
            __syncthreads();
            if (threadIdx.x == 0) {
                double t = 0.0;
                for (int w = 0; w < kSumThreads / 32; ++w) t += warp_sum[w];
                temp_sum[((size_t)blockIdx.x * B + b) * nch + ch] = make_double2(t, 0.0);
            }
            __syncthreads();
        }
    }
}

int grid_for(long long n, int bs)
{
    long long g = (n + bs - 1) / bs;
    return (int)(g < 1 ? 1 : (g > 65535 ? 65535 : g));
}

int ret(cudaError_t e) { return e == cudaSuccess ? EOB_OK : EOB_E_CUDA; }

}  // namespace

extern "C" {

int eob_tdinterp2(double *templateChannels, const double *dataTime, const double *ts, const double *propArrays,
                  const double *c1, const double *c2, const double *c3, int old_length, const int *old_lengths,
                  int data_length, int numBinAll, int numModes, const int *ls, const int *ms, const int *inds,
                  const int *lengths, int max_length, cudaStream_t stream)
{
    (void)ls;  // the reference reads l but only m enters the rotation
    if (numBinAll < 0 || numModes < 1 || numModes > kMaxTdModes || old_length < 1 || max_length < 0 ||
        data_length < max_length)
        return EOB_E_ARG;
    if (numBinAll == 0 || max_length == 0) return EOB_OK;
    if (!templateChannels || !dataTime || !ts || !propArrays || !c1 || !c2 || !c3 || !old_lengths || !ms || !inds ||
        !lengths)
        return EOB_E_ARG;
    const int bs = 256;
    dim3 grid(grid_for(max_length, bs), numBinAll < 65535 ? numBinAll : 65535);
    k_td2<<<grid, bs, 0, stream>>>((double2 *)templateChannels, dataTime, ts, propArrays, c1, c2, c3, old_length,
                                   old_lengths, data_length, numBinAll, numModes, ms, inds, lengths, max_length);
    return ret(cudaGetLastError());
}

int eob_tdinterp(const long long *templateChannels_ptrs, const double *dataTime, const long long *tsAll,
                 const long long *propArraysAll, const long long *c1All, const long long *c2All,
                 const long long *c3All, const int *old_lengths, int data_length, int numBinAll, int numModes,
                 const int *ls, const int *ms, const long long *inds_ptrs, const int *inds_start,
                 const int *ind_lengths, cudaStream_t stream)
{
    (void)ls;
    if (numBinAll < 0 || numModes < 1 || numModes > kMaxTdModes || data_length < 0) return EOB_E_ARG;
    if (numBinAll == 0) return EOB_OK;
    if (!templateChannels_ptrs || !dataTime || !tsAll || !propArraysAll || !c1All || !c2All || !c3All ||
        !old_lengths || !ms || !inds_ptrs || !inds_start || !ind_lengths)
        return EOB_E_ARG;
    // per-binary metadata are host arrays, as in the reference's host loop
    // (src/interpolate.cu:401-431); one launch per binary on the caller's stream
    const int bs = 256;
    for (int b = 0; b < numBinAll; ++b) {
        const int n = ind_lengths[b];
        if (n < 0 || old_lengths[b] < 1) return EOB_E_ARG;
        if (n == 0) continue;
        k_td1<<<grid_for(n, bs), bs, 0, stream>>>(
            (double2 *)templateChannels_ptrs[b], dataTime, (const double *)tsAll[b], (const double *)propArraysAll[b],
            (const double *)c1All[b], (const double *)c2All[b], (const double *)c3All[b], old_lengths[b], data_length,
            numModes, ms, (const int *)inds_ptrs[b], inds_start[b], n);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return EOB_E_CUDA;
    }
    return EOB_OK;
}

int eob_all_in_one_likelihood(double *temp_sum, const double *hp_fd, const double *hc_fd, const double *data,
                              const double *psd, const double *Fplus, const double *Fcross, const double *time_shift,
                              double df, int num_bin_all, int nchannels, int data_length, cudaStream_t stream)
{
    if (num_bin_all < 0 || nchannels < 0 || data_length < 0) return EOB_E_ARG;
    if (num_bin_all == 0 || nchannels == 0 || data_length == 0) return EOB_OK;
    if (!temp_sum || !hp_fd || !hc_fd || !data || !psd || !Fplus || !Fcross || !time_shift) return EOB_E_ARG;
    const int nblocks = (data_length + kSumBins - 1) / kSumBins;
    dim3 grid(nblocks, num_bin_all < 65535 ? num_bin_all : 65535, nchannels < 65535 ? nchannels : 65535);
    k_fd_lnl<<<grid, kSumThreads, 0, stream>>>((double2 *)temp_sum, (const double2 *)hp_fd, (const double2 *)hc_fd,
                                               (const double2 *)data, psd, Fplus, Fcross, time_shift, df, num_bin_all,
                                               nchannels, data_length);
    return ret(cudaGetLastError());
}

}  // extern "C"
