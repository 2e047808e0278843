// Frequency-domain likelihood of the waveform path (BBHWaveformTD.get_ll,
// eob/seobnrv4phm.py:772-823): detector response and the PSD-weighted
// residual, on the complex FFT of each binary's summed strain.
//
// The reference takes two real FFTs, of the plus (real) and cross
// (imaginary) parts of the strain (:736-744), projects them onto every
// detector with the antenna patterns and the geocenter time delay (:597-634)
// and reduces |d - h|^2 / S_n per 1024-bin block (src/interpolate.cu:551-627).
// Here one complex FFT H = FFT(h_+ + i h_x) per binary (a library FFT) replaces
// the two real ones, and one kernel per (block of bins, binary) splits
//   h~_+(f) = (H(f) + conj H(N - f)) / 2,  h~_x(f) = (H(f) - conj H(N - f)) / 2i
// on the fly -- the bins f < N/2 + 1 read H(f) from the lower half and
// H(N - f) from the mirrored block of the upper half, so every element of H
// is read once and h~_+, h~_x are never written -- then projects onto every
// detector and accumulates the residual.  The PSD enters as its reciprocal,
// formed once per call (a division costs about six FP64 issue slots on GB300,
// a product one).  A last kernel sums each binary's block partials in a fixed
// order (deterministic, no atomics).
#include "eob_device.cuh"

namespace {

constexpr int kFdThreads = 256;
constexpr int kFdPerThread = 16;                      // bins per thread, kFdThreads apart
constexpr int kFdBins = kFdThreads * kFdPerThread;    // frequency bins per block
constexpr int kFdMaxChannels = 8;
constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kSpeedOfLight = 299792458.0;  // m/s

// GPS - UTC in seconds: the GPS times at which each leap second took effect
// (1981-07-01 ... 2017-01-01 UTC); the count is the number of entries <= t.
__constant__ double c_leap_gps[18] = {46828801.0,  78364802.0,  109900803.0, 173059204.0,  252028805.0,  315187206.0,
                                      346723207.0, 393984008.0, 425520009.0, 457056010.0,  504489611.0,  551750412.0,
                                      599184013.0, 820108814.0, 914803215.0, 1025136016.0, 1119744017.0, 1167264018.0};

// Greenwich mean sidereal time [rad, in [0, 2 pi)] at a GPS time: the IAU 1982
// expression (Aoki et al. 1982, A&A 105, 359), GMST = 67310.54841 s +
// (876600 h + 8640184.812866 s) T + 0.093104 s T^2 - 6.2e-6 s T^3 with T the
// Julian centuries of UT1 since J2000.0, taking UT1 = UTC.
__device__ double gmst_from_gps(double gps)
{
    int leap = 0;
    for (int i = 0; i < 18; ++i) leap += (gps >= c_leap_gps[i]) ? 1 : 0;
    // days since J2000.0 (JD 2451545.0); the GPS epoch is JD 2444244.5 UTC
    const double days = (gps - (double)leap) / 86400.0 - (2451545.0 - 2444244.5);
    const double T = days / 36525.0;
    double s = 67310.54841 + T * ((876600.0 * 3600.0 + 8640184.812866) + T * (0.093104 - 6.2e-6 * T));
    s = fmod(s, 86400.0);
    if (s < 0.0) s += 86400.0;
    return s * (kTwoPi / 86400.0);
}

// F+, Fx and the delay from the geocenter for each (detector, binary):
// phi = ra - gmst, theta = pi/2 - dec; the wave frame m, n from the
// polarisation angle; F = D : e with e+ = m m - n n, ex = m n + n m; delay =
// (direction of the source) . (detector vertex) / c.
__global__ void k_detector_response(const double *ra, const double *dec, const double *psi, const double *gps,
                                    const double *tensors, const double *vertices, int B, int nch, double *Fplus,
                                    double *Fcross, double *tshift)
{
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        const double gmst = gmst_from_gps(gps[b]);
        const double ph = ra[b] - gmst, th = 0.5 * eob::kPi - dec[b];
        double sph, cph, sth, cth, sps, cps;
        sincos(ph, &sph, &cph);
        sincos(th, &sth, &cth);
        sincos(psi[b], &sps, &cps);
        const double u[3] = {cph * cth, cth * sph, -sth};
        const double v[3] = {-sph, cph, 0.0};
        double m[3], n[3];
        for (int i = 0; i < 3; ++i) {
            m[i] = -u[i] * sps - v[i] * cps;
            n[i] = -u[i] * cps + v[i] * sps;
        }
        const double w[3] = {sth * cph, sth * sph, cth};
        for (int c = 0; c < nch; ++c) {
            const double *D = tensors + 9 * (size_t)c;
            double fp = 0.0, fx = 0.0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    fp += D[3 * i + j] * (m[i] * m[j] - n[i] * n[j]);
                    fx += D[3 * i + j] * (m[i] * n[j] + n[i] * m[j]);
                }
            const double *V = vertices + 3 * (size_t)c;
            Fplus[(size_t)c * B + b] = fp;
            Fcross[(size_t)c * B + b] = fx;
            tshift[(size_t)c * B + b] = (w[0] * V[0] + w[1] * V[1] + w[2] * V[2]) / kSpeedOfLight;
        }
    }
}

// 1 / S_n for every (detector, bin)
__global__ void k_fd_inv_psd(const double *psd, long long n, double *ipsd)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        ipsd[i] = 1.0 / psd[i];
}

// One block of kFdBins bins (f = df i, i < Nf = N / 2 + 1) of one binary:
// sum over the NCH detectors of |d - (F+ h~_+ + Fx h~_x) e^{-2 pi i f tau}|^2
// / S_n, h~ zero below start_ind.  partial[blockIdx.x * B + b].  Each thread
// takes kFdPerThread bins kFdThreads apart; the delay phase comes from one
// sincos at its first bin and one for the step, then rotations (a sincos
// costs tens of FP64 instructions).  NCH is a template argument so that the
// per-detector values stay in registers.
template <int NCH>
__global__ void __launch_bounds__(kFdThreads) k_fd_split_lnl(const double2 *H, int N, int start_ind,
                                                             const double2 *data, const double *ipsd,
                                                             const double *Fplus, const double *Fcross,
                                                             const double *tshift, double df, int B, double *partial)
{
    __shared__ double warp_sum[kFdThreads / 32];
    const int Nf = N / 2 + 1;
    for (int b = blockIdx.y; b < B; b += gridDim.y) {
        const double2 *Hb = H + (size_t)b * N;
        double fp[NCH], fx[NCH], s[NCH], co[NCH], sd[NCH], cd[NCH];
        const int i0 = blockIdx.x * kFdBins + threadIdx.x;
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
            fp[c] = Fplus[(size_t)c * B + b];
            fx[c] = Fcross[(size_t)c * B + b];
            const double tau = tshift[(size_t)c * B + b];
            sincos(kTwoPi * (df * i0) * tau, &s[c], &co[c]);
            sincos(kTwoPi * (df * kFdThreads) * tau, &sd[c], &cd[c]);
        }
        double acc = 0.0;
#pragma unroll 4
        for (int q = 0; q < kFdPerThread; ++q) {
            const int i = i0 + q * kFdThreads;
            if (q > 0) {
#pragma unroll
                for (int c = 0; c < NCH; ++c) {
                    const double cn = fma(co[c], cd[c], -s[c] * sd[c]);
                    s[c] = fma(s[c], cd[c], co[c] * sd[c]);
                    co[c] = cn;
                }
            }
            if (i < Nf) {
                double pr = 0.0, pi = 0.0, xr = 0.0, xi = 0.0;
                if (i >= start_ind) {
                    const double2 a = Hb[i];
                    const double2 z = Hb[i == 0 ? 0 : N - i];
                    // h~_+ = (a + conj z) / 2, h~_x = (a - conj z) / 2i
                    pr = 0.5 * (a.x + z.x);
                    pi = 0.5 * (a.y - z.y);
                    xr = 0.5 * (a.y + z.y);
                    xi = -0.5 * (a.x - z.x);
                }
#pragma unroll
                for (int c = 0; c < NCH; ++c) {
                    const double gr = fma(fp[c], pr, fx[c] * xr), gi = fma(fp[c], pi, fx[c] * xi);
                    const double2 d = data[(size_t)c * Nf + i];
                    const double rr = d.x - fma(gr, co[c], gi * s[c]);
                    const double ri = d.y - fma(gi, co[c], -gr * s[c]);
                    acc = fma(fma(rr, rr, ri * ri), ipsd[(size_t)c * Nf + i], acc);
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < kFdThreads / 32; ++w) t += warp_sum[w];
            partial[(size_t)blockIdx.x * B + b] = t;
        }
        __syncthreads();
    }
}

// lnL[b] = -1/2 4 df sum over blocks (in block order)
__global__ void k_fd_finalize(const double *partial, int nblk, int B, double df, double *lnl)
{
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x) {
        double t = 0.0;
        for (int q = 0; q < nblk; ++q) t += partial[(size_t)q * B + b];
        lnl[b] = -0.5 * df * 4.0 * t;
    }
}

int blocks_for(long long n, int bs)
{
    long long g = (n + bs - 1) / bs;
    return (int)(g < 1 ? 1 : (g > 65535 ? 65535 : g));
}

}  // namespace

extern "C" {

int eob_detector_response(const double *ra, const double *dec, const double *psi, const double *geocent_time,
                          const double *detector_tensors, const double *vertices, int B, int nch, double *Fplus,
                          double *Fcross, double *time_shift, cudaStream_t stream)
{
    if (B < 0 || nch < 0) return EOB_E_ARG;
    if (B == 0 || nch == 0) return EOB_OK;
    if (!ra || !dec || !psi || !geocent_time || !detector_tensors || !vertices || !Fplus || !Fcross || !time_shift)
        return EOB_E_ARG;
    k_detector_response<<<blocks_for(B, 128), 128, 0, stream>>>(ra, dec, psi, geocent_time, detector_tensors,
                                                                 vertices, B, nch, Fplus, Fcross, time_shift);
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

// block partials of every binary, then 1 / S_n for up to kFdMaxChannels
// detectors (256-byte aligned)
size_t eob_fd_lnl_scratch_bytes(int B, int N)
{
    if (B < 1 || N < 2) return 0;
    const long long nblk = ((long long)(N / 2 + 1) + kFdBins - 1) / kFdBins;
    const size_t part = ((size_t)(nblk * B) * sizeof(double) + 255) & ~(size_t)255;
    return part + (size_t)kFdMaxChannels * (size_t)(N / 2 + 1) * sizeof(double);
}

int eob_fd_lnl_from_fft(const double *H, int N, int start_ind, const double *data, const double *psd,
                        const double *Fplus, const double *Fcross, const double *time_shift, double df, int B, int nch,
                        void *scratch, size_t scratch_bytes, double *lnl, cudaStream_t stream)
{
    if (B < 1 || N < 2 || (N & 1) || nch < 1 || nch > kFdMaxChannels || start_ind < 0) return EOB_E_ARG;
    if (!H || !data || !psd || !Fplus || !Fcross || !time_shift || !scratch || !lnl) return EOB_E_ARG;
    if (scratch_bytes < eob_fd_lnl_scratch_bytes(B, N)) return EOB_E_ARG;
    const int nblk = (N / 2 + 1 + kFdBins - 1) / kFdBins;
    double *partial = (double *)scratch;
    const size_t part = ((size_t)nblk * (size_t)B * sizeof(double) + 255) & ~(size_t)255;
    double *ipsd = (double *)((char *)scratch + part);
    const long long npsd = (long long)nch * (N / 2 + 1);
    k_fd_inv_psd<<<blocks_for(npsd, 256), 256, 0, stream>>>(psd, npsd, ipsd);
    if (cudaGetLastError() != cudaSuccess) return EOB_E_CUDA;
    dim3 grid(nblk, B < 65535 ? B : 65535);
    const double2 *H2 = (const double2 *)H, *d2 = (const double2 *)data;
#define EOB_FD_LAUNCH(K)                                                                                         \
    case K:                                                                                                      \
        k_fd_split_lnl<K><<<grid, kFdThreads, 0, stream>>>(H2, N, start_ind, d2, ipsd, Fplus, Fcross, time_shift, \
                                                           df, B, partial);                                      \
        break;
    switch (nch) {
        EOB_FD_LAUNCH(1) EOB_FD_LAUNCH(2) EOB_FD_LAUNCH(3) EOB_FD_LAUNCH(4)
        EOB_FD_LAUNCH(5) EOB_FD_LAUNCH(6) EOB_FD_LAUNCH(7) EOB_FD_LAUNCH(8)
    }
#undef EOB_FD_LAUNCH
    if (cudaGetLastError() != cudaSuccess) return EOB_E_CUDA;
    k_fd_finalize<<<blocks_for(B, 128), 128, 0, stream>>>(partial, nblk, B, df, lnl);
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

}  // extern "C"
