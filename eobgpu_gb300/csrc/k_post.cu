// After the integrator: packing, multipoles on the trajectory, batched
// not-a-knot splines, and the fused synthesis + likelihood pass.
//
//  k_scan_*    one block: per-binary row counts and waveform sample counts,
//              exclusive scans (packed ragged layout), sum of data^2.
//  k_modes     one thread per packed trajectory row: h_lm e^{i m phi} for the
//              requested modes (get_hlms, eob/seobnrv4phm.py:2138-2221, and
//              the de-rotation of compute_full_waveform, :2331).
//  k_spline    one warp per (binary, series): not-a-knot cubic spline with
//              the reference's tridiagonal set-up (src/interpolate.cu:10-267),
//              solved by a partition method (a block of rows per lane, the
//              block boundaries by lane 0) instead of one serial sweep.
//  k_synth     one block per 1024-sample chunk of one binary: spline
//              evaluation on the uniform grid (eob/seobnrv4phm.py:274-386,
//              2310-2372), mode sum (BBHWaveformTD, :715-721) and the
//              white-noise residual, reduced to one partial per chunk; in
//              likelihood mode the strain is never written to memory.
//  k_finalize  per binary, partials summed in a fixed order (deterministic).
#include "eob_device.cuh"

namespace eob {

constexpr int kScanThreads = 1024;

__device__ __forceinline__ double t_in_of(double t_M, double Mt)
{
    // reference: t[s] = t_M * mt * MTSUN_SI, then t / (M * MTSUN_SI)
    return (t_M * Mt * kMTSUN_SI) / (Mt * kMTSUN_SI);
}

// number of uniform samples of binary b: int((t_end - t_0) / dT) + 1
__device__ int binary_npts(const double *tr, int L, double Mt, double dt)
{
    const double t0 = t_in_of(tr[0], Mt);
    const double t1 = t_in_of(tr[(size_t)(L - 1) * kTrajStride], Mt);
    const double dT = dt / (Mt * kMTSUN_SI);
    return (int)((t1 - t0) / dT) + 1;
}

// block-wide exclusive scan helper: returns the exclusive prefix of v over the block
template <int NT>
__device__ long long block_exclusive_scan(long long v, long long *sm, long long *total)
{
    const int tid = threadIdx.x;
    sm[tid] = v;
    __syncthreads();
    for (int off = 1; off < NT; off <<= 1) {
        const long long add = (tid >= off) ? sm[tid - off] : 0;
        __syncthreads();
        sm[tid] += add;
        __syncthreads();
    }
    const long long incl = sm[tid];
    if (total) *total = sm[NT - 1];
    __syncthreads();
    return incl - v;
}

// rows and uniform-grid sample counts per binary; packed row offsets
__global__ void __launch_bounds__(kScanThreads) k_scan_rows(Ws w, int B, double dt)
{
    __shared__ long long sm[kScanThreads];
    const int tid = threadIdx.x;
    const int per = (B + kScanThreads - 1) / kScanThreads;
    const int b0 = tid * per;
    const int b1 = min(B, b0 + per);
    long long rows = 0;
    for (int b = b0; b < b1; ++b) {
        const int L = w.nsteps[b];
        int st = w.status[b];
        int np = 0;
        if (L >= 3 && !(st & (EOB_ST_NAN | EOB_ST_TRIES | EOB_ST_SHORT))) {
            np = binary_npts(w.traj + (size_t)b * w.L.Lc * kTrajStride, L, w.bins[b].Mt, dt);
            if (np < 1) np = 0;
        } else {
            st |= EOB_ST_SHORT;
            w.status[b] = st;
        }
        w.npts[b] = np;
        rows += (np > 0) ? L : 0;
    }
    long long total;
    long long ro = block_exclusive_scan<kScanThreads>(rows, sm, &total);
    for (int b = b0; b < b1; ++b) {
        w.row_off[b] = ro;
        ro += (w.npts[b] > 0) ? w.nsteps[b] : 0;
    }
    if (tid == 0) {
        w.row_off[B] = total;
        w.queue[1] = (unsigned long long)total;
    }
}

// synthesis work items: chunks of kChunk samples of min(npts, N) samples per
// binary (all N samples when cover_all); sum of data^2
__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(Ws w, int B, int N, int cover_all, const double *data,
                                                               int mixed)
{
    __shared__ long long sm[kScanThreads];
    __shared__ double s_sq[kScanThreads];
    const int tid = threadIdx.x;
    const int per = (B + kScanThreads - 1) / kScanThreads;
    const int b0 = tid * per;
    const int b1 = min(B, b0 + per);
    long long chunks = 0;
    for (int b = b0; b < b1; ++b) {
        const int np = w.npts[b];
        const int nuse = (np <= 0) ? 0 : (cover_all ? N : (np < N ? np : N));
        chunks += (nuse + kChunk - 1) / kChunk;
    }
    double sq = 0.0;
    if (data)
        for (int k = tid; k < N; k += kScanThreads) {
            sq += data[k] * data[k];
            if (mixed) w.dataf[k] = (float)data[k];
        }
    s_sq[tid] = sq;
    long long total;
    long long co = block_exclusive_scan<kScanThreads>(chunks, sm, &total);
    for (int b = b0; b < b1; ++b) {
        w.chunk_off[b] = co;
        const int np = w.npts[b];
        const int nuse = (np <= 0) ? 0 : (cover_all ? N : (np < N ? np : N));
        co += (nuse + kChunk - 1) / kChunk;
    }
    for (int off = kScanThreads / 2; off > 0; off >>= 1) {
        if (tid < off) s_sq[tid] += s_sq[tid + off];
        __syncthreads();
    }
    if (tid == 0) {
        w.chunk_off[B] = total;
        w.queue[2] = (unsigned long long)total;
        w.queue[3] = (unsigned long long)__double_as_longlong(s_sq[0]);
    }
}

// index b with off[b] <= v < off[b+1]
__device__ __forceinline__ int find_segment(const long long *off, int B, long long v)
{
    int lo = 0, hi = B;  // answer in [lo, hi)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= v) lo = mid; else hi = mid;
    }
    return lo;
}

struct ModeArgs {
    int K;
    int ells[kMaxModes], mms[kMaxModes];
    int imr;  // also r and p_r as series for the merger-ringdown attachment
};

__global__ void __launch_bounds__(128) k_modes(Ws w, int B, ModeArgs ma)
{
    const long long R = (long long)w.queue[1];
    const size_t Rc = (size_t)w.L.Bc * (size_t)w.L.Lc;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < R; r += (long long)gridDim.x * blockDim.x) {
        const int b = find_segment(w.row_off, B, r);
        const int i = (int)(r - w.row_off[b]);
        const BinaryRec &rec = w.bins[b];
        const double *row = w.traj + ((size_t)b * w.L.Lc + i) * kTrajStride;
        const double rr = row[1], phi = row[2], pr = row[3], pphi = row[4];
        w.tin[r] = t_in_of(row[0], rec.Mt);
        w.ys[r] = phi;
        if (ma.imr) {
            w.imr_ys[r] = rr;
            w.imr_ys[Rc + r] = pr;
        }
        HamEval e;
        ham_eval(rec.ham, rr, pr, pphi, &e);
        const double v = cbrt(e.dHdL);
        const double vphi_in = 1.0 / (e.omega_c * e.omega_c * rr * rr * rr);
        for (int j = 0; j < ma.K; ++j) {
            const int l = ma.ells[j], m = ma.mms[j];
            const int li = lm_index(l, m);
            const cdbl hl = mode_eval(w.fac[b], l, m, rec.pre_re[li], rec.pre_im[li], rec.nu, rr, phi, pphi, v,
                                      e.Hreal, vphi_in, 0.0, true);
            w.ys[(size_t)(1 + 2 * j) * Rc + r] = hl.re;
            w.ys[(size_t)(2 + 2 * j) * Rc + r] = hl.im;
        }
    }
}

// Row i of the not-a-knot slope system (src/interpolate.cu:10-120):
// a x_{i-1} + b x_i + c x_{i+1} = d.
__device__ __forceinline__ void spline_row(const double *x, const double *y, int n, int i, double *a, double *b,
                                           double *c, double *d)
{
    int i0, i1, i2;
    if (i == n - 1) { i0 = n - 3; i1 = n - 2; i2 = n - 1; }
    else if (i == 0) { i0 = 0; i1 = 1; i2 = 2; }
    else { i0 = i - 1; i1 = i; i2 = i + 1; }
    const double x0 = x[i0], x1 = x[i1], x2 = x[i2];
    const double dx1 = x1 - x0, dx2 = x2 - x1, dd = x2 - x0;
    const double y1 = y[i1];
    const double s1 = (y1 - y[i0]) / dx1, s2 = (y[i2] - y1) / dx2;
    if (i == n - 1) {
        *d = (dx2 * dx2 * s1 + (2 * dd + dx2) * dx1 * s2) / dd;
        *b = dx1; *a = dd; *c = 0.0;
    } else if (i == 0) {
        *d = ((dx1 + 2 * dd) * dx2 * s1 + dx1 * dx1 * s2) / dd;
        *c = dd; *a = 0.0; *b = dx2;
    } else {
        *d = 3.0 * (dx2 * s1 + dx1 * s2);
        *b = 2 * (dx1 + dx2); *c = dx1; *a = dx2;
    }
}

constexpr int kSplineRowsPerLane = 8;  // partition the system only when every lane gets this many rows
constexpr int kSplineMaxTile = 8;      // series (warps) per block

// One warp per series (binary, sub).  The tridiagonal slope system is solved
// by a partition method: lane k owns a contiguous block of rows, eliminates it
// with three right-hand sides (the data and the two couplings to the
// neighbouring blocks), lane 0 solves the 2x2-block tridiagonal system of the
// block boundaries (gathered by shuffles), and every lane back-substitutes
// its rows; the cubic coefficients are then computed lane-strided.  Scratch:
// the series' own coefficient rows (ld/dg/ud/Bv = c3/c2/c1/rhs arrays).
__global__ void __launch_bounds__(32 * kSplineMaxTile) k_spline(Ws w, int B, int nsubs, int nmain, int mixed)
{
    __shared__ double s_z[kSplineMaxTile][2][32];   // boundary solution: u_j = x_{e_j}, t_{j+1} = x_{s_{j+1}}
    __shared__ double s_f[kSplineMaxTile][5][32];   // reduced elimination per interface: d01, d10, f0, f1, ws_{j+1}
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * (blockDim.x >> 5) + wib;  // uniform across the warp
    if (blockIdx.x == 0 && threadIdx.x == 0) w.queue[6] = (unsigned long long)mixed;
    if (idx >= B * nsubs) return;
    const int b = idx / nsubs, sub = idx % nsubs;
    if (w.npts[b] <= 0) return;
    const int n = w.nsteps[b];
    const size_t Rc = (size_t)w.L.Bc * (size_t)w.L.Lc;
    const size_t base = (size_t)w.row_off[b];
    // series 0 .. nmain - 1: phase and modes; nmain, nmain + 1: r and p_r of the
    // merger-ringdown section
    const bool extra = sub >= nmain;
    const size_t o = (size_t)(extra ? sub - nmain : sub) * Rc + base;
    const double *x = w.tin + base, *y = (extra ? w.imr_ys : w.ys) + o;
    double *Bv = (extra ? w.imr_cD : w.cD) + o, *ud = (extra ? w.imr_cA : w.cA) + o,
           *dg = (extra ? w.imr_cB : w.cB) + o, *ld = (extra ? w.imr_cC : w.cC) + o;

    for (int i = lane; i < n; i += 32) spline_row(x, y, n, i, &ld[i], &dg[i], &ud[i], &Bv[i]);
    __syncwarp();

    int P = n / kSplineRowsPerLane;
    if (P > 32) P = 32;
    if (P < 2) {
        if (lane == 0) {  // short series: one Thomas sweep
            for (int i = 1; i < n; ++i) {
                const double wgt = ld[i] / dg[i - 1];
                dg[i] = dg[i] - wgt * ud[i - 1];
                Bv[i] = Bv[i] - wgt * Bv[i - 1];
            }
            Bv[n - 1] = Bv[n - 1] / dg[n - 1];
            for (int i = n - 2; i >= 0; --i) Bv[i] = (Bv[i] - ud[i] * Bv[i + 1]) / dg[i];
        }
    } else {
        const int q = n / P, r = n % P;
        const bool own = lane < P;
        const int s0 = lane * q + min(lane, r);
        const int e0 = s0 + q + (lane < r ? 1 : 0) - 1;
        double gs = 0.0, vs = 0.0, ws = 0.0, ge = 0.0, ve = 0.0, we = 0.0;
        if (own) {
            // forward elimination; dg <- 1/b', Bv <- d', ld <- v' (v' starts as a_s e_1)
            double ib = 1.0 / dg[s0], dp = Bv[s0], vp = ld[s0];
            dg[s0] = ib;
            ld[s0] = vp;
            for (int i = s0 + 1; i <= e0; ++i) {
                const double wgt = ld[i] * ib;
                ib = 1.0 / (dg[i] - wgt * ud[i - 1]);
                dp = Bv[i] - wgt * dp;
                vp = -wgt * vp;
                dg[i] = ib;
                Bv[i] = dp;
                ld[i] = vp;
            }
            // back substitution of g (data), v (left coupling), w (right coupling, c_e at row e only)
            double gx = dp * ib, vx = vp * ib, wx = ud[e0] * ib;
            Bv[e0] = gx;
            ld[e0] = vx;
            dg[e0] = wx;
            ge = gx;
            ve = vx;
            we = wx;
            for (int i = e0 - 1; i >= s0; --i) {
                const double ibi = dg[i], ci = ud[i];
                gx = (Bv[i] - ci * gx) * ibi;
                vx = (ld[i] - ci * vx) * ibi;
                wx = -ci * wx * ibi;
                Bv[i] = gx;
                ld[i] = vx;
                dg[i] = wx;
            }
            gs = gx;
            vs = vx;
            ws = wx;
        }
        // reduced system over the P-1 block interfaces j (between blocks j, j+1),
        // unknowns Z_j = (u_j, t_{j+1}) = (x at the end of block j, x at the start of block j+1):
        //   u_j + ve_j u_{j-1} + we_j t_{j+1} = ge_j
        //   vs_{j+1} u_j + t_{j+1} + ws_{j+1} t_{j+2} = gs_{j+1}
        // a 2x2-block tridiagonal system, eliminated by lane 0 (gathers by shuffles)
        double k00 = 0.0, k01 = 0.0, f0 = 0.0, f1 = 0.0;
        for (int j = 0; j < P - 1; ++j) {
            const double vej = __shfl_sync(0xffffffffu, ve, j), wej = __shfl_sync(0xffffffffu, we, j);
            const double gej = __shfl_sync(0xffffffffu, ge, j), wsj = __shfl_sync(0xffffffffu, ws, j);
            const double vsn = __shfl_sync(0xffffffffu, vs, j + 1), wsn = __shfl_sync(0xffffffffu, ws, j + 1);
            const double gsn = __shfl_sync(0xffffffffu, gs, j + 1);
            if (lane == 0) {
                double d01 = wej, h0 = gej;
                if (j > 0) {
                    d01 -= vej * k01 * wsj;
                    h0 -= vej * (k00 * f0 + k01 * f1);
                }
                const double idet = 1.0 / (1.0 - d01 * vsn);
                k00 = idet;
                k01 = -d01 * idet;
                f0 = h0;
                f1 = gsn;
                s_f[wib][0][j] = d01;
                s_f[wib][1][j] = vsn;
                s_f[wib][2][j] = h0;
                s_f[wib][3][j] = gsn;
                s_f[wib][4][j] = wsn;
            }
        }
        if (lane == 0) {
            double tn = 0.0;  // t_{j+2} of the interface after j
            for (int j = P - 2; j >= 0; --j) {
                const double d01 = s_f[wib][0][j], d10 = s_f[wib][1][j];
                const double h0 = s_f[wib][2][j];
                const double h1 = s_f[wib][3][j] - s_f[wib][4][j] * tn;
                const double idet = 1.0 / (1.0 - d01 * d10);
                const double uj = (h0 - d01 * h1) * idet;
                const double tj = (h1 - d10 * h0) * idet;
                s_z[wib][0][j] = uj;
                s_z[wib][1][j] = tj;
                tn = tj;
            }
        }
        __syncwarp();
        if (own) {
            const double L = (lane > 0) ? s_z[wib][0][lane - 1] : 0.0;
            const double R = (lane < P - 1) ? s_z[wib][1][lane] : 0.0;
            for (int i = s0; i <= e0; ++i) Bv[i] = Bv[i] - ld[i] * L - dg[i] * R;
        }
    }
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
        if (i == n - 1) {
            ud[i] = 0.0;
            dg[i] = 0.0;
            ld[i] = 0.0;
            continue;
        }
        const double dx = x[i + 1] - x[i];
        const double slope = (y[i + 1] - y[i]) / dx;
        const double bi = Bv[i];
        const double t = (bi + Bv[i + 1] - 2 * slope) / dx;
        ud[i] = bi;
        dg[i] = (slope - bi) / dx - t;
        ld[i] = t / dx;
    }
    if (mixed && sub >= 1 && sub < nmain) {
        __syncwarp();
        // FP32 copies of the amplitude series for the mixed-precision synthesis
        const size_t S = (size_t)2 * w.L.Kc * Rc;
        float *f = w.f32 + (size_t)(sub - 1) * Rc + base;
        for (int i = lane; i < n; i += 32) {
            f[i] = (float)y[i];
            f[S + i] = (float)ud[i];
            f[2 * S + i] = (float)dg[i];
            f[3 * S + i] = (float)ld[i];
        }
    }
}

struct SynthArgs {
    int B, N, K;
    int mms[kMaxModes];
    double dt, amp;
    const double *data;   // lnL mode
    double *out;          // strain modes
    int mode;             // 0: lnL, 1: summed strain (zero past the end), 2: per mode, t clamped to the end
};

// interval i with x[i] <= t < x[i+1] (searchsorted right - 1), t, x >= 0:
// integer comparison of the IEEE bit patterns keeps the FP64 pipe free.
__device__ __forceinline__ int knot_index(const double *x, int n, double t)
{
    const long long tb = __double_as_longlong(t);
    int lo = 0, hi = n;  // first index with x > t lies in [lo, hi]
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__double_as_longlong(x[mid]) <= tb) lo = mid + 1; else hi = mid;
    }
    int i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 1) i = n - 1;
    return i;
}

// the merger-ringdown of one mode x = t - t_match after the match point
// (compute_MR_mode_free, eob/seobnrv4phm.py:1830-1843)
__device__ __forceinline__ void ringdown_mode(const ImrRec &c, double x, double *hr, double *hi)
{
    const double A = c.c1c * tanh(c.c1f * x + c.c2f) + c.c2c;
    const double ph = c.phi_match - c.d1c * log((1 + c.d2f * exp(-c.d1f * x)) / (1 + c.d2f)) - c.om_re * x;
    const double mag = c.eta * A * exp(-c.om_im * x);
    double sp, cp;
    sincos(ph, &sp, &cp);
    *hr = mag * cp;
    *hi = mag * sp;
}

__global__ void __launch_bounds__(256) k_synth(Ws w, SynthArgs sa)
{
    __shared__ double s_red[256 / 32];
    const long long C = (long long)w.queue[2];
    const size_t Rc = (size_t)w.L.Bc * (size_t)w.L.Lc;
    for (long long c = blockIdx.x; c < C; c += gridDim.x) {
        const int b = find_segment(w.chunk_off, sa.B, c);
        const int j = (int)(c - w.chunk_off[b]);
        const int np = w.npts[b];
        // with the merger-ringdown: samples 0 .. idx are the NQC-corrected
        // inspiral, idx + 1 .. np - 1 the ringdown, zero beyond (per mode too)
        const bool imr = w.imr_bin && w.imr_bin[b].on;
        const int idx = imr ? w.imr_bin[b].idx : np;
        const int nuse = (sa.mode == 2) ? sa.N : (np < sa.N ? np : sa.N);
        const int n = w.nsteps[b];
        const size_t base = (size_t)w.row_off[b];
        const double *x = w.tin + base;
        const double Mts = w.bins[b].Mt * kMTSUN_SI;
        const double dT = sa.dt / Mts;
        const double t0 = x[0], tend = x[n - 1];
        const ImrRec *recs = imr ? w.imr_rec + (size_t)b * w.L.Kc : nullptr;
        double acc = 0.0;
        const int kbeg = j * kChunk;
        const int kend = min(nuse, kbeg + kChunk);
        for (int k = kbeg + threadIdx.x; k < kend; k += blockDim.x) {
            double hsum = 0.0, hsum_i = 0.0;
            if (imr && k > idx) {
                if (k < np) {
                    const double xr = (k - idx) * dT;
                    for (int q = 0; q < sa.K; ++q) {
                        double hr, hi;
                        ringdown_mode(recs[q], xr, &hr, &hi);
                        if (sa.mode == 2) {
                            const size_t oo = 2 * (((size_t)b * sa.K + q) * (size_t)sa.N + k);
                            sa.out[oo] = hr;
                            sa.out[oo + 1] = hi;
                        }
                        hsum += hr;
                        hsum_i += hi;
                    }
                } else if (sa.mode == 2) {
                    for (int q = 0; q < sa.K; ++q) {
                        const size_t oo = 2 * (((size_t)b * sa.K + q) * (size_t)sa.N + k);
                        sa.out[oo] = 0.0;
                        sa.out[oo + 1] = 0.0;
                    }
                }
                if (sa.mode == 1) {
                    sa.out[2 * ((size_t)b * sa.N + k)] = hsum;
                    sa.out[2 * ((size_t)b * sa.N + k) + 1] = hsum_i;
                } else if (sa.mode == 0) {
                    const double hk = sa.amp * hsum;
                    acc += hk * hk - 2.0 * sa.data[k] * hk;
                }
                continue;
            }
            double t = k * dT + t0;
            if (t > tend) t = tend;
            const int i = knot_index(x, n, t);
            const double xx = t - x[i], x2 = xx * xx, x3 = x2 * xx;
            const size_t o = base + i;
            const double phi = w.ys[o] + w.cA[o] * xx + w.cB[o] * x2 + w.cC[o] * x3;
            double rr = 0.0, pr = 0.0, om = 0.0;
            if (imr) {
                om = w.cA[o] + 2 * w.cB[o] * xx + 3 * w.cC[o] * x2;
                rr = w.imr_ys[o] + w.imr_cA[o] * xx + w.imr_cB[o] * x2 + w.imr_cC[o] * x3;
                const size_t op = Rc + o;
                pr = w.imr_ys[op] + w.imr_cA[op] * xx + w.imr_cB[op] * x2 + w.imr_cC[op] * x3;
            }
            for (int q = 0; q < sa.K; ++q) {
                const size_t orr = (size_t)(1 + 2 * q) * Rc + o, oi = (size_t)(2 + 2 * q) * Rc + o;
                const double re = w.ys[orr] + w.cA[orr] * xx + w.cB[orr] * x2 + w.cC[orr] * x3;
                const double im = w.ys[oi] + w.cA[oi] * xx + w.cB[oi] * x2 + w.cC[oi] * x3;
                double sp, cp;
                sincos(sa.mms[q] * phi, &sp, &cp);
                // (re + i im) e^{-i m phi}
                double hr = re * cp + im * sp, hi = im * cp - re * sp;
                if (imr) {
                    // NQC correction (EOBNonQCCorrection, eob/seobnrv4phm.py:1686-1700)
                    const ImrRec &cq = recs[q];
                    const double sr = sqrt(rr), rO = rr * om;
                    const double mag = 1.0 + (pr * pr / (rO * rO)) * (cq.a1 + cq.a2 / rr + cq.a3 / (rr * sr));
                    const double nph = cq.b1 * pr / rO + pr * pr * pr / rO * cq.b2;
                    double ns, nc;
                    sincos(nph, &ns, &nc);
                    const double tr = mag * (hr * nc - hi * ns);
                    hi = mag * (hr * ns + hi * nc);
                    hr = tr;
                }
                if (sa.mode == 2) {
                    const size_t oo = 2 * (((size_t)b * sa.K + q) * (size_t)sa.N + k);
                    sa.out[oo] = hr;
                    sa.out[oo + 1] = hi;
                }
                hsum += hr;
                hsum_i += hi;
            }
            if (sa.mode == 1) {
                sa.out[2 * ((size_t)b * sa.N + k)] = hsum;
                sa.out[2 * ((size_t)b * sa.N + k) + 1] = hsum_i;
            } else if (sa.mode == 0) {
                const double hk = sa.amp * hsum;
                acc += hk * hk - 2.0 * sa.data[k] * hk;
            }
        }
        // block reduction (fixed order)
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0 && sa.mode == 0) {
            double s = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += s_red[q];
            w.partial[c] = s;
        }
        __syncthreads();
    }
}

// Mixed precision synthesis: the phase spline and its reduction mod 2 pi run
// in FP64; the amplitude splines (FP32 coefficient copies written at spline
// build), sin/cos and the residual run in FP32.  mode 0 accumulates the lnL
// terms with a Kahan-compensated FP32 sum per thread and FP64 chunk partials;
// mode 1 writes the summed strain (zero past each waveform's end).  The
// FP32 copies exist only if the spline build ran with precision 1 (workspace
// flag queue[6]); otherwise the lnL comes out NaN.
__global__ void __launch_bounds__(256) k_synth_mixed(Ws w, SynthArgs sa)
{
    __shared__ double s_red[256 / 32];
    const long long C = (long long)w.queue[2];
    const bool have_f32 = w.queue[6] == 1ull;
    const size_t Rc = (size_t)w.L.Bc * (size_t)w.L.Lc;
    const size_t S = (size_t)2 * w.L.Kc * Rc;
    const double two_pi_hi = 6.283185307179586232, two_pi_lo = 2.4492935982947064e-16;
    for (long long c = blockIdx.x; c < C; c += gridDim.x) {
        const int b = find_segment(w.chunk_off, sa.B, c);
        const int j = (int)(c - w.chunk_off[b]);
        const int np = w.npts[b];
        const int nuse = np < sa.N ? np : sa.N;
        // the merger-ringdown runs in the FP64 synthesis only
        const bool imr_bin = w.imr_bin && w.imr_bin[b].on;
        const int n = w.nsteps[b];
        const size_t base = (size_t)w.row_off[b];
        const double *x = w.tin + base;
        const double Mts = w.bins[b].Mt * kMTSUN_SI;
        const double dT = sa.dt / Mts;
        const double t0 = x[0], tend = x[n - 1];
        float acc = 0.0f, comp = 0.0f;
        const int kbeg = j * kChunk;
        const int kend = have_f32 ? min(nuse, kbeg + kChunk) : kbeg;
        for (int k = kbeg + threadIdx.x; k < kend; k += blockDim.x) {
            double t = k * dT + t0;
            if (t > tend) t = tend;
            const int i = knot_index(x, n, t);
            const double xx = t - x[i];
            const size_t o = base + i;
            const double phi = w.ys[o] + xx * (w.cA[o] + xx * (w.cB[o] + xx * w.cC[o]));
            const float xf = (float)xx;
            float h = 0.0f, hi = 0.0f;
            for (int q = 0; q < sa.K; ++q) {
                const size_t orr = (size_t)(2 * q) * Rc + o, oi = (size_t)(2 * q + 1) * Rc + o;
                const float re = w.f32[orr] + xf * (w.f32[S + orr] + xf * (w.f32[2 * S + orr] + xf * w.f32[3 * S + orr]));
                const float im = w.f32[oi] + xf * (w.f32[S + oi] + xf * (w.f32[2 * S + oi] + xf * w.f32[3 * S + oi]));
                const double ph = sa.mms[q] * phi;
                const double nn = rint(ph * 0.15915494309189533577);
                const double red = fma(-nn, two_pi_lo, fma(-nn, two_pi_hi, ph));
                float sp, cp;
                sincosf((float)red, &sp, &cp);
                // (re + i im) e^{-i m phi}
                h = fmaf(re, cp, fmaf(im, sp, h));
                hi = fmaf(im, cp, fmaf(-re, sp, hi));
            }
            if (sa.mode == 1) {
                sa.out[2 * ((size_t)b * sa.N + k)] = (double)h;
                sa.out[2 * ((size_t)b * sa.N + k) + 1] = (double)hi;
            } else {
                const float hk = (float)sa.amp * h;
                const float term = hk * (hk - 2.0f * w.dataf[k]);
                // Kahan summation
                const float yv = term - comp;
                const float tv = acc + yv;
                comp = (tv - acc) - yv;
                acc = tv;
            }
        }
        double dacc = (double)acc - (double)comp;
        for (int off = 16; off > 0; off >>= 1) dacc += __shfl_down_sync(0xffffffffu, dacc, off);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = dacc;
        __syncthreads();
        if (threadIdx.x == 0 && sa.mode == 0) {
            double sum = 0.0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) sum += s_red[q];
            w.partial[c] = (have_f32 && !imr_bin) ? sum : __longlong_as_double(0x7ff8000000000000ll);
        }
        __syncthreads();
    }
}

__global__ void k_finalize(Ws w, int B, double *lnl, int *status_out)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const double dsq = __longlong_as_double((long long)w.queue[3]);
    const int st = w.status[b];
    double s = 0.0;
    for (long long c = w.chunk_off[b]; c < w.chunk_off[b + 1]; ++c) s += w.partial[c];
    const bool bad = (w.npts[b] <= 0);
    if (lnl) lnl[b] = bad ? __longlong_as_double(0x7ff8000000000000LL) : -0.5 * (dsq + s);
    if (status_out) status_out[b] = st;
}

cudaError_t launch_prepare_post(const Ws &w, const RunArgs &a, cudaStream_t s)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    k_scan_rows<<<1, kScanThreads, 0, s>>>(w, a.B, a.dt);
    ModeArgs ma;
    ma.K = a.K;
    for (int j = 0; j < kMaxModes; ++j) { ma.ells[j] = a.ells[j]; ma.mms[j] = a.mms[j]; }
    ma.imr = (a.opt.imr && w.imr_ys) ? 1 : 0;
    k_modes<<<nsm * 8, 128, 0, s>>>(w, a.B, ma);
    const int nmain = 1 + 2 * a.K;
    const int nsubs = nmain + (ma.imr ? 2 : 0);
    const int tile = (a.opt.spline_tile >= 1 && a.opt.spline_tile <= kSplineMaxTile) ? a.opt.spline_tile : 4;
    const long long series = (long long)a.B * nsubs;
    k_spline<<<(unsigned)((series + tile - 1) / tile), 32 * tile, 0, s>>>(w, a.B, nsubs, nmain,
                                                                         a.opt.precision == 1 ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_synth(const Ws &w, const RunArgs &a, int mode, double *out, cudaStream_t s)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int mixed = (mode != 2 && a.opt.precision == 1 && !a.opt.imr) ? 1 : 0;
    k_scan_chunks<<<1, kScanThreads, 0, s>>>(w, a.B, a.N, mode == 2 ? 1 : 0, mode == 0 ? a.data : nullptr,
                                             mode == 0 ? mixed : 0);
    if (mode == 1) {
        cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * 2 * (size_t)a.B * a.N, s);
        if (e != cudaSuccess) return e;
    }
    SynthArgs sa;
    sa.B = a.B;
    sa.N = a.N;
    sa.K = a.K;
    for (int j = 0; j < kMaxModes; ++j) sa.mms[j] = a.mms[j];
    sa.dt = a.dt;
    sa.amp = a.amp;
    sa.data = a.data;
    sa.out = out;
    sa.mode = mode;
    if (mixed) k_synth_mixed<<<nsm * 8, 256, 0, s>>>(w, sa);
    else k_synth<<<nsm * 8, 256, 0, s>>>(w, sa);
    k_finalize<<<(a.B + 127) / 128, 128, 0, s>>>(w, a.B, mode == 0 ? a.lnl : nullptr, a.status_out);
    return cudaGetLastError();
}

}  // namespace eob
