// Merger-ringdown attachment of the waveform (SEOBNRv4PHM.compute_full_waveform,
// eob/seobnrv4phm.py:2374-2557), after the splines of the inspiral.
//
// One warp per (binary, mode).  On the uniform grid t_k = k dT + t0 of the
// binary's inspiral (k < npts):
//   t_peak     knot of the largest orbital frequency (the phase spline's slope)
//   attachment t_peak - Delta t_22 (NR fit); the (5,5) mode's NQC point 10 M earlier
//   NQC        samples idx - 7 .. npts - 1 around the mode's point: splines of
//              q_j |h|, p_j, |h| and the unwrapped phase, their values and
//              derivatives there, 3x3 and 2x2 solves against the NR fits
//              (EOBCalculateNQCCoefficientsV4_freeattach, :1465-1683)
//   ringdown   samples idx - (int(20 / dT) + 1) .. npts - 1 of the NQC-corrected
//              mode: amplitude, its slope, phase and frequency at the match
//              point, the free and constrained ansatz coefficients, the QNM of
//              the remnant (compute_MR_mode_free, :1779-1844)
// A second kernel commits per binary: the IMR length (the inspiral to the
// attachment sample, then 30 (2,2) damping times of ringdown) or, if a window
// fell outside the waveform or exceeded kImrWin samples, the inspiral alone
// with EOB_ST_IMR.  The windows live in the block's shared memory.
#include "eob_device.cuh"
#include "physics/imr_fits.h"

namespace eob {
namespace {

struct ImrArgs {
    int B, K;
    int ells[kMaxModes], mms[kMaxModes];
    double dt;
};

// interval i with x[i] <= t < x[i + 1] (searchsorted right - 1); t, x >= 0
__device__ __forceinline__ int knot_at(const double *x, int n, double t)
{
    const long long tb = __double_as_longlong(t);
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__double_as_longlong(x[mid]) <= tb) lo = mid + 1; else hi = mid;
    }
    int i = lo - 1;
    if (i < 0) i = 0;
    if (i > n - 1) i = n - 1;
    return i;
}

struct Grid {
    const double *x;  // knots [M]
    int n;            // knots
    size_t base;      // packed row offset
    double t0, tend, dT;
    int np;           // inspiral samples
};

__device__ __forceinline__ double grid_t(const Grid &g, int k)
{
    double t = k * g.dT + g.t0;
    return t > g.tend ? g.tend : t;
}

// first k in [0, np) minimising |t_k - target| (numpy's argmin)
__device__ int grid_nearest(const Grid &g, double target)
{
    double c = floor((target - g.t0) / g.dT);
    if (c < -2.0) c = -2.0;
    if (c > (double)g.np) c = (double)g.np;
    const int k0 = (int)c;
    int best = -1;
    double bd = 0.0;
    for (int k = k0 - 1; k <= k0 + 2; ++k) {
        if (k < 0 || k >= g.np) continue;
        const double d = fabs(grid_t(g, k) - target);
        if (best < 0 || d < bd) { best = k; bd = d; }
    }
    if (best < 0) best = (target < g.t0) ? 0 : g.np - 1;
    return best;
}

struct Sample {
    double hr, hi, r, pr, om;
};

// mode q of binary b, r, p_r and the orbital frequency at sample k
__device__ Sample eval_sample(const Ws &w, const Grid &g, int k, int q, int m)
{
    const size_t Rc = (size_t)w.L.Bc * (size_t)w.L.Lc;
    const double t = grid_t(g, k);
    const int i = knot_at(g.x, g.n, t);
    const double xx = t - g.x[i], x2 = xx * xx, x3 = x2 * xx;
    const size_t o = g.base + i;
    const double phi = w.ys[o] + w.cA[o] * xx + w.cB[o] * x2 + w.cC[o] * x3;
    Sample s;
    s.om = w.cA[o] + 2 * w.cB[o] * xx + 3 * w.cC[o] * x2;
    s.r = w.imr_ys[o] + w.imr_cA[o] * xx + w.imr_cB[o] * x2 + w.imr_cC[o] * x3;
    const size_t op = Rc + o;
    s.pr = w.imr_ys[op] + w.imr_cA[op] * xx + w.imr_cB[op] * x2 + w.imr_cC[op] * x3;
    const size_t orr = (size_t)(1 + 2 * q) * Rc + o, oi = (size_t)(2 + 2 * q) * Rc + o;
    const double re = w.ys[orr] + w.cA[orr] * xx + w.cB[orr] * x2 + w.cC[orr] * x3;
    const double im = w.ys[oi] + w.cA[oi] * xx + w.cB[oi] * x2 + w.cC[oi] * x3;
    double sp, cp;
    sincos(m * phi, &sp, &cp);
    s.hr = re * cp + im * sp;
    s.hi = im * cp - re * sp;
    return s;
}

// EOBNonQCCorrection (eob/seobnrv4phm.py:1686-1700): (mag, phase)
__device__ __forceinline__ void nqc_factor(const ImrRec &c, double r, double pr, double om, double *mag,
                                           double *phase)
{
    const double sr = sqrt(r);
    const double rO = r * om;
    *mag = 1.0 + (pr * pr / (rO * rO)) * (c.a1 + c.a2 / r + c.a3 / (r * sr));
    *phase = c.b1 * pr / rO + pr * pr * pr / rO * c.b2;
}

// row i of the not-a-knot slope system (src/interpolate.cu:10-120) on knots t, values y
__device__ __forceinline__ void nak_row(const double *t, const double *y, int n, int i, double *a, double *b,
                                        double *c, double *d)
{
    int i0, i1, i2;
    if (i == n - 1) { i0 = n - 3; i1 = n - 2; i2 = n - 1; }
    else if (i == 0) { i0 = 0; i1 = 1; i2 = 2; }
    else { i0 = i - 1; i1 = i; i2 = i + 1; }
    const double dx1 = t[i1] - t[i0], dx2 = t[i2] - t[i1], dd = t[i2] - t[i0];
    const double s1 = (y[i1] - y[i0]) / dx1, s2 = (y[i2] - y[i1]) / dx2;
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

// value, first and second derivative at te of the not-a-knot spline through
// (t, y)[0..n), evaluated as CubicSplineInterpolantTD: interval
// searchsorted(right) - 1, the last knot with its own degenerate row.
// dg, bb: scratch of n doubles (the forward sweep's diagonal and right-hand
// side, carried from row to row in registers and stored for the back
// substitution).
__device__ void window_spline(const double *t, const double *y, int n, double *dg, double *bb, double te,
                              double out[3])
{
    double a, b, c, d, cprev = 0.0, dgp = 0.0, bbp = 0.0;
    for (int i = 0; i < n; ++i) {
        nak_row(t, y, n, i, &a, &b, &c, &d);
        if (i == 0) {
            dgp = b;
            bbp = d;
        } else {
            const double wgt = a / dgp;
            dgp = b - wgt * cprev;
            bbp = d - wgt * bbp;
        }
        dg[i] = dgp;
        bb[i] = bbp;
        cprev = c;
    }
    // interval of te
    int j = 0;
    {
        int lo = 0, hi = n;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (t[mid] <= te) lo = mid + 1; else hi = mid;
        }
        j = lo - 1;
        if (j < 0) j = 0;
        if (j > n - 1) j = n - 1;
    }
    const double xx = te - t[j];
    double c1, c2, c3;
    if (j == n - 1) {
        nak_row(t, y, n, n - 1, &a, &b, &c, &d);
        c1 = 0.0;
        c2 = dg[n - 1];
        c3 = a;
    } else {
        // back substitution from the last row down to row j
        double bn = bb[n - 1] / dg[n - 1];
        double bj1 = bn, bj = bn;
        for (int i = n - 2; i >= j; --i) {
            nak_row(t, y, n, i, &a, &b, &c, &d);
            const double bi = (bb[i] - c * bj1) / dg[i];
            if (i > j) bj1 = bi;
            else bj = bi;
        }
        if (j == n - 2) bj1 = bn;
        const double dx = t[j + 1] - t[j];
        const double slope = (y[j + 1] - y[j]) / dx;
        const double tt = (bj + bj1 - 2 * slope) / dx;
        c1 = bj;
        c2 = (slope - bj) / dx - tt;
        c3 = tt / dx;
    }
    out[0] = y[j] + c1 * xx + c2 * xx * xx + c3 * xx * xx * xx;
    out[1] = c1 + 2 * c2 * xx + 3 * c3 * xx * xx;
    out[2] = 2 * c2 + 6 * c3 * xx;
}

// np.unwrap of angles a[0..n) in place (discontinuity pi) by one warp: each
// lane forms the corrections of its samples from the original values (corr:
// scratch of n doubles), then lane 0 accumulates them in order.  Adding a
// zero correction leaves the running sum's bits unchanged (it starts at +0
// and a sum of doubles is never -0 unless both terms are), so the result is
// that of the serial loop.
__device__ void unwrap_warp(double *a, double *corr, int n, int lane)
{
    const double pi = kPi, two_pi = 2.0 * kPi;
    for (int i = 1 + lane; i < n; i += 32) {
        const double dd = a[i] - a[i - 1];
        double dm = fmod(dd + pi, two_pi);
        if (dm < 0.0) dm += two_pi;
        dm -= pi;
        if (dm == -pi && dd > 0.0) dm = pi;
        corr[i] = (fabs(dd) >= pi) ? dm - dd : 0.0;
    }
    __syncwarp();
    if (lane == 0) {
        double cum = 0.0;
        for (int i = 1; i < n; ++i) {
            cum += corr[i];
            a[i] += cum;
        }
    }
    __syncwarp();
}

// A x = y for 3x3 / 2x2 by elimination with partial pivoting (LAPACK gesv's method)
template <int N>
__device__ void solve_small(double A[N][N], double y[N], double x[N])
{
    for (int c = 0; c < N; ++c) {
        int p = c;
        for (int r = c + 1; r < N; ++r)
            if (fabs(A[r][c]) > fabs(A[p][c])) p = r;
        if (p != c) {
            for (int k = 0; k < N; ++k) { const double t = A[c][k]; A[c][k] = A[p][k]; A[p][k] = t; }
            const double t = y[c]; y[c] = y[p]; y[p] = t;
        }
        for (int r = c + 1; r < N; ++r) {
            const double f = A[r][c] / A[c][c];
            for (int k = c; k < N; ++k) A[r][k] -= f * A[c][k];
            y[r] -= f * y[c];
        }
    }
    for (int r = N - 1; r >= 0; --r) {
        double s = y[r];
        for (int k = r + 1; k < N; ++k) s -= A[r][k] * x[k];
        x[r] = s / A[r][r];
    }
}

// Shared memory of one (binary, mode): the window's samples t, |h|, phase,
// r, p_r, omega (arrays 0..5), the series of the NQC columns q_1..q_3 |h|,
// p_1, p_2 (6..10) and the elimination scratch of the splines (11..21, then
// r, p_r and omega once the series exist): 22 arrays of kImrWin doubles.
constexpr int kImrArr = 22;
// scratch array k = 0..13 of the splines (lane s: diagonal 2 s, right-hand side 2 s + 1)
__device__ __forceinline__ int imr_scr_arr(int k) { return k < 11 ? 11 + k : k - 8; }

// One warp per (binary, mode): the lanes evaluate the window samples side by
// side, the seven NQC splines (three q columns, |h|, two p columns, the
// phase) run on lanes 0..6 and the two ringdown splines on lanes 0..1, each
// the same serial solve as before; the small solves and the fits are formed
// by every lane alike from shuffled values.
__global__ void __launch_bounds__(32) k_imr(Ws w, ImrArgs ia)
{
    __shared__ double sm[kImrArr * kImrWin];
    const int lane = threadIdx.x;
    const int item = blockIdx.x;  // b * K + q
    if (item >= ia.B * ia.K) return;
    const int b = item / ia.K, q = item % ia.K;
    const int l = ia.ells[q], m = ia.mms[q];
    ImrBin &bin = w.imr_bin[b];
    const int np = w.npts[b];
    if (np <= 0) return;
    const BinaryRec &rec = w.bins[b];
    Grid g;
    g.n = w.nsteps[b];
    g.base = (size_t)w.row_off[b];
    g.x = w.tin + g.base;
    g.t0 = g.x[0];
    g.tend = g.x[g.n - 1];
    g.dT = ia.dt / (rec.Mt * kMTSUN_SI);
    g.np = np;
    const double m1 = rec.m1s, m2 = rec.m2s, chi1 = rec.chi1, chi2 = rec.chi2;
    const double chiS = 0.5 * (chi1 + chi2), chiA = 0.5 * (chi1 - chi2);
    const double eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
    const bool is55 = (l == 5 && m == 5);
    auto arr = [&](int k) { return sm + k * kImrWin; };

    // t_peak: the knot with the largest slope of the phase spline, the first
    // of equals (a running maximum from knot 0 with a strict comparison:
    // NaN slopes never win, and a NaN at knot 0 keeps knot 0).  Each lane
    // takes every 32nd knot; the lanes' bests are merged by (value, lowest
    // knot), an order in which every lane ends with the same winner.
    int ip = 0;
    {
        const double *om = w.cA + g.base;
        double lv = 0.0;
        int li = -1;
        for (int i = lane; i < g.n; i += 32) {
            const double v = om[i];
            if (li < 0 ? (v == v) : (v > lv)) {
                lv = v;
                li = i;
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double ov = __shfl_xor_sync(0xffffffffu, lv, off);
            const int oi = __shfl_xor_sync(0xffffffffu, li, off);
            if (oi >= 0 && (li < 0 || ov > lv || (ov == lv && oi < li))) {
                lv = ov;
                li = oi;
            }
        }
        const double v0 = om[0];
        ip = (v0 == v0 && li >= 0) ? li : 0;
    }
    const double t_peak = g.x[ip];
    const double dt22 = nr_delta_t22(m1, m2, chi1, chi2);
    const int idx = grid_nearest(g, t_peak - dt22);

    double *T = arr(0), *AMP = arr(1), *PH = arr(2), *R = arr(3), *PR = arr(4), *OM = arr(5);
    ImrRec c;

    // ---- NQC coefficients
    const double t_nr = t_peak - (dt22 + (is55 ? 10.0 : 0.0));
    const int idn = grid_nearest(g, t_nr);
    const int lo = idn - 7, W = np - lo;
    if (lo < 0 || W < 3 || W > kImrWin) {
        if (lane == 0) atomicOr(&bin.fail, 1);
        return;
    }
    for (int j = lane; j < W; j += 32) {
        const Sample s = eval_sample(w, g, lo + j, q, m);
        T[j] = grid_t(g, lo + j);
        AMP[j] = sqrt(s.hr * s.hr + s.hi * s.hi);
        PH[j] = atan2(s.hi, s.hr);
        R[j] = s.r;
        PR[j] = s.pr;
        OM[j] = s.om;
    }
    __syncwarp();
    unwrap_warp(PH, arr(11), W, lane);
    // the series of the amplitude columns q_1 |h|, q_2 |h|, q_3 |h| and of the
    // phase columns p_1, p_2
    for (int j = lane; j < W; j += 32) {
        const double rO = R[j] * OM[j];
        const double q1 = PR[j] * PR[j] / (rO * rO);
        const double q2 = q1 / R[j];
        const double q3 = q2 / sqrt(R[j]);
        arr(6)[j] = q1 * AMP[j];
        arr(7)[j] = q2 * AMP[j];
        arr(8)[j] = q3 * AMP[j];
        const double p1 = PR[j] / (R[j] * OM[j]);
        arr(9)[j] = p1;
        arr(10)[j] = p1 * PR[j] * PR[j];
    }
    __syncwarp();
    // lane 0..2: q columns, 3: |h|, 4..5: p columns, 6: phase
    double so[3] = {0.0, 0.0, 0.0};
    if (lane < 7) {
        const double *Y = (lane < 3) ? arr(6 + lane) : (lane == 3) ? AMP : (lane < 6) ? arr(5 + lane) : PH;
        window_spline(T, Y, W, arr(imr_scr_arr(2 * lane)), arr(imr_scr_arr(2 * lane + 1)), t_nr, so);
    }
    double Q[3][3];
    for (int col = 0; col < 3; ++col)
        for (int i = 0; i < 3; ++i) Q[i][col] = __shfl_sync(0xffffffffu, so[i], col);
    double av[3];
    for (int i = 0; i < 3; ++i) av[i] = __shfl_sync(0xffffffffu, so[i], 3);
    double ya[3] = {fabs(nr_peak_amp(l, m, m1, m2, chiS, chiA)) - av[0], nr_peak_adot(l, m, m1, m2, chiS, chiA) - av[1],
                    nr_peak_addot(l, m, m1, m2, chiS, chiA) - av[2]};
    double xa[3];
    solve_small<3>(Q, ya, xa);
    double P[2][2];
    for (int col = 0; col < 2; ++col) {
        P[0][col] = -__shfl_sync(0xffffffffu, so[1], 4 + col);
        P[1][col] = -__shfl_sync(0xffffffffu, so[2], 4 + col);
    }
    double om = __shfl_sync(0xffffffffu, so[1], 6), omd = __shfl_sync(0xffffffffu, so[2], 6);
    omd = (om * omd > 0.0) ? fabs(omd) : -fabs(omd);
    om = fabs(om);
    const double chi_n = chiS + chiA * (m1 - m2) / (m1 + m2) / (1.0 - 2.0 * eta);
    double yb[2] = {nr_peak_omega(l, m, eta, chi_n) - om, nr_peak_omegadot(l, m, eta, chi_n) - omd};
    double xb[2];
    solve_small<2>(P, yb, xb);
    c.a1 = xa[0]; c.a2 = xa[1]; c.a3 = xa[2];
    c.b1 = xb[0]; c.b2 = xb[1];

    // ---- ringdown fit window on the NQC-corrected mode
    const int nfit = (int)(20.0 / g.dT) + 1;
    const int lo2 = idx - nfit, W2 = np - lo2;
    if (lo2 < 0 || W2 < 3 || W2 > kImrWin) {
        if (lane == 0) atomicOr(&bin.fail, 1);
        return;
    }
    __syncwarp();  // every lane's spline is done before the samples overwrite t, |h| and the phase
    for (int j = lane; j < W2; j += 32) {
        const Sample s = eval_sample(w, g, lo2 + j, q, m);
        double mag, ph;
        nqc_factor(c, s.r, s.pr, s.om, &mag, &ph);
        double sp, cp;
        sincos(ph, &sp, &cp);
        const double hr = mag * (s.hr * cp - s.hi * sp), hi = mag * (s.hr * sp + s.hi * cp);
        T[j] = grid_t(g, lo2 + j);
        AMP[j] = sqrt(hr * hr + hi * hi);
        PH[j] = atan2(hi, hr);
    }
    __syncwarp();
    unwrap_warp(PH, arr(11), W2, lane);
    const double t_match = grid_t(g, idx);
    const double tq = t_match - (is55 ? 10.0 : 0.0);
    // lane 0: |h|, lane 1: the phase
    double sr[3] = {0.0, 0.0, 0.0};
    if (lane < 2) window_spline(T, lane == 0 ? AMP : PH, W2, arr(imr_scr_arr(2 * lane)), arr(imr_scr_arr(2 * lane + 1)), tq, sr);
    const double amp0 = __shfl_sync(0xffffffffu, sr[0], 0), damp0 = __shfl_sync(0xffffffffu, sr[1], 0);
    const double phi0 = __shfl_sync(0xffffffffu, sr[0], 1), om0 = __shfl_sync(0xffffffffu, sr[1], 1);

    // ---- remnant, QNM, ansatz coefficients
    const double Mf = final_mass_seobnrv4(m1, m2, chi1, chi2);
    const double af = final_spin_hbr2016(m1, m2, chi1, chi2);
    double qr, qi;
    qnm_lookup(l, m, af, &qr, &qi);
    c.om_re = qr / Mf;
    c.om_im = -qi / Mf;  // 1 / tau > 0
    const double sigmaR = -c.om_im, sigmaI = -c.om_re;
    const double chi_rd = 0.5 * (chi1 + chi2) + 0.5 * (chi1 - chi2) * (m1 - m2) / (m1 + m2) / (1.0 - 2.0 * eta);
    double c1f = rd_coeff(0, l, m, eta, chi_rd);
    const double c2f = rd_coeff(1, l, m, eta, chi_rd);
    if (l == 2 && m == 2 && sigmaR > 2.0 * c1f * tanh(c2f)) c1f = sigmaR / (2.0 * tanh(c2f));
    const double d1f = rd_coeff(2, l, m, eta, chi_rd), d2f = rd_coeff(3, l, m, eta, chi_rd);
    const double ch = cosh(c2f);
    c.c1c = 1.0 / (c1f * eta) * (damp0 - sigmaR * amp0) * ch * ch;
    c.c2c = amp0 / eta - 1.0 / (c1f * eta) * (damp0 - sigmaR * amp0) * ch * sinh(c2f);
    c.d1c = (om0 - sigmaI) * (1 + d2f) / (d1f * d2f);
    c.c1f = c1f;
    c.c2f = c2f;
    c.d1f = d1f;
    c.d2f = d2f;
    c.phi_match = phi0;
    c.eta = eta;
    if (lane != 0) return;
    w.imr_rec[(size_t)b * w.L.Kc + q] = c;
    if (q == 0) {
        // ringdown length: 30 damping times of the (2,2) QNM, truncated to whole M
        double r22, i22;
        qnm_lookup(2, 2, af, &r22, &i22);
        const double tau22 = Mf / (-i22);
        const int rd_time = (int)(30.0 * tau22);
        const int num_add = (int)((double)rd_time / g.dT) + 1;
        bin.idx = idx;
        bin.npts = idx + num_add;
    }
}

// per binary: the IMR length, or the inspiral alone with EOB_ST_IMR
__global__ void k_imr_commit(Ws w, int B)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    ImrBin &bin = w.imr_bin[b];
    if (w.npts[b] <= 0) {
        bin.on = 0;
        return;
    }
    if (bin.fail) {
        bin.on = 0;
        w.status[b] |= EOB_ST_IMR;
    } else {
        bin.on = 1;
        w.npts[b] = bin.npts;
    }
}

}  // namespace

cudaError_t launch_imr(const Ws &w, const RunArgs &a, cudaStream_t s)
{
    if (!w.imr_bin) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(w.imr_bin, 0, sizeof(ImrBin) * (size_t)a.B, s);
    if (e != cudaSuccess || !a.opt.imr) return e;
    ImrArgs ia;
    ia.B = a.B;
    ia.K = a.K;
    for (int j = 0; j < kMaxModes; ++j) { ia.ells[j] = a.ells[j]; ia.mms[j] = a.mms[j]; }
    ia.dt = a.dt;
    k_imr<<<a.B * a.K, 32, 0, s>>>(w, ia);
    k_imr_commit<<<(a.B + 127) / 128, 128, 0, s>>>(w, a.B);
    return cudaGetLastError();
}

}  // namespace eob
