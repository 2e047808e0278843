// Reference-shaped entry points: the functions the reference's Cython layer
// exposes (src/eob.pyx, src/dopr853.pyx, src/tdinterp.pyx), with the same
// array layouts, as plain launches on a caller stream.  They reuse the
// product's physics (ham_eval, flux_eval, mode_eval); the fused path of
// eob_api.cu is what the waveform class runs.
//
// The "SEOBNRv5 class" (src/EOB.cu:3343-3496) is a caller-owned device
// buffer holding one FacCoeffs table per system (eob_ctx_bytes).
#include "eob_device.cuh"
#include "physics/hyperdual.h"

using namespace eob;

namespace {

constexpr int kTPB = 128;
inline int nblk(long long n) { return (int)((n + kTPB - 1) / kTPB); }

__device__ void ham_of_add(HamCoeffs *h, const double *add, int n, int i)
{
    ham_coeffs_build(h, add[i], add[(size_t)n + i], add[2 * (size_t)n + i], add[3 * (size_t)n + i],
                     add[5 * (size_t)n + i], add[6 * (size_t)n + i], add[7 * (size_t)n + i], add[8 * (size_t)n + i]);
}

__device__ FacFluxView flux_view(const FacCoeffs *fc, const double *add, int n, int i, double nu)
{
    FacFluxView v;
    v.fc = fc;
    v.add = add + i;
    v.n = n;
    double eta = nu;
    if (eta > 0.25 && eta < 0.25 + 1e-4) eta = 0.25;
    v.eta = eta;
    v.equal_mass = (eta == 0.25) ? 1.0 : 0.0;
    v.h22 = add[9 * (size_t)n + i];
    return v;
}

__global__ void k_eval_ham(double *out, const double *r, const double *pr, const double *pphi, const double *m1,
                           const double *m2, const double *c1, const double *c2, double K, double d5, double dSO,
                           double dSS, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HamCoeffs h;
    ham_coeffs_build(&h, m1[i], m2[i], c1[i], c2[i], K, d5, dSO, dSS);
    HamEval e;
    ham_eval(h, r[i], pr[i], pphi[i], &e);
    out[i] = e.H;
}

__global__ void k_grad_ham(const double *arg, double *g, const double *add, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HamCoeffs h;
    ham_of_add(&h, add, n, i);
    HamEval e;
    ham_eval(h, arg[i], arg[2 * (size_t)n + i], arg[3 * (size_t)n + i], &e);
    g[i] = e.dHdr;
    g[(size_t)n + i] = 0.0;
    g[2 * (size_t)n + i] = e.dHdpr;
    g[3 * (size_t)n + i] = e.dHdL;
}

__global__ void k_hess_ham(const double *arg, double *hs, const double *add, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HamCoeffs h;
    ham_of_add(&h, add, n, i);
    using hd::HD3;
    HD3 r(arg[i]), pr(arg[2 * (size_t)n + i]), L(arg[3 * (size_t)n + i]);
    r.g[0] = 1.0;
    pr.g[1] = 1.0;
    L.g[2] = 1.0;
    const HD3 he = ham_heff<HD3>(h, r, pr, L);
    const double H = ham_H_from_heff<double>(h, he.v);
    const double M2nu = h.M * h.M / h.nu;
    // (r, phi, pr, pphi) -> jet variable (0, -, 1, 2); symmetric index map
    const int map[4] = {0, -1, 1, 2};
    const int hq[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
            const int p = map[a], q = map[b];
            double v = 0.0;
            if (p >= 0 && q >= 0) v = (-(he.g[p] * he.g[q] / (H * H * H)) * M2nu + he.h[hq[p][q]] / H) * M2nu;
            hs[(size_t)(4 * a + b) * n + i] = v;
        }
}

__global__ void k_ic_cons(double *res, const double *x, double *args, const double *add, double *g, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HamCoeffs h;
    ham_of_add(&h, add, n, i);
    const double r = x[i], pphi = x[(size_t)n + i];
    args[i] = r;
    args[(size_t)n + i] = 0.0;
    args[2 * (size_t)n + i] = 0.0;
    args[3 * (size_t)n + i] = pphi;
    HamEval e;
    ham_eval(h, r, 0.0, pphi, &e);
    g[i] = e.dHdr;
    g[(size_t)n + i] = 0.0;
    g[2 * (size_t)n + i] = e.dHdpr;
    g[3 * (size_t)n + i] = e.dHdL;
    res[i] = e.dHdL - add[4 * (size_t)n + i];
    res[(size_t)n + i] = e.dHdr;
}

__device__ void newton_res(const HamCoeffs &h, double omega0, double r, double pphi, double res[2])
{
    HamEval e;
    ham_eval(h, r, 0.0, pphi, &e);
    res[0] = e.dHdL - omega0;
    res[1] = e.dHdr;
}

__global__ void k_root_find_all(double *xOut, const double *x0In, const double *add, int max_iter, double err, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HamCoeffs h;
    ham_of_add(&h, add, n, i);
    const double omega0 = add[4 * (size_t)n + i];
    const double sq_eps = sqrt(2.22e-16);
    double x0[2] = {x0In[i], x0In[(size_t)n + i]}, x1[2] = {x0[0], x0[1]};
    for (int it = 0; it < max_iter; ++it) {
        x1[0] = x0[0];
        x1[1] = x0[1];
        double r1[2], J[2][2];
        newton_res(h, omega0, x1[0], x1[1], r1);
        for (int j = 0; j < 2; ++j) {
            const double dj = sq_eps * fabs(x1[j]);
            double xt[2] = {x1[0], x1[1]};
            xt[j] += dj;
            double r2[2];
            newton_res(h, omega0, xt[0], xt[1], r2);
            J[0][j] = (r2[0] - r1[0]) / dj;
            J[1][j] = (r2[1] - r1[1]) / dj;
        }
        const double det = 1.0 / (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
        x1[0] -= det * J[1][1] * r1[0] + det * -J[0][1] * r1[1];
        x1[1] -= det * -J[1][0] * r1[0] + det * J[0][0] * r1[1];
        const double d0 = fabs(x1[0] - x0[0]) / x0[0], d1 = fabs(x1[1] - x0[1]) / x0[1];
        x0[0] = x1[0];
        x0[1] = x1[1];
        if ((d1 > d0 ? d1 : d0) < err) break;
    }
    xOut[i] = x1[0];
    xOut[(size_t)n + i] = x1[1];
}

__global__ void k_ctx_update(FacCoeffs *ctx, const double *m1, const double *m2, const double *eta, const double *tpl,
                             const double *chiS, const double *chiA, int use_hm, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fac_coeffs_build(&ctx[i], use_hm, m1[i], m2[i], eta[i], tpl[i], chiS[i], chiA[i]);
}

__device__ void rhs_ref(const FacCoeffs *ctx, const double *add, int n, int i, int idx, const double y[4], double k[4])
{
    HamCoeffs h;
    ham_of_add(&h, add, n, i);
    const FacFluxView v = flux_view(&ctx[idx], add, n, i, h.nu);
    eob_rhs(h, v, y, k);
}

__global__ void k_ctx_ode(const FacCoeffs *ctx, const double *arg, double *k, const double *add, int n, const int *idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double y[4] = {arg[i], arg[(size_t)n + i], arg[2 * (size_t)n + i], arg[3 * (size_t)n + i]};
    double kk[4];
    rhs_ref(ctx, add, n, i, idx ? idx[i] : i, y, kk);
    for (int q = 0; q < 4; ++q) k[(size_t)q * n + i] = kk[q];
}

__global__ void k_ctx_rr_force(const FacCoeffs *ctx, double *force, double *g, const double *args, const double *add,
                               int n, const int *idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HamCoeffs h;
    ham_of_add(&h, add, n, i);
    const double r = args[i], pr = args[2 * (size_t)n + i], L = args[3 * (size_t)n + i];
    HamEval e;
    ham_eval(h, r, pr, L, &e);
    HamEval e0;
    ham_eval(h, r, 0.0, L, &e0);
    if (g) {
        g[i] = e0.dHdr;
        g[(size_t)n + i] = 0.0;
        g[2 * (size_t)n + i] = e0.dHdpr;
        g[3 * (size_t)n + i] = e0.dHdL;
    }
    const FacFluxView v = flux_view(&ctx[idx ? idx[i] : i], add, n, i, h.nu);
    const double omega = add[4 * (size_t)n + i];
    const double flux = flux_eval(v, r, L, omega, e.Hreal, e.omega_c) / h.nu;
    const double fo = flux / omega;
    force[i] = -pr / L * fo;
    force[(size_t)n + i] = -fo;
}

__device__ double diss_res(const FacCoeffs *fc, const double *add, int n, int i, const HamCoeffs &h, double r,
                           double pr, double L, int ic_mode)
{
    HamEval e;
    ham_eval(h, r, pr, L, &e);
    if (ic_mode == 0) return -e.dHdpr;
    using hd::HD3;
    HD3 R(r), P(pr), Lv(L);
    R.g[0] = 1.0;
    P.g[1] = 1.0;
    Lv.g[2] = 1.0;
    const HD3 he = ham_heff<HD3>(h, R, P, Lv);
    const double H = ham_H_from_heff<double>(h, he.v);
    const double M2nu = h.M * h.M / h.nu;
    const double d2rr = (-(he.g[0] * he.g[0] / (H * H * H)) * M2nu + he.h[0] / H) * M2nu;
    const double d2rL = (-(he.g[0] * he.g[2] / (H * H * H)) * M2nu + he.h[2] / H) * M2nu;
    const FacFluxView v = flux_view(fc, add, n, i, h.nu);
    const double flux = flux_eval(v, r, L, e.dHdL, e.Hreal, e.omega_c) / h.nu;
    return (-flux / e.dHdL) / (-d2rr / d2rL) - e.dHdpr;
}

__global__ void k_ctx_root_scalar(const FacCoeffs *ctx, double *pr_res, const double *bounds, const double *argsIn,
                                  const double *add, int max_iter, double err, int n, int ic_mode)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    HamCoeffs h;
    ham_of_add(&h, add, n, i);
    const double r = argsIn[i], L = argsIn[3 * (size_t)n + i];
    double A = bounds[i], B = bounds[(size_t)n + i];
    double fa = diss_res(&ctx[i], add, n, i, h, r, A, L, ic_mode), fb = diss_res(&ctx[i], add, n, i, h, r, B, L, ic_mode);
    double c = 0.0;
    if (fb == fa) {
        c = (fb == 0.0) ? B : A;
    } else {
        for (int it = 1; it <= max_iter; ++it) {
            c = (A * fb - B * fa) / (fb - fa);
            const double fc = diss_res(&ctx[i], add, n, i, h, r, c, L, ic_mode);
            if ((fb < 0.0 && fc < 0.0) || (fb >= 0.0 && fc >= 0.0)) { B = c; fb = fc; } else { A = c; fa = fc; }
            if (fabs(fc) < err) break;
        }
    }
    pr_res[i] = c;
}

__global__ void k_ctx_waveform(const FacCoeffs *ctx, double *out, const double *r, const double *phi,
                               const double *pphi, const double *v, const double *Hreal, const double *eta,
                               const double *vPhi, int l, int m, const double *prefix, double h22, int numSys, int L,
                               const int *idx)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= (long long)numSys * L) return;
    const int b = (int)(j / L);
    const cdbl hl = mode_eval(ctx[idx ? idx[b] : b], l, m, prefix[2 * b], prefix[2 * b + 1], eta[b], r[j], phi[j],
                              pphi[j], v[j], Hreal[j], vPhi[j], h22, false);
    out[2 * j] = hl.re;
    out[2 * j + 1] = hl.im;
}

// compute_hlms (src/EOB.cu:3147-3322) as the function it was written to be:
// one thread per (binary, trajectory row), every mode of the list.  H and
// its gradients at the state and at p_r = 0 from the binary's additionalArgs
// (as the reference's gradient calls), nu from m1_arr/m2_arr (as its
// H_val), v = omega^(1/3), the vPhi input 1/(omega_c^2 r^3), the prefixes
// [K][num_bin_all] that update_information was given.
__global__ void k_ctx_compute_hlms(const FacCoeffs *ctx, double *hlms, const double *r_arr, const double *phi_arr,
                                   const double *pr_arr, const double *L_arr, const double *m1_arr,
                                   const double *m2_arr, const int *num_steps, int num_steps_max, const int *ells,
                                   const int *mms, int K, int n, const double *add, const double *prefixes)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= (long long)n * num_steps_max) return;
    const int b = (int)(j / num_steps_max), i = (int)(j % num_steps_max);
    if (i >= num_steps[b]) return;
    HamCoeffs h;
    ham_of_add(&h, add, n, b);
    const double r = r_arr[j], phi = phi_arr[j], pr = pr_arr[j], L = L_arr[j];
    HamEval e;
    ham_eval(h, r, pr, L, &e);
    const double m1 = m1_arr[b], m2 = m2_arr[b];
    const double nu = m1 * m2 / ((m1 + m2) * (m1 + m2));
    const double Hval = nu * e.H;
    const double v = cbrt(e.dHdL);
    const double vPhi = 1.0 / (e.omega_c * e.omega_c * (r * r * r));
    const double h22 = add[9 * (size_t)n + b];
    for (int k = 0; k < K; ++k) {
        const size_t pk = 2 * ((size_t)k * n + b);
        const cdbl hl = mode_eval(ctx[b], ells[k], mms[k], prefixes[pk], prefixes[pk + 1], nu, r, phi, L, v, Hval,
                                  vPhi, h22, false);
        const size_t o = 2 * (((size_t)b * K + k) * num_steps_max + i);
        hlms[o] = hl.re;
        hlms[o + 1] = hl.im;
    }
}

// ---- DOPR853 pieces (src/DOPR853.cu) ----
__constant__ double kA[13][11];  // a[s][slot] (slot 1..10), zero where unused; filled by the host once
__constant__ double kC[13];

__global__ void k_dopr_steps(const double *x, double *xCurrent, const double *solOld, const double *h, double *arg,
                             const double *add, double *k1, double *k2, double *k3, double *k4, double *k5, double *k6,
                             double *k7, double *k8, double *k9, double *k10, double *ak, int nargs, int n,
                             const FacCoeffs *ctx, const int *idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double *ks[11] = {nullptr, k1, k2, k3, k4, k5, k6, k7, k8, k9, k10};
    const int out_slot[13] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 2, 3};
    const double hh = h[i];
    double kv[11][4];
    for (int s = 1; s <= 12; ++s) {
        double a4[4];
        for (int q = 0; q < nargs; ++q) {
            double acc = 0.0;
            // accumulation order of the reference: k1, k4.., stage 11 includes k2 last
            for (int t = 1; t <= 10; ++t) {
                if (kA[s][t] != 0.0 && !(s == 12 && t == 2)) acc += kA[s][t] * kv[t][q];
            }
            if (s == 12) acc += kA[12][2] * kv[2][q];
            ak[(size_t)q * n + i] = acc;
            a4[q] = solOld[(size_t)q * n + i] + hh * acc;
            arg[(size_t)q * n + i] = a4[q];
        }
        xCurrent[i] = x[i] + kC[s] * hh;
        double kk[4];
        rhs_ref(ctx, add, n, i, idx ? idx[i] : i, a4, kk);
        for (int q = 0; q < 4; ++q) {
            kv[out_slot[s]][q] = kk[q];
            ks[out_slot[s]][(size_t)q * n + i] = kk[q];
        }
    }
}

__global__ void k_dopr_error(double *err, const double *solOld, double *solNew, const double *h, const double *k1,
                             const double *k2, const double *k3, const double *k6, const double *k7, const double *k8,
                             const double *k9, const double *k10, int n, int nargs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double b1 = 5.42937341165687622380535766363e-2, b6 = 4.45031289275240888144113950566e0,
                 b7 = 1.89151789931450038304281599044e0, b8 = -5.8012039600105847814672114227e0,
                 b9 = 3.1116436695781989440891606237e-1, b10 = -1.52160949662516078556178806805e-1,
                 b11 = 2.01365400804030348374776537501e-1, b12 = 4.47106157277725905176885569043e-2;
    const double bhh1 = 0.244094488188976377952755905512e+00, bhh2 = 0.733846688281611857341361741547e+00,
                 bhh3 = 0.220588235294117647058823529412e-01;
    const double er1 = 0.1312004499419488073250102996e-01, er6 = -0.1225156446376204440720569753e+01,
                 er7 = -0.4957589496572501915214079952e+00, er8 = 0.1664377182454986536961530415e+01,
                 er9 = -0.3503288487499736816886487290e+00, er10 = 0.3341791187130174790297318841e+00,
                 er11 = 0.8192320648511571246570742613e-01, er12 = -0.2235530786388629525884427845e-01;
    const double hh = h[i];
    double e1 = 0.0, e2 = 0.0;
    for (int q = 0; q < nargs; ++q) {
        const size_t o = (size_t)q * n + i;
        const double t = b1 * k1[o] + b6 * k6[o] + b7 * k7[o] + b8 * k8[o] + b9 * k9[o] + b10 * k10[o] + b11 * k2[o] +
                         b12 * k3[o];
        const double so = solOld[o];
        const double sn = so + hh * t;
        solNew[o] = sn;
        const double mx = (so > sn) ? so : sn;
        const double sk = 1.0 / (1e-12 + 1e-12 * mx);
        double v = (t - bhh1 * k1[o] - bhh2 * k9[o] - bhh3 * k3[o]) * sk;
        double v2 = v * v;
        double w = 1.0;
        for (int p = 0; p < nargs / 2; ++p) w *= v2;
        if (nargs % 2) w *= v;
        e2 += w;
        v = (er1 * k1[o] + er6 * k6[o] + er7 * k7[o] + er8 * k8[o] + er9 * k9[o] + er10 * k10[o] + er11 * k2[o] +
             er12 * k3[o]) * sk;
        v2 = v * v;
        w = 1.0;
        for (int p = 0; p < nargs / 2; ++p) w *= v2;
        if (nargs % 2) w *= v;
        e1 += w;
    }
    double denom = e1 + 0.01 * e2;
    denom = (denom < 0.0) ? 1.0 : denom;
    err[i] = fabs(hh) * e1 * sqrt(1.0 / ((double)nargs * denom));
}

__global__ void k_dopr_controller(unsigned char *flag, const double *err, double *errOld, unsigned char *prev,
                                  double *h, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double e = err[i];
    if (e <= 1.0) {
        double scale;
        if (e == 0.0) scale = 6.0;
        else {
            scale = 0.9 / sqrt(sqrt(sqrt(e)));
            if (scale > 6.0) scale = 6.0; else if (scale < 1.0 / 3.0) scale = 1.0 / 3.0;
        }
        if (prev[i] && scale > 1.0) scale = 1.0;
        h[i] = h[i] * scale;
        double eo = e;
        if (eo < 1e-4) eo = 1e-4; else if (eo > 1e300) eo = 1e300;
        errOld[i] = eo;
        prev[i] = 0;
        flag[i] = 1;
    } else {
        prev[i] = 1;
        flag[i] = 0;
        double t = 0.9 / sqrt(sqrt(sqrt(e)));
        if (t < 1.0 / 3.0) t = 1.0 / 3.0; else if (t > 1e300) t = 1e300;
        h[i] = h[i] * t;
    }
}

// interpolate_TD layout: t[L][numBinAll], y[L][ninterp] with interp = sub * numBinAll + bin
__global__ void k_interp_td(const double *t, const double *y, double *Bv, double *ud, double *dg, double *ld,
                            const int *lengths, int numBinAll, int ninterp)
{
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= ninterp) return;
    const int b = ip % numBinAll;
    const int n = lengths[b];
    if (n < 3) return;
#define X(i) t[(size_t)(i) * numBinAll + b]
#define Y(i) y[(size_t)(i) * ninterp + ip]
#define R(a, i) a[(size_t)(i) * ninterp + ip]
    for (int i = 0; i < n; ++i) {
        int i0, i1, i2;
        if (i == n - 1) { i0 = n - 3; i1 = n - 2; i2 = n - 1; }
        else if (i == 0) { i0 = 0; i1 = 1; i2 = 2; }
        else { i0 = i - 1; i1 = i; i2 = i + 1; }
        const double dx1 = X(i1) - X(i0), dx2 = X(i2) - X(i1), d = X(i2) - X(i0);
        const double y1 = Y(i1);
        const double s1 = (y1 - Y(i0)) / dx1, s2 = (Y(i2) - y1) / dx2;
        if (i == n - 1) { R(Bv, i) = (dx2 * dx2 * s1 + (2 * d + dx2) * dx1 * s2) / d; R(dg, i) = dx1; R(ld, i) = d; R(ud, i) = 0.0; }
        else if (i == 0) { R(Bv, i) = ((dx1 + 2 * d) * dx2 * s1 + dx1 * dx1 * s2) / d; R(ud, i) = d; R(ld, i) = 0.0; R(dg, i) = dx2; }
        else { R(Bv, i) = 3.0 * (dx2 * s1 + dx1 * s2); R(dg, i) = 2 * (dx1 + dx2); R(ud, i) = dx1; R(ld, i) = dx2; }
    }
    for (int i = 1; i < n; ++i) {
        const double w = R(ld, i) / R(dg, i - 1);
        R(dg, i) = R(dg, i) - w * R(ud, i - 1);
        R(Bv, i) = R(Bv, i) - w * R(Bv, i - 1);
    }
    R(Bv, n - 1) = R(Bv, n - 1) / R(dg, n - 1);
    for (int i = n - 2; i >= 0; --i) R(Bv, i) = (R(Bv, i) - R(ud, i) * R(Bv, i + 1)) / R(dg, i);
    for (int i = 0; i < n - 1; ++i) {
        const double dx = X(i + 1) - X(i);
        const double slope = (Y(i + 1) - Y(i)) / dx;
        const double bi = R(Bv, i);
        const double tt = (bi + R(Bv, i + 1) - 2 * slope) / dx;
        R(ud, i) = bi;
        R(dg, i) = (slope - bi) / dx - tt;
        R(ld, i) = tt / dx;
    }
#undef X
#undef Y
#undef R
}

bool g_tableau_ready = false;

cudaError_t ensure_tableau()
{
    if (g_tableau_ready) return cudaSuccess;
    // a[s][slot] of the stages (src/DOPR853.cu:52-128); stage 11 writes k2, stage 12 writes k3
    double A[13][11] = {};
    double C[13] = {0.0, 0.0, 0.526001519587677318785587544488e-01, 0.789002279381515978178381316732e-01,
                    0.118350341907227396726757197510e+00, 0.281649658092772603273242802490e+00,
                    0.333333333333333333333333333333e+00, 0.25e+00, 0.307692307692307692307692307692e+00,
                    0.651282051282051282051282051282e+00, 0.6e+00, 0.857142857142857142857142857142e+00, 1.0};
    A[2][1] = 5.26001519587677318785587544488e-2;
    A[3][1] = 1.97250569845378994544595329183e-2; A[3][2] = 5.91751709536136983633785987549e-2;
    A[4][1] = 2.95875854768068491816892993775e-2; A[4][3] = 8.87627564304205475450678981324e-2;
    A[5][1] = 2.41365134159266685502369798665e-1; A[5][3] = -8.84549479328286085344864962717e-1;
    A[5][4] = 9.24834003261792003115737966543e-1;
    A[6][1] = 3.7037037037037037037037037037e-2; A[6][4] = 1.70828608729473871279604482173e-1;
    A[6][5] = 1.25467687566822425016691814123e-1;
    A[7][1] = 3.7109375e-2; A[7][4] = 1.70252211019544039314978060272e-1; A[7][5] = 6.02165389804559606850219397283e-2;
    A[7][6] = -1.7578125e-2;
    A[8][1] = 3.70920001185047927108779319836e-2; A[8][4] = 1.70383925712239993810214054705e-1;
    A[8][5] = 1.07262030446373284651809199168e-1; A[8][6] = -1.53194377486244017527936158236e-2;
    A[8][7] = 8.27378916381402288758473766002e-3;
    A[9][1] = 6.24110958716075717114429577812e-1; A[9][4] = -3.36089262944694129406857109825e0;
    A[9][5] = -8.68219346841726006818189891453e-1; A[9][6] = 2.75920996994467083049415600797e1;
    A[9][7] = 2.01540675504778934086186788979e1; A[9][8] = -4.34898841810699588477366255144e1;
    A[10][1] = 4.77662536438264365890433908527e-1; A[10][4] = -2.48811461997166764192642586468e0;
    A[10][5] = -5.90290826836842996371446475743e-1; A[10][6] = 2.12300514481811942347288949897e1;
    A[10][7] = 1.52792336328824235832596922938e1; A[10][8] = -3.32882109689848629194453265587e1;
    A[10][9] = -2.03312017085086261358222928593e-2;
    A[11][1] = -9.3714243008598732571704021658e-1; A[11][4] = 5.18637242884406370830023853209e0;
    A[11][5] = 1.09143734899672957818500254654e0; A[11][6] = -8.14978701074692612513997267357e0;
    A[11][7] = -1.85200656599969598641566180701e1; A[11][8] = 2.27394870993505042818970056734e1;
    A[11][9] = 2.49360555267965238987089396762e0; A[11][10] = -3.0467644718982195003823669022e0;
    A[12][1] = 2.27331014751653820792359768449e0; A[12][4] = -1.05344954667372501984066689879e1;
    A[12][5] = -2.00087205822486249909675718444e0; A[12][6] = -1.79589318631187989172765950534e1;
    A[12][7] = 2.79488845294199600508499808837e1; A[12][8] = -2.85899827713502369474065508674e0;
    A[12][9] = -8.87285693353062954433549289258e0; A[12][10] = 1.23605671757943030647266201528e1;
    A[12][2] = 6.43392746015763530355970484046e-1;
    cudaError_t e = cudaMemcpyToSymbol(kA, A, sizeof(A));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(kC, C, sizeof(C));
    if (e == cudaSuccess) g_tableau_ready = true;
    return e;
}

inline int ret(cudaError_t e) { return e == cudaSuccess ? EOB_OK : EOB_E_CUDA; }

}  // namespace

extern "C" {

int eob_evaluate_ham(double *out, const double *r, const double *phi, const double *pr, const double *pphi,
                     const double *m_1, const double *m_2, const double *chi_1, const double *chi_2, double K,
                     double d5, double dSO, double dSS, int numSys, cudaStream_t stream)
{
    (void)phi;
    if (numSys < 0 || (numSys > 0 && (!out || !r || !pr || !pphi || !m_1 || !m_2 || !chi_1 || !chi_2))) return EOB_E_ARG;
    if (numSys == 0) return EOB_OK;
    k_eval_ham<<<nblk(numSys), kTPB, 0, stream>>>(out, r, pr, pphi, m_1, m_2, chi_1, chi_2, K, d5, dSO, dSS, numSys);
    return ret(cudaGetLastError());
}

int eob_grad_ham(const double *arg, double *grad_out, const double *add, int numSys, cudaStream_t stream)
{
    if (numSys < 0 || (numSys > 0 && (!arg || !grad_out || !add))) return EOB_E_ARG;
    if (numSys == 0) return EOB_OK;
    k_grad_ham<<<nblk(numSys), kTPB, 0, stream>>>(arg, grad_out, add, numSys);
    return ret(cudaGetLastError());
}

int eob_hessian_ham(const double *arg, double *hessian_out, const double *add, int numSys, cudaStream_t stream)
{
    if (numSys < 0 || (numSys > 0 && (!arg || !hessian_out || !add))) return EOB_E_ARG;
    if (numSys == 0) return EOB_OK;
    k_hess_ham<<<nblk(numSys), kTPB, 0, stream>>>(arg, hessian_out, add, numSys);
    return ret(cudaGetLastError());
}

int eob_ic_cons(double *res, const double *x, double *args, const double *add, double *grad_out, int numSys,
                cudaStream_t stream)
{
    if (numSys < 0 || (numSys > 0 && (!res || !x || !args || !add || !grad_out))) return EOB_E_ARG;
    if (numSys == 0) return EOB_OK;
    k_ic_cons<<<nblk(numSys), kTPB, 0, stream>>>(res, x, args, add, grad_out, numSys);
    return ret(cudaGetLastError());
}

int eob_root_find_all(double *xOut, const double *x0In, const double *argsIn, const double *add, int max_iter,
                      double err, int numBinAll, int n, int num_args, int num_add_args, cudaStream_t stream)
{
    (void)argsIn;
    if (n != 2 || num_args != 4 || num_add_args < 10 || numBinAll < 0 || max_iter < 0) return EOB_E_ARG;
    if (numBinAll == 0) return EOB_OK;
    if (!xOut || !x0In || !add) return EOB_E_ARG;
    k_root_find_all<<<nblk(numBinAll), kTPB, 0, stream>>>(xOut, x0In, add, max_iter, err, numBinAll);
    return ret(cudaGetLastError());
}

size_t eob_ctx_bytes(int numSys) { return numSys > 0 ? sizeof(FacCoeffs) * (size_t)numSys : 0; }

int eob_ctx_update_information(void *ctx, const double *m1, const double *m2, const double *eta, const double *tplspin,
                               const double *chi_S, const double *chi_A, int use_hm, int numSys, cudaStream_t stream)
{
    if (!ctx || numSys < 1 || !m1 || !m2 || !eta || !tplspin || !chi_S || !chi_A) return EOB_E_ARG;
    k_ctx_update<<<nblk(numSys), kTPB, 0, stream>>>((FacCoeffs *)ctx, m1, m2, eta, tplspin, chi_S, chi_A, use_hm,
                                                     numSys);
    return ret(cudaGetLastError());
}

int eob_ctx_ode(const void *ctx, const double *x, const double *arg, double *k, const double *add, int numSys,
                const int *idx, cudaStream_t stream)
{
    (void)x;
    if (!ctx || numSys < 0 || (numSys > 0 && (!arg || !k || !add))) return EOB_E_ARG;
    if (numSys == 0) return EOB_OK;
    k_ctx_ode<<<nblk(numSys), kTPB, 0, stream>>>((const FacCoeffs *)ctx, arg, k, add, numSys, idx);
    return ret(cudaGetLastError());
}

int eob_ctx_rr_force(const void *ctx, double *force_out, double *grad_out, const double *args, const double *add,
                     int numSys, const int *idx, cudaStream_t stream)
{
    if (!ctx || numSys < 0 || (numSys > 0 && (!force_out || !args || !add))) return EOB_E_ARG;
    if (numSys == 0) return EOB_OK;
    k_ctx_rr_force<<<nblk(numSys), kTPB, 0, stream>>>((const FacCoeffs *)ctx, force_out, grad_out, args, add, numSys,
                                                       idx);
    return ret(cudaGetLastError());
}

int eob_ctx_root_find_scalar_all(const void *ctx, double *pr_res, const double *start_bounds, const double *argsIn,
                                 const double *add, int max_iter, double err, int numBinAll, int num_args,
                                 int num_add_args, int ic_mode, cudaStream_t stream)
{
    if (!ctx || num_args != 4 || num_add_args < 80 || numBinAll < 0 || max_iter < 0) return EOB_E_ARG;
    if (numBinAll == 0) return EOB_OK;
    if (!pr_res || !start_bounds || !argsIn || !add) return EOB_E_ARG;
    k_ctx_root_scalar<<<nblk(numBinAll), kTPB, 0, stream>>>((const FacCoeffs *)ctx, pr_res, start_bounds, argsIn, add,
                                                             max_iter, err, numBinAll, ic_mode);
    return ret(cudaGetLastError());
}

int eob_ctx_waveform(const void *ctx, double *out, const double *r, const double *phi, const double *pr,
                     const double *pphi, const double *v, const double *Hreal, const double *eta,
                     const double *vPhiInput, int l, int m, const double *prefix, double h22_calib, int numSys,
                     int traj_length, const int *idx, cudaStream_t stream)
{
    (void)pr;
    if (!ctx || l < 2 || l > kLMax || m < 1 || m > l || numSys < 0 || traj_length < 0) return EOB_E_ARG;
    const long long n = (long long)numSys * traj_length;
    if (n == 0) return EOB_OK;
    if (!out || !r || !phi || !pphi || !v || !Hreal || !eta || !vPhiInput || !prefix) return EOB_E_ARG;
    k_ctx_waveform<<<nblk(n), kTPB, 0, stream>>>((const FacCoeffs *)ctx, out, r, phi, pphi, v, Hreal, eta, vPhiInput,
                                                  l, m, prefix, h22_calib, numSys, traj_length, idx);
    return ret(cudaGetLastError());
}

int eob_ctx_compute_hlms(const void *ctx, double *hlms, const double *r_arr, const double *phi_arr,
                         const double *pr_arr, const double *L_arr, const double *m1_arr, const double *m2_arr,
                         const double *chi1_arr, const double *chi2_arr, const int *num_steps, int num_steps_max,
                         const int *ell_arr, const int *mm_arr, int num_modes, int num_bin_all,
                         const double *additionalArgs, int num_add_args, const double *newtonian_prefixes,
                         cudaStream_t stream)
{
    (void)chi1_arr;
    (void)chi2_arr;
    if (num_bin_all < 0 || num_steps_max < 0 || num_modes < 0) return EOB_E_ARG;
    if (num_bin_all == 0 || num_steps_max == 0 || num_modes == 0) return EOB_OK;
    if (!ctx || !hlms || !r_arr || !phi_arr || !pr_arr || !L_arr || !m1_arr || !m2_arr || !num_steps || !ell_arr ||
        !mm_arr || !additionalArgs || !newtonian_prefixes || num_add_args < 10)
        return EOB_E_ARG;
    const long long total = (long long)num_bin_all * num_steps_max;
    k_ctx_compute_hlms<<<nblk(total), kTPB, 0, stream>>>((const FacCoeffs *)ctx, hlms, r_arr, phi_arr, pr_arr, L_arr,
                                                          m1_arr, m2_arr, num_steps, num_steps_max, ell_arr, mm_arr,
                                                          num_modes, num_bin_all, additionalArgs, newtonian_prefixes);
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

int eob_dopr853_steps(const double *x, double *xCurrent, const double *solOld, const double *h, double *arg,
                      const double *add, double *k1, double *k2, double *k3, double *k4, double *k5, double *k6,
                      double *k7, double *k8, double *k9, double *k10, double *ak, int nargs, int numEq,
                      int num_add_args, const void *ctx, const int *idx, cudaStream_t stream)
{
    if (nargs != 4 || num_add_args < 80 || numEq < 0 || !ctx) return EOB_E_ARG;
    if (numEq == 0) return EOB_OK;
    cudaError_t e = ensure_tableau();
    if (e != cudaSuccess) return EOB_E_CUDA;
    k_dopr_steps<<<nblk(numEq), kTPB, 0, stream>>>(x, xCurrent, solOld, h, arg, add, k1, k2, k3, k4, k5, k6, k7, k8,
                                                    k9, k10, ak, nargs, numEq, (const FacCoeffs *)ctx, idx);
    return ret(cudaGetLastError());
}

int eob_dopr853_error(double *err, const double *solOld, double *solNew, const double *h, const double *k1,
                      const double *k2, const double *k3, const double *k6, const double *k7, const double *k8,
                      const double *k9, const double *k10, int numEq, int nargs, cudaStream_t stream)
{
    if (numEq < 0 || nargs < 1) return EOB_E_ARG;
    if (numEq == 0) return EOB_OK;
    k_dopr_error<<<nblk(numEq), kTPB, 0, stream>>>(err, solOld, solNew, h, k1, k2, k3, k6, k7, k8, k9, k10, numEq,
                                                    nargs);
    return ret(cudaGetLastError());
}

int eob_dopr853_controller(unsigned char *flagSuccess, const double *err, double *errOld, unsigned char *prev,
                           double *h, const double *x, int numEq, int nargs, cudaStream_t stream)
{
    (void)x;
    (void)nargs;
    if (numEq < 0) return EOB_E_ARG;
    if (numEq == 0) return EOB_OK;
    k_dopr_controller<<<nblk(numEq), kTPB, 0, stream>>>(flagSuccess, err, errOld, prev, h, numEq);
    return ret(cudaGetLastError());
}

int eob_interpolate_td(const double *t_arr, const double *propArrays, double *B, double *upper_diag, double *diag,
                       double *lower_diag, const int *lengths, int numBinAll, int nsubs, cudaStream_t stream)
{
    if (numBinAll < 0 || nsubs < 1) return EOB_E_ARG;
    if (numBinAll == 0) return EOB_OK;
    if (!t_arr || !propArrays || !B || !upper_diag || !diag || !lower_diag || !lengths) return EOB_E_ARG;
    const int ninterp = numBinAll * nsubs;
    k_interp_td<<<nblk(ninterp), kTPB, 0, stream>>>(t_arr, propArrays, B, upper_diag, diag, lower_diag, lengths,
                                                     numBinAll, ninterp);
    return ret(cudaGetLastError());
}

}  // extern "C"
