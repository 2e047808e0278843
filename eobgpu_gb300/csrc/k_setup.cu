// Setup kernel: per-binary coefficient tables and initial conditions.
//
// One thread per binary.  Restates, per binary, the reference's setup_class
// (eob/seobnrv4phm.py:1922-1964: mass scaling, Newtonian prefixes, packing),
// SEOBNRv5::update_information (src/EOB.cu:3355-3374: waveform coefficients)
// and get_initial_conditions (eob/seobnrv4phm.py:1966-2070):
//   (r0, pphi0): discrete Newton on (dH/dpphi - omega0, dH/dr) at p_r = 0
//                (src/EOB.cu:2864-2968: forward differences with
//                sqrt(2.22e-16)|x|, stop when max |dx/x| < 1e-12, <= 1000 its),
//   p_r0:        false position on [-0.03, 0] (src/EOB.cu:2711-2775).
#include "eob_device.cuh"
#include "physics/hyperdual.h"

namespace eob {

__device__ void ic_cons_res(const HamCoeffs &h, double omega0, double r, double pphi, double res[2])
{
    HamEval e;
    ham_eval(h, r, 0.0, pphi, &e);
    res[0] = e.dHdL - omega0;
    res[1] = e.dHdr;
}

__device__ int ic_newton(const HamCoeffs &h, double omega0, double x[2], int max_iter, double err)
{
    const double sq_eps = sqrt(2.22e-16);
    double x0[2] = {x[0], x[1]};
    double x1[2] = {x[0], x[1]};
    for (int it = 0; it < max_iter; ++it) {
        x1[0] = x0[0];
        x1[1] = x0[1];
        double r1[2], J[2][2];
        ic_cons_res(h, omega0, x1[0], x1[1], r1);
        for (int j = 0; j < 2; ++j) {
            const double dj = sq_eps * fabs(x1[j]);
            double xt[2] = {x1[0], x1[1]};
            xt[j] += dj;
            double r2[2];
            ic_cons_res(h, omega0, xt[0], xt[1], r2);
            J[0][j] = (r2[0] - r1[0]) / dj;
            J[1][j] = (r2[1] - r1[1]) / dj;
        }
        const double det = 1.0 / (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
        const double i00 = det * J[1][1], i01 = det * -J[0][1], i10 = det * -J[1][0], i11 = det * J[0][0];
        x1[0] -= i00 * r1[0] + i01 * r1[1];
        x1[1] -= i10 * r1[0] + i11 * r1[1];
        const double d0 = fabs(x1[0] - x0[0]) / x0[0], d1 = fabs(x1[1] - x0[1]) / x0[1];
        const double rel = (d1 > d0) ? d1 : d0;
        x0[0] = x1[0];
        x0[1] = x1[1];
        if (rel < err) {
            x[0] = x1[0];
            x[1] = x1[1];
            return it + 1;
        }
    }
    x[0] = x1[0];
    x[1] = x1[1];
    return -1;
}

// Dissipative residual rdot(F) - dH/dpr.  ic_mode 0 reproduces the
// reference's evaluation, whose d2H/dr2 (src/EOB.cu:322) is larger than the
// true value by more than 1e6 so that its rdot term vanishes below the solver
// tolerance; ic_mode 1 is the physical condition with the exact Hessian.
__device__ double ic_diss_res(const BinaryRec &b, double r, double pr, double L, int ic_mode)
{
    HamEval e;
    ham_eval(b.ham, r, pr, L, &e);
    if (ic_mode == 0) return -e.dHdpr;
    // d2Heff/dr2 and d2Heff/dr dL from the generic evaluator with hyper-duals
    using hd::HD2;
    HD2 R(r), P(pr), Lv(L);
    R.g0 = 1.0;
    Lv.g1 = 1.0;
    const HD2 heff = ham_heff<HD2>(b.ham, R, P, Lv);
    const double H = ham_H_from_heff<double>(b.ham, heff.v);
    const double M2nu = b.ham.M * b.ham.M / b.ham.nu;
    const double d2rr = (-(heff.g0 * heff.g0 / (H * H * H)) * M2nu + heff.h00 / H) * M2nu;
    const double d2rL = (-(heff.g0 * heff.g1 / (H * H * H)) * M2nu + heff.h01 / H) * M2nu;
    const double flux = flux_eval(b.flux, r, L, e.dHdL, e.Hreal, e.omega_c) / b.ham.nu;
    const double Fphi = -flux / e.dHdL;
    const double dLdr = -d2rr / d2rL;
    return Fphi / dLdr - e.dHdpr;
}

__device__ double ic_false_position(const BinaryRec &b, double r, double L, double lo, double hi, int max_iter,
                                    double err, int ic_mode)
{
    double A = lo, B = hi;
    double fa = ic_diss_res(b, r, A, L, ic_mode), fb = ic_diss_res(b, r, B, L, ic_mode);
    if (fb == fa) return (fb == 0.0) ? B : A;
    double c = 0.0;
    for (int it = 1; it <= max_iter; ++it) {
        c = (A * fb - B * fa) / (fb - fa);
        const double fc = ic_diss_res(b, r, c, L, ic_mode);
        if ((fb < 0.0 && fc < 0.0) || (fb >= 0.0 && fc >= 0.0)) {
            B = c;
            fb = fc;
        } else {
            A = c;
            fa = fc;
        }
        if (fabs(fc) < err) break;
    }
    return c;
}

// Builds BinaryRec + FacCoeffs of binary i from its physical parameters.
__device__ void setup_binary(BinaryRec *rec, FacCoeffs *fac, const double *p, double h22_calib)
{
    const double m1 = p[0], m2 = p[1], chi1 = p[2], chi2 = p[3], f0 = p[4];
    const double Mt = m1 + m2;
    const double m1s = m1 / Mt, m2s = m2 / Mt;
    const double omega0 = f0 * (Mt * kMTSUN_SI * kPi);
    const double eta = m1s * m2s / ((m1s + m2s) * (m1s + m2s));
    const double chiS = (chi1 + chi2) / 2.0, chiA = (chi1 - chi2) / 2.0;
    const double tpl = (1.0 - 2.0 * eta) * chiS + (m1s - m2s) / (m1s + m2s) * chiA;
    fac_coeffs_build(fac, 1, m1s, m2s, eta, tpl, chiS, chiA);
    for (int l = 2; l <= kLMax; ++l)
        for (int m = 1; m <= l; ++m) {
            const int i = lm_index(l, m);
            newton_prefix(m1s, m2s, l, m, &rec->pre_re[i], &rec->pre_im[i]);
        }
    ham_coeffs_build(&rec->ham, m1s, m2s, chi1, chi2, 0.0, 0.0, 0.0, 0.0);
    ham_jets_build(rec->ham, &rec->jets);
    flux_table_build(&rec->flux, *fac, rec->pre_re, rec->pre_im, h22_calib, rec->ham.nu);
    rec->m1s = m1s;
    rec->m2s = m2s;
    rec->chi1 = chi1;
    rec->chi2 = chi2;
    rec->Mt = Mt;
    rec->omega0 = omega0;
    rec->nu = rec->ham.nu;
}

__global__ void __launch_bounds__(64) k_setup(Ws w, RunArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.B) return;
    BinaryRec *rec = &w.bins[i];
    setup_binary(rec, &w.fac[i], a.params + 5 * (size_t)i, 0.0);
    int st = 0;
    const double r_guess = pow(rec->omega0, -2.0 / 3.0);
    double x[2] = {r_guess, sqrt(r_guess)};
    const int its = ic_newton(rec->ham, rec->omega0, x, 1000, 1e-12);
    if (its < 0) st |= EOB_ST_IC_NOCONV;
    const double pr0 = ic_false_position(*rec, x[0], x[1], -3e-2, 0.0, 1000, 1e-12, a.opt.ic_mode);
    rec->y0[0] = x[0];
    rec->y0[1] = 0.0;
    rec->y0[2] = pr0;
    rec->y0[3] = x[1];
    rec->ic_iters = its;
    w.status[i] = st;
    w.rhs[i] = 0;
}

cudaError_t launch_setup(const Ws &w, const RunArgs &a, cudaStream_t s)
{
    const int bs = 64;
    k_setup<<<(a.B + bs - 1) / bs, bs, 0, s>>>(w, a);
    return cudaGetLastError();
}

}  // namespace eob
