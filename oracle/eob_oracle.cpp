// ORACLE -- test infrastructure, never part of the product path.
//
// A plain, serial C++ restatement of the reference (mikekatz04/EOBGPU)
// batched EOB waveform + likelihood path, used only by tests/, by the smoke
// check and as the CPU baseline of bench.py.  Every routine names the
// reference file:line it follows.  Pinned against the reference's own CPU
// build (oracle/_ref, see oracle/ref/build_ref.sh) through the golden fixtures
// in tests/golden/.
//
// Shared with the product: the per-binary coefficient tables
// (eobgpu_gb300/csrc/physics/{fac_coeffs,ham_coeffs}.h).  Everything evaluated
// from them here -- Hamiltonian derivatives (dual numbers), flux, RR force,
// initial conditions, DOPR853 driver and stopping rule, multipoles (own complex
// Gamma), splines, synthesis, likelihood -- is an independent serial
// implementation.
//
// Layouts follow the reference: state arg[4][n], additionalArgs[80][n]
// (m1, m2, chi1, chi2, omega, K, d5, dSO, dSS, h22_calib, 35 x (Re, Im)
// Newtonian prefixes), all doubles.
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <complex>
#include <vector>
#include <algorithm>
#include "../eobgpu_gb300/csrc/physics/fac_coeffs.h"
#include "../eobgpu_gb300/csrc/physics/ham_coeffs.h"
#include "../eobgpu_gb300/csrc/physics/imr_fits.h"
#include "oracle_dual.h"

using eob::FacCoeffs;
using eob::HamCoeffs;
using oracle::D3;
using oracle::H3;
typedef std::complex<double> cplx;

static const double PI = eob::kPi;
static const int NADD = 80;

namespace {

struct AddArgs {
    double m1, m2, chi1, chi2, omega, K, d5, dSO, dSS, h22;
    cplx prefix[eob::kNumLM];
};

AddArgs read_add(const double *add, int n, int i)
{
    AddArgs a;
    a.m1 = add[0 * n + i]; a.m2 = add[1 * n + i]; a.chi1 = add[2 * n + i]; a.chi2 = add[3 * n + i];
    a.omega = add[4 * n + i]; a.K = add[5 * n + i]; a.d5 = add[6 * n + i]; a.dSO = add[7 * n + i];
    a.dSS = add[8 * n + i]; a.h22 = add[9 * n + i];
    for (int j = 0; j < eob::kNumLM; ++j) a.prefix[j] = cplx(add[(10 + 2 * j) * n + i], add[(11 + 2 * j) * n + i]);
    return a;
}

HamCoeffs ham_of(const AddArgs &a)
{
    HamCoeffs h;
    eob::ham_coeffs_build(&h, a.m1, a.m2, a.chi1, a.chi2, a.K, a.d5, a.dSO, a.dSS);
    return h;
}

// ---- Hamiltonian and derivatives (src/EOB.cu:16-107, 139-222, 254-371) ----
double ham_H(const HamCoeffs &h, double r, double pr, double L)
{
    return eob::ham_H_from_heff<double>(h, eob::ham_heff<double>(h, r, pr, L));
}

// grad[4] = dH/d(r, phi, pr, pphi); returns H
double ham_grad(const HamCoeffs &h, double r, double pr, double L, double grad[4])
{
    const D3 heff = eob::ham_heff<D3>(h, D3::var(r, 0), D3::var(pr, 1), D3::var(L, 2));
    const double H = eob::ham_H_from_heff<double>(h, heff.v);
    const double f = h.M * h.M / (h.nu * H);  // dH = M^2 dHeff / (nu H)   (src/EOB.cu:212-215)
    grad[0] = f * heff.d[0];
    grad[1] = 0.0;
    grad[2] = f * heff.d[1];
    grad[3] = f * heff.d[2];
    return H;
}

// hess[16] row-major over (r, phi, pr, pphi), as src/EOB.cu:344-370
void ham_hessian(const HamCoeffs &h, double r, double pr, double L, double hess[16])
{
    const H3 heff = eob::ham_heff<H3>(h, H3::var(r, 0), H3::var(pr, 1), H3::var(L, 2));
    const double H = eob::ham_H_from_heff<double>(h, heff.v);
    const double M2nu = h.M * h.M / h.nu;
    const int map[4] = {0, -1, 1, 2};
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
            const int i = map[a], j = map[b];
            if (i < 0 || j < 0) { hess[4 * a + b] = 0.0; continue; }
            hess[4 * a + b] = (-(heff.g[i] * heff.g[j] / (H * H * H)) * M2nu + heff.h[i][j] / H) * M2nu;
        }
}

// ---- radiation-reaction flux (src/EOB.cu:1705-1943, 2505-2561) ----
double flux_oracle(const FacCoeffs &fc, const AddArgs &a, double nu, double r, double pphi, double omega, double Hreal,
                   double vPhiInput)
{
    double eta = nu;
    if (eta > 0.25 && eta < 0.25 + 1e-4) eta = 0.25;
    const double v = pow(omega, 1.0 / 3.0);
    const double v2 = v * v;
    double vPhi = r * pow(vPhiInput, 1.0 / 3.0);
    vPhi *= omega;
    const double vPhi2 = vPhi * vPhi;
    double flux = 0.0;
    for (int l = 2; l <= eob::kLMax; ++l) {
        for (int m = 1; m <= l; ++m) {
            const int i = eob::lm_index(l, m);
            const int eps = (l + m) % 2;
            const double eulerlog = eob::kEulerGamma + log(2.0 * m * v);
            const double ylm = fabs(eob::ylm_equator(l - eps, m));
            const cplx hN = a.prefix[i] * pow(vPhi2, (l + eps) / 2.0) * ylm;
            const double Slm = (eps == 0) ? (Hreal * Hreal - 1.0) / (2.0 * eta) + 1.0 : v * pphi;
            const double hk = Hreal * m * omega;
            const double x4 = 4.0 * PI * hk;
            double prod = 1.0;
            for (int j = 1; j <= l; ++j) prod *= 4.0 * hk * hk + (double)(j * j);
            const double Tlm = sqrt(x4 / (1.0 - exp(-x4))) / tgamma((double)(l + 1)) * sqrt(prod);
            // truncated rho_lm of the flux
            const int kmax = eob::flux_rho_maxdeg(l, m);
            double rho = 0.0;
            for (int k = kmax; k >= 1; --k) {
                const double ck = fc.rho[i][k] + (eob::flux_keeps_rhol(l, m, k) ? fc.rhol[i][k] * eulerlog : 0.0);
                rho = (rho + ck) * v;
            }
            rho += 1.0;
            if (l == 2 && m == 2) rho += a.h22 * pow(v, 12);
            double aux = 0.0;
            for (int k = 1; k <= 3; ++k)
                if (eob::flux_keeps_f(l, m, k)) aux += fc.fre[i][k] * pow(v, k);
            double rpl = pow(rho, l);
            if (eta == 0.25 && (m % 2)) rpl = aux; else rpl += aux;
            const cplx hlm = Tlm * Slm * rpl * hN;
            flux += (double)(m * m) * omega * omega * std::norm(hlm);
        }
    }
    (void)v2;
    return flux / PI / 8.0;
}

// RR force (src/EOB.cu:2563-2642). omega is the value in the omega slot of
// additionalArgs at the time of the call.
void rr_force(const HamCoeffs &h, const FacCoeffs &fc, const AddArgs &a, double r, double pr, double L, double omega,
              double *Fr, double *Fphi)
{
    double g0[4];
    ham_grad(h, r, 0.0, L, g0);
    const double omega_circ = g0[3];
    const double vPhi = 1.0 / (omega_circ * omega_circ * r * r * r);
    const double nu = h.nu;
    const double Hval = nu * ham_H(h, r, pr, L);
    double flux = flux_oracle(fc, a, nu, r, L, omega, Hval, vPhi);
    flux /= nu;
    const double fo = flux / omega;
    *Fr = -pr / L * fo;
    *Fphi = -fo;
}

// ODE right-hand side (src/EOB.cu:3046-3145)
void rhs(const HamCoeffs &h, const FacCoeffs &fc, const AddArgs &a, const double y[4], double k[4])
{
    double g[4];
    ham_grad(h, y[0], y[2], y[3], g);
    double Fr, Fphi;
    rr_force(h, fc, a, y[0], y[2], y[3], g[3], &Fr, &Fphi);
    k[0] = g[2];
    k[1] = g[3];
    k[2] = -g[0] + Fr;
    k[3] = -g[1] + Fphi;
}

// ---- complex Gamma: Stirling series for log Gamma after an upward shift
// (Abramowitz & Stegun 6.1.40 and the recurrence 6.1.15); exp() of the
// series makes the branch of the logarithm irrelevant.
cplx cgamma(cplx z)
{
    cplx shift = 1.0;
    while (z.real() < 30.0) { shift *= z; z += 1.0; }
    // B_2k / (2k (2k-1)) for k = 1..8
    static const double c[8] = {1.0 / 12.0, -1.0 / 360.0, 1.0 / 1260.0, -1.0 / 1680.0,
                                1.0 / 1188.0, -691.0 / 360360.0, 1.0 / 156.0, -3617.0 / 122400.0};
    const cplx iz = 1.0 / z, iz2 = iz * iz;
    cplx s = c[7];
    for (int k = 6; k >= 0; --k) s = s * iz2 + c[k];
    s *= iz;
    const cplx lg = (z - 0.5) * std::log(z) - z + 0.5 * ::log(2.0 * PI) + s;
    return std::exp(lg) / shift;
}

// ---- waveform multipole on the trajectory (src/EOB.cu:1235-1613) ----
cplx waveform_mode(const FacCoeffs &fc, double r, double phi, double pphi, double v, double Hreal, int l, int m,
                   cplx prefix, double eta, double vPhiInput, double h22_calib)
{
    if (eta > 0.25 && eta < 0.25 + 1e-4) eta = 0.25;
    const int i = eob::lm_index(l, m);
    const double v2 = v * v;
    const double Omega = v2 * v;
    const double vh3 = Hreal * Omega;
    const double vh = pow(vh3, 1.0 / 3.0);
    const double eulerlog = eob::kEulerGamma + log(2.0 * m * v);
    double vPhi = r * pow(vPhiInput, 1.0 / 3.0);
    vPhi *= Omega;
    const double vPhi2 = vPhi * vPhi;
    const int eps = (l + m) % 2;
    // Y_{l-eps}^{-m}(pi/2, phi) = (-1)^m Y_{l-eps}^{m}(pi/2, 0) e^{-i m phi}
    const double y0 = ((m % 2) ? -1.0 : 1.0) * eob::ylm_equator(l - eps, m);
    const cplx ylm = y0 * std::exp(cplx(0.0, -m * phi));
    const cplx hN = prefix * pow(vPhi2, (l + eps) / 2.0) * ylm;
    const double Slm = (eps == 0) ? (Hreal * Hreal - 1.0) / (2.0 * eta) + 1.0 : v * pphi;
    const double k = m * Omega;
    const double hk = Hreal * k;
    const cplx T = std::exp(cplx(PI * hk, 2.0 * hk * log(4.0 * k / sqrt(M_E)))) *
                   cgamma(cplx(l + 1.0, -2.0 * hk)) / tgamma((double)(l + 1));
    double delta = 0.0, vhp = 1.0, vp = 1.0;
    for (int kk = 1; kk < 10; ++kk) { vhp *= vh; delta += fc.dvh[i][kk] * vhp; }
    for (int kk = 1; kk < 9; ++kk) { vp *= v; delta += fc.dv[i][kk] * vp; }
    double rho = 0.0;
    for (int kk = eob::kRhoDeg; kk >= 1; --kk) rho = (rho + fc.rho[i][kk] + fc.rhol[i][kk] * eulerlog) * v;
    rho += 1.0;
    if (l == 2 && m == 2) rho += h22_calib * pow(v, 12);
    cplx aux = 0.0;
    vp = 1.0;
    for (int kk = 1; kk < 8; ++kk) { vp *= v; aux += fc.fre[i][kk] * vp; }
    aux += cplx(0.0, fc.fim_vh6[i] * vh3 * vh3);
    cplx rpl = pow(rho, l);
    if (eta == 0.25 && (m % 2)) rpl = aux; else rpl += aux;
    cplx hlm = T * std::exp(cplx(0.0, delta)) * Slm * rpl;
    return hlm * hN;
}

// ---- initial conditions (src/EOB.cu:404-431, 2864-3041; 2665-2838) ----
void ic_cons(const HamCoeffs &h, double omega0, double r, double pphi, double res[2])
{
    double g[4];
    ham_grad(h, r, 0.0, pphi, g);
    res[0] = g[3] - omega0;
    res[1] = g[0];
}

// discrete Newton on (r, pphi); returns the number of iterations used
int root_find_cons(const HamCoeffs &h, double omega0, double x[2], int max_iter, double err)
{
    const double sq_eps = sqrt(2.22e-16);
    double x0[2] = {x[0], x[1]}, x1[2];
    for (int it = 0; it < max_iter; ++it) {
        x1[0] = x0[0]; x1[1] = x0[1];
        double r1[2], r2[2], J[2][2];
        ic_cons(h, omega0, x1[0], x1[1], r1);
        for (int kk = 0; kk < 2; ++kk)
            for (int j = 0; j < 2; ++j) {
                const double dj = sq_eps * fabs(x1[j]);
                double xt[2] = {x1[0], x1[1]};
                xt[j] += dj;
                ic_cons(h, omega0, xt[0], xt[1], r2);
                J[kk][j] = (r2[kk] - r1[kk]) / dj;
            }
        const double det = 1.0 / (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
        const double inv[2][2] = {{det * J[1][1], det * -J[0][1]}, {det * -J[1][0], det * J[0][0]}};
        for (int kk = 0; kk < 2; ++kk) {
            double t = 0.0;
            for (int j = 0; j < 2; ++j) t += inv[kk][j] * r1[j];
            x1[kk] -= t;
        }
        double rel = 0.0;
        for (int j = 0; j < 2; ++j) {
            const double d = fabs(x1[j] - x0[j]) / x0[j];
            if (d > rel) rel = d;
        }
        x0[0] = x1[0]; x0[1] = x1[1];
        if (rel < err) { x[0] = x1[0]; x[1] = x1[1]; return it + 1; }
    }
    x[0] = x1[0]; x[1] = x1[1];
    return max_iter;
}

// Dissipative initial-condition residual rdot(F) - dH/dpr (src/EOB.cu:2665-2689).
// physical = 0 reproduces what the reference evaluates: its d2H/dr2
// (src/EOB.cu:322, 344) exceeds the true value by more than 1e6 over the whole
// parameter space, so its rdot term is below the solver tolerance and the root
// is p_r0 = 0 to within 1e-12.  physical = 1 uses the exact Hessian.
double ic_diss(const HamCoeffs &h, const FacCoeffs &fc, const AddArgs &a, double r, double pr, double L, int physical)
{
    double g[4], hs[16];
    ham_grad(h, r, pr, L, g);
    if (!physical) return -g[2];
    ham_hessian(h, r, pr, L, hs);
    double Fr, Fphi;
    rr_force(h, fc, a, r, pr, L, g[3], &Fr, &Fphi);
    const double dLdr = -hs[0] / hs[12];
    const double rdot = Fphi / dLdr;
    return rdot - g[2];
}

double root_find_diss(const HamCoeffs &h, const FacCoeffs &fc, const AddArgs &a, double r, double L, double lo,
                      double hi, int max_iter, double err, int *iters, int physical)
{
    double A = lo, B = hi;
    double fa = ic_diss(h, fc, a, r, A, L, physical), fb = ic_diss(h, fc, a, r, B, L, physical);
    if (fb == fa) { if (iters) *iters = 0; return (fb == 0.0) ? B : A; }
    double c = 0.0;
    int it = 0;
    while (it < max_iter) {
        c = (A * fb - B * fa) / (fb - fa);
        const double fcv = ic_diss(h, fc, a, r, c, L, physical);
        if ((fb < 0.0 && fcv < 0.0) || (fb >= 0.0 && fcv >= 0.0)) { B = c; fb = fcv; }
        else { A = c; fa = fcv; }
        it += 1;
        if (it > max_iter || fabs(fcv) < err) break;
    }
    if (iters) *iters = it;
    return c;
}

// ---- DOPR853 (src/DOPR853.cu:6-192 tableau; 357-517 stages; 537-618 error;
// 674-762 controller) driven as eob/new_Dormand_horiz.py:424-778 for one binary.
namespace dp {
const double c[13] = {0.0, 0.0, 0.526001519587677318785587544488e-01, 0.789002279381515978178381316732e-01,
                      0.118350341907227396726757197510e+00, 0.281649658092772603273242802490e+00,
                      0.333333333333333333333333333333e+00, 0.25e+00, 0.307692307692307692307692307692e+00,
                      0.651282051282051282051282051282e+00, 0.6e+00, 0.857142857142857142857142857142e+00, 1.0};
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
// a[s][j]: stage s (1..12) weights on the stored slopes j in the reference's
// accumulation order (slot numbering k1..k10; stage 11 writes k2, stage 12 k3)
struct Term { int slot; double a; };
const Term st2[] = {{1, 5.26001519587677318785587544488e-2}};
const Term st3[] = {{1, 1.97250569845378994544595329183e-2}, {2, 5.91751709536136983633785987549e-2}};
const Term st4[] = {{1, 2.95875854768068491816892993775e-2}, {3, 8.87627564304205475450678981324e-2}};
const Term st5[] = {{1, 2.41365134159266685502369798665e-1}, {3, -8.84549479328286085344864962717e-1},
                    {4, 9.24834003261792003115737966543e-1}};
const Term st6[] = {{1, 3.7037037037037037037037037037e-2}, {4, 1.70828608729473871279604482173e-1},
                    {5, 1.25467687566822425016691814123e-1}};
const Term st7[] = {{1, 3.7109375e-2}, {4, 1.70252211019544039314978060272e-1},
                    {5, 6.02165389804559606850219397283e-2}, {6, -1.7578125e-2}};
const Term st8[] = {{1, 3.70920001185047927108779319836e-2}, {4, 1.70383925712239993810214054705e-1},
                    {5, 1.07262030446373284651809199168e-1}, {6, -1.53194377486244017527936158236e-2},
                    {7, 8.27378916381402288758473766002e-3}};
const Term st9[] = {{1, 6.24110958716075717114429577812e-1}, {4, -3.36089262944694129406857109825e0},
                    {5, -8.68219346841726006818189891453e-1}, {6, 2.75920996994467083049415600797e1},
                    {7, 2.01540675504778934086186788979e1}, {8, -4.34898841810699588477366255144e1}};
const Term st10[] = {{1, 4.77662536438264365890433908527e-1}, {4, -2.48811461997166764192642586468e0},
                     {5, -5.90290826836842996371446475743e-1}, {6, 2.12300514481811942347288949897e1},
                     {7, 1.52792336328824235832596922938e1}, {8, -3.32882109689848629194453265587e1},
                     {9, -2.03312017085086261358222928593e-2}};
const Term st11[] = {{1, -9.3714243008598732571704021658e-1}, {4, 5.18637242884406370830023853209e0},
                     {5, 1.09143734899672957818500254654e0}, {6, -8.14978701074692612513997267357e0},
                     {7, -1.85200656599969598641566180701e1}, {8, 2.27394870993505042818970056734e1},
                     {9, 2.49360555267965238987089396762e0}, {10, -3.0467644718982195003823669022e0}};
const Term st12[] = {{1, 2.27331014751653820792359768449e0}, {4, -1.05344954667372501984066689879e1},
                     {5, -2.00087205822486249909675718444e0}, {6, -1.79589318631187989172765950534e1},
                     {7, 2.79488845294199600508499808837e1}, {8, -2.85899827713502369474065508674e0},
                     {9, -8.87285693353062954433549289258e0}, {10, 1.23605671757943030647266201528e1},
                     {2, 6.43392746015763530355970484046e-1}};
const Term *const stages[13] = {nullptr, nullptr, st2, st3, st4, st5, st6, st7, st8, st9, st10, st11, st12};
const int nterms[13] = {0, 0, 1, 2, 2, 3, 3, 4, 5, 6, 7, 8, 9};
const int out_slot[13] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 2, 3};
const double safe = 0.9, alpha = 1.0 / 8.0, minscale = 1.0 / 3.0, maxscale = 6.0;
}  // namespace dp

struct Binary {
    HamCoeffs h;
    FacCoeffs fc;
    AddArgs a;
};

// 12 stages; k[slot][4], slots 1..10
void dopr_stages(const Binary &b, const double y[4], double hstep, double k[11][4])
{
    for (int s = 1; s <= 12; ++s) {
        double arg[4];
        for (int q = 0; q < 4; ++q) {
            double ak = 0.0;
            for (int t = 0; t < dp::nterms[s]; ++t) ak += dp::stages[s][t].a * k[dp::stages[s][t].slot][q];
            arg[q] = y[q] + hstep * ak;
        }
        rhs(b.h, b.fc, b.a, arg, k[dp::out_slot[s]]);
    }
}

double dopr_error(const double y[4], double hstep, double k[11][4], double ynew[4], double rtol, double atol)
{
    double err = 0.0, err2 = 0.0;
    for (int q = 0; q < 4; ++q) {
        const double t = dp::b1 * k[1][q] + dp::b6 * k[6][q] + dp::b7 * k[7][q] + dp::b8 * k[8][q] + dp::b9 * k[9][q] +
                         dp::b10 * k[10][q] + dp::b11 * k[2][q] + dp::b12 * k[3][q];
        ynew[q] = y[q] + hstep * t;
        const double mx = (y[q] > ynew[q]) ? y[q] : ynew[q];
        const double sk = 1.0 / (atol + rtol * mx);
        err2 += pow((t - dp::bhh1 * k[1][q] - dp::bhh2 * k[9][q] - dp::bhh3 * k[3][q]) * sk, 4);
        err += pow((dp::er1 * k[1][q] + dp::er6 * k[6][q] + dp::er7 * k[7][q] + dp::er8 * k[8][q] + dp::er9 * k[9][q] +
                    dp::er10 * k[10][q] + dp::er11 * k[2][q] + dp::er12 * k[3][q]) * sk, 4);
    }
    double denom = err + 0.01 * err2;
    denom = (denom < 0.0) ? 1.0 : denom;
    const double e = fabs(hstep) * err * sqrt(1.0 / (4.0 * denom));
    // a NaN estimate (a trial stage outside the Hamiltonian's domain) counts
    // as +inf, a rejection with the smallest scale, as in the CUDA path; the
    // reference's controller would carry the NaN into h
    return (e != e) ? INFINITY : e;
}

// returns accept flag; updates h, errOld, prevReject
bool dopr_controller(double err, double *errOld, bool *prevReject, double *h)
{
    if (err <= 1.0) {
        double scale;
        if (err == 0.0) scale = dp::maxscale;
        else {
            scale = dp::safe * pow(err, -dp::alpha) * pow(*errOld, 0.0);
            if (scale > dp::maxscale) scale = dp::maxscale;
            else if (scale < dp::minscale) scale = dp::minscale;
        }
        if (*prevReject && scale > 1.0) scale = 1.0;
        *h = *h * scale;
        if (err < 1e-4) err = 1e-4; else if (err > 1e300) err = 1e300;
        *errOld = err;
        *prevReject = false;
        return true;
    }
    *prevReject = true;
    double t = dp::safe * pow(err, -dp::alpha);
    if (t < dp::minscale) t = dp::minscale; else if (t > 1e300) t = 1e300;
    *h = *h * t;
    return false;
}

struct Dense {
    std::vector<double> t;      // [max_step]
    std::vector<double> y;      // [max_step][4]
};

// Stopping rule of eob/seobnrv4phm.py:82-150 for one binary (the single-binary
// reading of its batched indexing). omegas: history row per step.
int stop_code(const Binary &b, const double y[4], int step, std::vector<double> &omegas)
{
    double k[4];
    rhs(b.h, b.fc, b.a, y, k);
    const double r = y[0], drdt = k[0], omega = k[1], dprdt = k[2];
    int stop = 0;
    if (r < 1.0) stop = 2;
    else if (r < 6.0 && drdt > 0.0) stop = 3;
    else if (r < 6.0 && dprdt > 0.0) stop = 4;
    else if (step > 5) {
        const bool c1 = r < 6.0;
        const bool c2 = omega < omegas[step - 1];
        bool c3 = true;
        for (int j = step - 4; j < step - 1; ++j) c3 = c3 && (omegas[j + 1] - omegas[j] < 0.0);
        if (c1 && c2 && c3) stop = 5;
    }
    omegas[step] = omega;
    return stop;
}

// One integrate() call for one binary (eob/new_Dormand_horiz.py:424-778).
// Returns the final step_num; *status gets the stop code of the last step.
int integrate(const Binary &b, Dense &d, int step_num, double hInit, bool fix_step, int max_step, double tmax,
              double rtol, double atol, int *stop_out)
{
    double x = d.t[step_num];
    double y[4];
    for (int q = 0; q < 4; ++q) y[q] = d.y[4 * step_num + q];
    double h = hInit, hfix = hInit, errOld = 1e-4;
    bool prevReject = false;
    bool stop = true;  // reference initialises its stop flags to True
    int stop_info = 0;
    std::vector<double> omegas((size_t)max_step, 0.0);
    double k[11][4];
    long long tries = 0;  // attempt limit of the CUDA path (2 max_step + 100): every loop ends
    for (;;) {
        dopr_stages(b, y, h, k);
        double ynew[4];
        const double err = dopr_error(y, h, k, ynew, rtol, atol);
        const double hOld = h;
        const bool ok = dopr_controller(err, &errOld, &prevReject, &h);
        if (fix_step && !ok) hfix /= 2.0;
        if (fix_step) h = hfix;
        if (ok) {
            for (int q = 0; q < 4; ++q) y[q] = ynew[q];
            x = x + hOld;
            step_num += 1;
            for (int q = 0; q < 4; ++q) d.y[4 * step_num + q] = y[q];
            d.t[step_num] = x;
            stop_info = stop_code(b, y, step_num, omegas);
            stop = stop_info != 0;
        }
        if (x >= tmax || step_num >= max_step - 1 || stop || ++tries >= 2LL * max_step + 100) break;
    }
    if (stop_out) *stop_out = stop_info;
    return step_num;
}

void build_binary(Binary &b, double m1s, double m2s, double chi1, double chi2, double omega0, int use_hm)
{
    const double eta = m1s * m2s / ((m1s + m2s) * (m1s + m2s));
    const double chiS = 0.5 * (chi1 + chi2), chiA = 0.5 * (chi1 - chi2);
    const double tplspin = (1.0 - 2.0 * eta) * chiS + (m1s - m2s) / (m1s + m2s) * chiA;
    eob::fac_coeffs_build(&b.fc, use_hm, m1s, m2s, eta, tplspin, chiS, chiA);
    b.a.m1 = m1s; b.a.m2 = m2s; b.a.chi1 = chi1; b.a.chi2 = chi2; b.a.omega = omega0;
    b.a.K = 0.0; b.a.d5 = 0.0; b.a.dSO = 0.0; b.a.dSS = 0.0; b.a.h22 = 0.0;
    for (int l = 2; l <= eob::kLMax; ++l)
        for (int m = 1; m <= l; ++m) {
            double re, im;
            eob::newton_prefix(m1s, m2s, l, m, &re, &im);
            b.a.prefix[eob::lm_index(l, m)] = cplx(re, im);
        }
    b.h = ham_of(b.a);
}

// ---- splines (src/interpolate.cu:10-267), one interpolant of n knots ----
void spline_build(const double *x, const double *y, int n, double *c1, double *c2, double *c3)
{
    std::vector<double> B(n), ud(n), dg(n), ld(n);
    for (int i = 0; i < n; ++i) {
        int i0, i1, i2;
        if (i == n - 1) { i0 = n - 3; i1 = n - 2; i2 = n - 1; }
        else if (i == 0) { i0 = 0; i1 = 1; i2 = 2; }
        else { i0 = i - 1; i1 = i; i2 = i + 1; }
        const double dx1 = x[i1] - x[i0], dx2 = x[i2] - x[i1], dd = x[i2] - x[i0];
        const double s1 = (y[i1] - y[i0]) / dx1, s2 = (y[i2] - y[i1]) / dx2;
        if (i == n - 1) { B[i] = (dx2 * dx2 * s1 + (2 * dd + dx2) * dx1 * s2) / dd; dg[i] = dx1; ld[i] = dd; ud[i] = 0.0; }
        else if (i == 0) { B[i] = ((dx1 + 2 * dd) * dx2 * s1 + dx1 * dx1 * s2) / dd; ud[i] = dd; ld[i] = 0.0; dg[i] = dx2; }
        else { B[i] = 3.0 * (dx2 * s1 + dx1 * s2); dg[i] = 2 * (dx1 + dx2); ud[i] = dx1; ld[i] = dx2; }
    }
    for (int i = 1; i < n; ++i) {
        const double w = ld[i] / dg[i - 1];
        dg[i] = dg[i] - w * ud[i - 1];
        B[i] = B[i] - w * B[i - 1];
    }
    B[n - 1] = B[n - 1] / dg[n - 1];
    for (int i = n - 2; i >= 0; --i) B[i] = (B[i] - ud[i] * B[i + 1]) / dg[i];
    for (int i = 0; i < n - 1; ++i) {
        const double dx = x[i + 1] - x[i];
        const double slope = (y[i + 1] - y[i]) / dx;
        const double t = (B[i] + B[i + 1] - 2 * slope) / dx;
        c1[i] = B[i];
        c2[i] = (slope - B[i]) / dx - t;
        c3[i] = t / dx;
    }
    // row n-1 keeps the tridiagonal entries in the reference (its c1/c2/c3
    // alias ud/diag/ld); only x = 0 is ever evaluated there.
    c1[n - 1] = ud[n - 1]; c2[n - 1] = dg[n - 1]; c3[n - 1] = ld[n - 1];
}

// interval index as CubicSplineInterpolantTD._get_inds (eob/seobnrv4phm.py:221-260)
int spline_index(const double *x, int n, double tnew)
{
    int i = (int)(std::upper_bound(x, x + n, tnew) - x) - 1;
    if (i == n) i -= 1;
    if (i < 0) i = 0;
    return i;
}

}  // namespace

// ============================================================================
extern "C" {

int oracle_nadd(void) { return NADD; }

// src/EOB.cu:127 evaluate_Ham_align_AD_wrap
void oracle_evaluate_H(double *out, const double *r, const double *phi, const double *pr, const double *pphi,
                       const double *m1, const double *m2, const double *chi1, const double *chi2, double K, double d5,
                       double dSO, double dSS, int n)
{
    (void)phi;
    for (int i = 0; i < n; ++i) {
        HamCoeffs h;
        eob::ham_coeffs_build(&h, m1[i], m2[i], chi1[i], chi2[i], K, d5, dSO, dSS);
        out[i] = ham_H(h, r[i], pr[i], pphi[i]);
    }
}

// src/EOB.cu:242 grad_Ham_align_AD_wrap
void oracle_grad_H(const double *arg, double *grad, const double *add, int n)
{
    for (int i = 0; i < n; ++i) {
        const HamCoeffs h = ham_of(read_add(add, n, i));
        double g[4];
        ham_grad(h, arg[i], arg[2 * n + i], arg[3 * n + i], g);
        for (int q = 0; q < 4; ++q) grad[q * n + i] = g[q];
    }
}

// src/EOB.cu:391 hessian_Ham_align_AD_wrap
void oracle_hessian_H(const double *arg, double *hess, const double *add, int n)
{
    for (int i = 0; i < n; ++i) {
        const HamCoeffs h = ham_of(read_add(add, n, i));
        double hs[16];
        ham_hessian(h, arg[i], arg[2 * n + i], arg[3 * n + i], hs);
        for (int q = 0; q < 16; ++q) hess[q * n + i] = hs[q];
    }
}

// Per-binary coefficient context: the SEOBNRv5 class of src/EOB.cu:3343-3383.
struct OracleCtx { int n; std::vector<FacCoeffs> fc; };

void *oracle_ctx_create(const double *m1, const double *m2, const double *eta, const double *tplspin,
                        const double *chiS, const double *chiA, int use_hm, int n)
{
    OracleCtx *c = new OracleCtx();
    c->n = n;
    c->fc.resize((size_t)n);
    for (int i = 0; i < n; ++i) eob::fac_coeffs_build(&c->fc[i], use_hm, m1[i], m2[i], eta[i], tplspin[i], chiS[i], chiA[i]);
    return c;
}
void oracle_ctx_destroy(void *p) { delete (OracleCtx *)p; }

// dense coefficient table of binary i: rho, rhol, fre, fim_vh6, dvh, dv (see FacCoeffs)
int oracle_fac_ndouble(void) { return (int)(sizeof(FacCoeffs) / sizeof(double)); }
void oracle_ctx_coeffs(void *p, int i, double *out) { memcpy(out, &((OracleCtx *)p)->fc[i], sizeof(FacCoeffs)); }

// src/EOB.cu:3486 ODE_Ham_align_AD_wrap (idx: coefficient row per system)
void oracle_ctx_ode(void *p, const double *arg, double *k, const double *add, int n, const int *idx)
{
    OracleCtx *c = (OracleCtx *)p;
    for (int i = 0; i < n; ++i) {
        const AddArgs a = read_add(add, n, i);
        const HamCoeffs h = ham_of(a);
        const double y[4] = {arg[i], arg[n + i], arg[2 * n + i], arg[3 * n + i]};
        double kk[4];
        rhs(h, c->fc[idx[i]], a, y, kk);
        for (int q = 0; q < 4; ++q) k[q * n + i] = kk[q];
    }
}

// src/EOB.cu:3385 RR_force_wrap
void oracle_ctx_rr_force(void *p, double *force, const double *arg, const double *add, int n, const int *idx)
{
    OracleCtx *c = (OracleCtx *)p;
    for (int i = 0; i < n; ++i) {
        const AddArgs a = read_add(add, n, i);
        const HamCoeffs h = ham_of(a);
        double Fr, Fphi;
        rr_force(h, c->fc[idx[i]], a, arg[i], arg[2 * n + i], arg[3 * n + i], a.omega, &Fr, &Fphi);
        force[i] = Fr;
        force[n + i] = Fphi;
    }
}

// src/EOB.cu:3423 EOBGetSpinFactorizedWaveform_wrap; out/prefix interleaved (re, im)
void oracle_ctx_waveform(void *p, double *out, const double *r, const double *phi, const double *pr,
                         const double *pphi, const double *v, const double *Hreal, const double *eta,
                         const double *vPhi, int l, int m, const double *prefix, double h22_calib, int numSys,
                         int traj_length, const int *idx)
{
    (void)pr;
    OracleCtx *c = (OracleCtx *)p;
    for (int b = 0; b < numSys; ++b)
        for (int i = 0; i < traj_length; ++i) {
            const int j = b * traj_length + i;
            const cplx hl = waveform_mode(c->fc[idx[b]], r[j], phi[j], pphi[j], v[j], Hreal[j], l, m,
                                          cplx(prefix[2 * b], prefix[2 * b + 1]), eta[b], vPhi[j], h22_calib);
            out[2 * j] = hl.real();
            out[2 * j + 1] = hl.imag();
        }
}

// src/EOB.cu:3033 root_find_all_wrap (n = 2 unknowns: r, pphi)
void oracle_root_find_all(double *xOut, const double *x0In, const double *add, int max_iter, double err, int numBinAll)
{
    for (int i = 0; i < numBinAll; ++i) {
        const AddArgs a = read_add(add, numBinAll, i);
        const HamCoeffs h = ham_of(a);
        double x[2] = {x0In[i], x0In[numBinAll + i]};
        root_find_cons(h, a.omega, x, max_iter, err);
        xOut[i] = x[0];
        xOut[numBinAll + i] = x[1];
    }
}

// src/EOB.cu:3398 root_find_scalar_all_wrap
void oracle_ctx_root_find_scalar_all(void *p, double *pr_res, const double *bounds, const double *argsIn,
                                     const double *add, int max_iter, double err, int numBinAll, int physical)
{
    OracleCtx *c = (OracleCtx *)p;
    for (int i = 0; i < numBinAll; ++i) {
        const AddArgs a = read_add(add, numBinAll, i);
        const HamCoeffs h = ham_of(a);
        pr_res[i] = root_find_diss(h, c->fc[i], a, argsIn[i], argsIn[3 * numBinAll + i], bounds[i],
                                   bounds[numBinAll + i], max_iter, err, nullptr, physical);
    }
}

// src/interpolate.cu:269 interpolate_TD: x[L][B], y[L][nsubs][B]; c1/c2/c3 like y
void oracle_interpolate_td(const double *t, const double *y, double *c1, double *c2, double *c3, const int *lengths,
                           int numBinAll, int nsubs, int Lmax)
{
    const int ninterp = numBinAll * nsubs;
    std::vector<double> xs(Lmax), ys(Lmax), a1(Lmax), a2(Lmax), a3(Lmax);
    for (int ip = 0; ip < ninterp; ++ip) {
        const int b = ip % numBinAll;
        const int n = lengths[b];
        for (int i = 0; i < n; ++i) { xs[i] = t[i * numBinAll + b]; ys[i] = y[i * ninterp + ip]; }
        spline_build(xs.data(), ys.data(), n, a1.data(), a2.data(), a3.data());
        for (int i = 0; i < n; ++i) { c1[i * ninterp + ip] = a1[i]; c2[i * ninterp + ip] = a2[i]; c3[i * ninterp + ip] = a3[i]; }
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Whole path for one binary: the pieces shared by the free-running and replayed runs.
namespace {

// multipoles on the trajectory (eob/seobnrv4phm.py:2138-2221): hl[j * L + i]
std::vector<cplx> modes_on_trajectory(const Binary &b, const Dense &d, int L, const int *ls, const int *ms, int K)
{
    const double nu = b.h.nu;
    std::vector<cplx> hl((size_t)K * L);
    for (int i = 0; i < L; ++i) {
        const double r = d.y[4 * i], ph = d.y[4 * i + 1], pr = d.y[4 * i + 2], L_ = d.y[4 * i + 3];
        double g[4], g0[4];
        ham_grad(b.h, r, pr, L_, g);
        ham_grad(b.h, r, 0.0, L_, g0);
        const double omega = g[3], omega_c = g0[3];
        const double vPhi = 1.0 / (omega_c * omega_c * r * r * r);
        const double Hval = nu * ham_H(b.h, r, pr, L_);
        const double v = pow(omega, 1.0 / 3.0);
        for (int j = 0; j < K; ++j)
            hl[(size_t)j * L + i] = waveform_mode(b.fc, r, ph, L_, v, Hval, ls[j], ms[j],
                                                  b.a.prefix[eob::lm_index(ls[j], ms[j])], nu, vPhi, 0.0);
    }
    return hl;
}

double post_trajectory(const Binary &b, const Dense &d, int L, double Mt, double dt, int N, const int *ls,
                       const int *ms, int K, const double *data, double amp, int *npts, double *h_out)
{
    const std::vector<cplx> hl = modes_on_trajectory(b, d, L, ls, ms, K);
    // synthesis on the uniform grid (eob/seobnrv4phm.py:2310-2372)
    const double Mts = Mt * eob::kMTSUN_SI;
    const double dT = dt / Mts;
    std::vector<double> tin(L), phv(L), c1(L), c2(L), c3(L);
    for (int i = 0; i < L; ++i) { tin[i] = (d.t[i] * Mt * eob::kMTSUN_SI) / Mts; phv[i] = d.y[4 * i + 1]; }
    spline_build(tin.data(), phv.data(), L, c1.data(), c2.data(), c3.data());
    const int np = (int)((tin[L - 1] - tin[0]) / dT) + 1;
    if (npts) *npts = np;
    const int nuse = std::min(np, N);
    std::vector<double> tk(nuse), phik(nuse);
    std::vector<int> ik(nuse);
    for (int k = 0; k < nuse; ++k) {
        double t = k * dT + tin[0];
        if (t > tin[L - 1]) t = tin[L - 1];
        tk[k] = t;
        const int i = spline_index(tin.data(), L, t);
        ik[k] = i;
        const double xx = t - tin[i], x2 = xx * xx, x3 = x2 * xx;
        phik[k] = phv[i] + c1[i] * xx + c2[i] * x2 + c3[i] * x3;
    }
    std::vector<cplx> hsum(nuse, cplx(0.0, 0.0));
    std::vector<double> yr(L), yi(L), r1(L), r2(L), r3(L), i1(L), i2(L), i3(L);
    for (int j = 0; j < K; ++j) {
        const int m = ms[j];
        for (int i = 0; i < L; ++i) {
            const cplx z = hl[(size_t)j * L + i] * std::exp(cplx(0.0, m * phv[i]));
            yr[i] = z.real(); yi[i] = z.imag();
        }
        spline_build(tin.data(), yr.data(), L, r1.data(), r2.data(), r3.data());
        spline_build(tin.data(), yi.data(), L, i1.data(), i2.data(), i3.data());
        for (int k = 0; k < nuse; ++k) {
            const int i = ik[k];
            const double xx = tk[k] - tin[i], x2 = xx * xx, x3 = x2 * xx;
            const double re = yr[i] + r1[i] * xx + r2[i] * x2 + r3[i] * x3;
            const double im = yi[i] + i1[i] * xx + i2[i] * x2 + i3[i] * x3;
            hsum[k] += cplx(re, im) * std::exp(cplx(0.0, -m * phik[k]));
        }
    }
    // white-noise likelihood: h_k = A Re sum_lm h_lm(t_k) for k < npts, 0 beyond
    double lnl = 0.0;
    for (int k = 0; k < N; ++k) {
        const double hk = (k < nuse) ? amp * hsum[k].real() : 0.0;
        const double rr = data[k] - hk;
        lnl += rr * rr;
    }
    if (h_out)
        for (int k = 0; k < N; ++k) {
            h_out[2 * k] = (k < nuse) ? hsum[k].real() : 0.0;
            h_out[2 * k + 1] = (k < nuse) ? hsum[k].imag() : 0.0;
        }
    return -0.5 * lnl;
}

// the two adaptive passes of run_trajectory (eob/seobnrv4phm.py:2072-2136); returns the row count
int free_trajectory(const Binary &b, Dense &d, int max_step, double rtol, double atol, double h_init, int *status)
{
    const double tmax = 1e7 * 1e6;
    int stopc = 0;
    int S = integrate(b, d, 0, h_init, false, max_step, tmax, rtol, atol, &stopc);
    if (S < 2 || S >= max_step - 1) { *status = 1; }
    const double t_stop = d.t[(S >= 1) ? S - 1 : 0];
    const double t_des = t_stop - 10.0;
    int idx = 0;
    double best = fabs(d.t[0] - t_des);
    for (int i = 1; i < max_step; ++i) {
        const double dd = fabs(d.t[i] - t_des);
        if (dd < best) { best = dd; idx = i; }
    }
    if (idx < 1) { *status = 1; idx = 1; }
    for (int i = idx; i < max_step; ++i) { d.t[i] = 0.0; for (int q = 0; q < 4; ++q) d.y[4 * i + q] = 0.0; }
    S = integrate(b, d, idx - 1, 0.05, true, max_step, tmax, rtol, atol, &stopc);
    return S + 1;
}

// one always-accepted DOPR853 step per pair of consecutive given knots
int replay_trajectory(const Binary &b, Dense &d, const double *knots, int L, double rtol, double atol, int *status)
{
    double k[11][4];
    for (int i = 1; i < L; ++i) {
        const double hstep = knots[i] - knots[i - 1];
        if (!(hstep > 0.0)) { *status = 1; return i; }
        double y[4], ynew[4];
        for (int q = 0; q < 4; ++q) y[q] = d.y[4 * (i - 1) + q];
        dopr_stages(b, y, hstep, k);
        dopr_error(y, hstep, k, ynew, rtol, atol);
        for (int q = 0; q < 4; ++q) d.y[4 * i + q] = ynew[q];
        d.t[i] = knots[i];
    }
    return L;
}

}  // namespace

namespace {
// IC (eob/seobnrv4phm.py:1966-2070) and the trajectory, free-running or on
// given knots; returns the row count (status 1 on failure)
int trajectory_ex(const double *params, int max_step, double rtol, double atol, double h_init, const double *replay_t,
                  int replay_L, Binary &b, Dense &d, double *ic, int *status)
{
    *status = 0;
    const double m1 = params[0], m2 = params[1], chi1 = params[2], chi2 = params[3], f0 = params[4];
    const double Mt = m1 + m2;
    const double m1s = m1 / Mt, m2s = m2 / Mt;
    const double omega0 = f0 * (Mt * eob::kMTSUN_SI * PI);
    build_binary(b, m1s, m2s, chi1, chi2, omega0, 1);
    const double r_guess = pow(omega0, -2.0 / 3.0);
    double x[2] = {r_guess, sqrt(r_guess)};
    root_find_cons(b.h, omega0, x, 1000, 1e-12);
    const double r0 = x[0], pphi0 = x[1];
    const double pr0 = root_find_diss(b.h, b.fc, b.a, r0, pphi0, -3e-2, 0.0, 1000, 1e-12, nullptr, 0);
    if (ic) { ic[0] = r0; ic[1] = pphi0; ic[2] = pr0; }
    if (replay_t && (replay_L < 2 || replay_L > max_step)) { *status = 1; return 0; }
    d.t.assign((size_t)max_step, 0.0);
    d.y.assign((size_t)max_step * 4, 0.0);
    d.y[0] = r0; d.y[1] = 0.0; d.y[2] = pr0; d.y[3] = pphi0;
    return replay_t ? replay_trajectory(b, d, replay_t, replay_L, rtol, atol, status)
                    : free_trajectory(b, d, max_step, rtol, atol, h_init, status);
}
}  // namespace

extern "C" {

// Whole path for one binary: IC, trajectory, multipoles, splines, synthesis
// on the uniform grid and the white-noise likelihood.
//
// params: m1, m2 [Msun], chi1, chi2, f0 [Hz]
// cfg: dt [s], N samples, modes (ls, ms, K), max_step, rtol, atol
// h_init: first step of the adaptive pass [M] (the reference's 0.01,
//   eob/new_Dormand_horiz.py:527-531; another value samples the same
//   trajectory on other knots)
// replay_t (may be null): knot times [M] of a trajectory of replay_L rows,
//   replay_t[0] = 0.  Instead of the two adaptive passes, the state is carried
//   from row i - 1 to row i by one DOPR853 step of h = replay_t[i] -
//   replay_t[i - 1], always accepted: the reference's integrator on a given
//   sequence of accepted steps (every row of both passes is one accepted
//   step from the row before it, src/DOPR853.cu:357-618), so that two
//   implementations can be compared on the same knots.
// data: d[N]; amp: template amplitude A (h_k = A Re sum_lm h_lm(t_k))
// outputs (optional, may be null):
//   ic[3] = (r0, pphi0, pr0); nsteps (trajectory rows); traj_t[max_step], traj_y[max_step][4]
//   npts (waveform samples of this binary); h_out[N] complex (re, im interleaved, summed modes)
// returns lnL; status codes in *status (0 ok, 1 bad trajectory)
double oracle_lnl_ex(const double *params, double dt, int N, const int *ls, const int *ms, int K, int max_step,
                     double rtol, double atol, double h_init, const double *replay_t, int replay_L,
                     const double *data, double amp, double *ic, int *nsteps, double *traj_t, double *traj_y,
                     int *npts, double *h_out, int *status)
{
    Binary b;
    Dense d;
    const int L = trajectory_ex(params, max_step, rtol, atol, h_init, replay_t, replay_L, b, d, ic, status);
    if (nsteps) *nsteps = L;
    if (traj_t) for (int i = 0; i < L; ++i) traj_t[i] = d.t[i];
    if (traj_y) for (int i = 0; i < 4 * L; ++i) traj_y[i] = d.y[i];
    if (L < 2) { *status = 1; return 0.0; }
    return post_trajectory(b, d, L, params[0] + params[1], dt, N, ls, ms, K, data, amp, npts, h_out);
}

// The same run up to the multipoles on the trajectory: rows t[L] [M],
// y[L][4], modes hl[K][L] (complex, interleaved); returns L
int oracle_knots_ex(const double *params, const int *ls, const int *ms, int K, int max_step, double rtol, double atol,
                    double h_init, const double *replay_t, int replay_L, double *traj_t, double *traj_y, double *hl_out,
                    int *status)
{
    Binary b;
    Dense d;
    const int L = trajectory_ex(params, max_step, rtol, atol, h_init, replay_t, replay_L, b, d, nullptr, status);
    if (L < 2) { *status = 1; return L; }
    for (int i = 0; i < L; ++i) traj_t[i] = d.t[i];
    for (int i = 0; i < 4 * L; ++i) traj_y[i] = d.y[i];
    const std::vector<cplx> hl = modes_on_trajectory(b, d, L, ls, ms, K);
    for (size_t i = 0; i < hl.size(); ++i) { hl_out[2 * i] = hl[i].real(); hl_out[2 * i + 1] = hl[i].imag(); }
    return L;
}

// the QNM table lookup of physics/imr_fits.h at spin a: out = (re, im), unit mass
void oracle_qnm(int l, int m, double a, double *out) { eob::qnm_lookup(l, m, a, &out[0], &out[1]); }

// The fits of the merger-ringdown completion (physics/imr_fits.h) for mode
// (l, m): out = [delta t_22, |h| peak fit, its first and second derivative,
// omega, omega dot, c1f, c2f, d1f, d2f, final mass, final spin, QNM re, QNM im
// (unit remnant mass)]
void oracle_imr_fits(int l, int m, double m1, double m2, double chi1, double chi2, double *out)
{
    const double chiS = 0.5 * (chi1 + chi2), chiA = 0.5 * (chi1 - chi2);
    const double eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
    const double chi = chiS + chiA * (m1 - m2) / (m1 + m2) / (1.0 - 2.0 * eta);
    out[0] = eob::nr_delta_t22(m1, m2, chi1, chi2);
    out[1] = eob::nr_peak_amp(l, m, m1, m2, chiS, chiA);
    out[2] = eob::nr_peak_adot(l, m, m1, m2, chiS, chiA);
    out[3] = eob::nr_peak_addot(l, m, m1, m2, chiS, chiA);
    out[4] = eob::nr_peak_omega(l, m, eta, chi);
    out[5] = eob::nr_peak_omegadot(l, m, eta, chi);
    for (int w = 0; w < 4; ++w) out[6 + w] = eob::rd_coeff(w, l, m, eta, chi);
    out[10] = eob::final_mass_seobnrv4(m1, m2, chi1, chi2);
    out[11] = eob::final_spin_hbr2016(m1, m2, chi1, chi2);
    eob::qnm_lookup(l, m, out[11], &out[12], &out[13]);
}

double oracle_lnl_one(const double *params, double dt, int N, const int *ls, const int *ms, int K, int max_step,
                      double rtol, double atol, const double *data, double amp, double *ic, int *nsteps, double *traj_t,
                      double *traj_y, int *npts, double *h_out, int *status)
{
    return oracle_lnl_ex(params, dt, N, ls, ms, K, max_step, rtol, atol, 0.01, nullptr, 0, data, amp, ic, nsteps,
                         traj_t, traj_y, npts, h_out, status);
}

// batch convenience: params[B][5]; lnl[B]; status[B]
void oracle_lnl_batch(const double *params, int B, double dt, int N, const int *ls, const int *ms, int K, int max_step,
                      double rtol, double atol, const double *data, double amp, double *lnl, int *status)
{
    for (int i = 0; i < B; ++i)
        lnl[i] = oracle_lnl_one(params + 5 * i, dt, N, ls, ms, K, max_step, rtol, atol, data, amp, nullptr, nullptr,
                                nullptr, nullptr, nullptr, nullptr, &status[i]);
}

}  // extern "C"
