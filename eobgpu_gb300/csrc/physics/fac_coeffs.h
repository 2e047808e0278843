// Per-binary factorized-waveform coefficients of the SEOBNRv4HM resummed
// multipoles h_lm = h^N_lm * S_lm * T_lm * exp(i delta_lm) * (rho_lm^l + f_lm),
// l = 2..8, m = 1..l.
//
// Restates the coefficient routine of EOBGPU src/EOB.cu:1945-2462
// (EOBCalcSpinFacWaveformCoefficients, struct include/EOB.hh:17-362), itself
// the LALSuite SEOBNRv4HM routine.  The PN coefficients are physics constants
// and are kept identical; the layout is ours: per (l,m) dense coefficient
// arrays in powers of v (rho, eulerlog part of rho, real f) and of vh / v
// (delta), so that one loop evaluates any mode.  Coefficients the reference
// never assigns (its equal-mass branches, delta21v7, delta44v5, delta55v5)
// are 0 here, matching a zero-initialised reference allocation.
//
// Host + device (plain C++ when compiled without nvcc).
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define EOB_HD __host__ __device__ __forceinline__
#else
#define EOB_HD inline
#endif

namespace eob {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kEulerGamma = 0.57721566490153286060651209008240243104215933593992;
constexpr double kMTSUN_SI = 4.925491025543575903411922162094833998e-6;

constexpr int kLMax = 8;
constexpr int kNumLM = 35;  // (l, m) pairs l = 2..8, m = 1..l
constexpr int kRhoDeg = 12;  // highest power of v in any rho_lm (h22 calibration v^12)

// Index of (l, m) in the l-major ordering used by the reference's flux loop
// (src/EOB.cu:2534-2536) and by its Newtonian-prefix packing
// (eob/seobnrv4phm.py:1873-1882).
EOB_HD constexpr int lm_index(int l, int m) { return (l - 2) * (l + 1) / 2 + (m - 1); }

// Dense factorized-waveform coefficients for every (l, m), l <= 8.
struct FacCoeffs {
    double rho[kNumLM][kRhoDeg + 1];   // rho_lm = 1 + sum_k (rho[k] + rhol[k] * eulerlog_m(v)) v^k
    double rhol[kNumLM][kRhoDeg + 1];
    double fre[kNumLM][8];             // real part of f_lm: sum_k fre[k] v^k
    double fim_vh6[kNumLM];            // imaginary part of f_lm: fim_vh6 * vh^6 (only (3,3))
    double dvh[kNumLM][10];            // delta_lm = sum_k dvh[k] vh^k + sum_k dv[k] v^k
    double dv[kNumLM][9];
    double eta;                        // symmetric mass ratio used by the modes
    int equal_mass;                    // eta == 0.25: odd-m modes use f_lm alone
};

// ---------------------------------------------------------------------------
// Builder.  m1, m2 in units of the total mass; a = tplspin (Kerr parameter
// of the test-particle limit); chiS, chiA = (chi1 +- chi2)/2.  use_hm = 1 is
// the SEOBNRv4HM setting used by the waveform class.
EOB_HD void fac_coeffs_build(FacCoeffs *c, int use_hm, double m1, double m2, double eta, double a,
                             double chiS, double chiA)
{
    for (int i = 0; i < kNumLM; ++i) {
        for (int k = 0; k <= kRhoDeg; ++k) { c->rho[i][k] = 0.0; c->rhol[i][k] = 0.0; }
        for (int k = 0; k < 8; ++k) c->fre[i][k] = 0.0;
        for (int k = 0; k < 10; ++k) c->dvh[i][k] = 0.0;
        for (int k = 0; k < 9; ++k) c->dv[i][k] = 0.0;
        c->fim_vh6[i] = 0.0;
    }
    const double pi = kPi;
    const double eta2 = eta * eta, eta3 = eta2 * eta;
    double dM2 = 1.0 - 4.0 * eta;
    const double chiA2 = chiA * chiA, chiS2 = chiS * chiS;
    const double chiA3 = chiA2 * chiA, chiS3 = chiS2 * chiS;
    if (dM2 < 0.0 && dM2 > -1e-4) dM2 = 0.0;
    double dM = sqrt(dM2);
    if (m1 < m2) dM = -dM;
    const bool neq = (dM2 != 0.0);  // unequal masses
    double a2 = a * a, a3 = a2 * a;
    const double p3 = -1.0 + 3.0 * eta;  // (3 eta - 1)
    const double p3sq = p3 * p3, p3cu = p3sq * p3;
    const double e12 = -1.0 + 2.0 * eta;  // (2 eta - 1)
    const double e155 = 1.0 - 5.0 * eta + 5.0 * eta2;
    const double e7 = -1.0 + 7.0 * eta - 14.0 * eta2 + 7.0 * eta3;
    const double e6 = -1.0 + 6.0 * eta - 10.0 * eta2 + 4.0 * eta3;
    const double dM2eta = dM2 + 3.0 * eta2;

    // ---- (2,2) -- the only mode that keeps the spin parameter a
    {
        const int i = lm_index(2, 2);
        c->dvh[i][3] = 7.0 / 3.0;
        c->dvh[i][6] = -4.0 / 3.0 * (dM * chiA + chiS * (1 - 2 * eta)) + (428.0 * pi) / 105.0;
        c->dvh[i][9] = -2203.0 / 81.0 + (1712.0 * pi * pi) / 315.0;
        c->dv[i][5] = -24.0 * eta;
        c->rho[i][2] = -43.0 / 42.0 + (55.0 * eta) / 84.0;
        c->rho[i][3] = (-2.0 * (chiS + chiA * dM - chiS * eta)) / 3.0;
        c->rho[i][4] = -20555.0 / 10584.0 + 0.5 * (chiS + chiA * dM) * (chiS + chiA * dM) - (33025.0 * eta) / 21168.0 +
                       (19583.0 * eta2) / 42336.0;
        c->rho[i][5] = (-34.0 / 21.0 + 49.0 * eta / 18.0 + 209.0 * eta2 / 126.0) * chiS +
                       (-34.0 / 21.0 - 19.0 * eta / 42.0) * dM * chiA;
        c->rho[i][6] = 1556919113.0 / 122245200.0 + (89.0 * a2) / 252.0 - (48993925.0 * eta) / 9779616.0 -
                       (6292061.0 * eta2) / 3259872.0 + (10620745.0 * eta3) / 39118464.0 +
                       (41.0 * eta * pi * pi) / 192.0;
        c->rhol[i][6] = -428.0 / 105.0;
        c->rho[i][7] = a3 / 3.0 + chiA * dM * (18733.0 / 15876.0 + (50140.0 * eta) / 3969.0 + (97865.0 * eta2) / 63504.0) +
                       chiS * (18733.0 / 15876.0 + (74749.0 * eta) / 5292.0 - (245717.0 * eta2) / 63504.0 +
                               (50803.0 * eta3) / 63504.0);
        c->rho[i][8] = -387216563023.0 / 160190110080.0 + (18353.0 * a2) / 21168.0 - a2 * a2 / 8.0;
        c->rhol[i][8] = 9202.0 / 2205.0;
        c->rho[i][10] = -16094530514677.0 / 533967033600.0;
        c->rhol[i][10] = 439877.0 / 55566.0;
    }
    if (use_hm) { a = 0.0; a2 = 0.0; a3 = 0.0; }

    // ---- (2,1)
    {
        const int i = lm_index(2, 1);
        c->dvh[i][3] = 2.0 / 3.0;
        c->dvh[i][6] = (107.0 * pi) / 105.0;
        c->dvh[i][9] = -272.0 / 81.0 + (214.0 * pi * pi) / 315.0;
        c->dv[i][5] = -493.0 * eta / 42.0;
        if (neq) {
            c->rho[i][2] = -59.0 / 56 + (23.0 * eta) / 84.0;
            c->rho[i][4] = -47009.0 / 56448.0 - (865.0 * a2) / 1792.0 - (405.0 * a2 * a2) / 2048.0 -
                           (10993.0 * eta) / 14112.0 + (617.0 * eta2) / 4704.0;
            c->rho[i][5] = (-98635.0 * a) / 75264.0 + (2031.0 * a * a2) / 7168.0 - (1701.0 * a2 * a3) / 8192.0;
            c->rho[i][6] = 7613184941.0 / 2607897600.0 + (9032393.0 * a2) / 1806336.0 + (3897.0 * a2 * a2) / 16384.0 -
                           (15309.0 * a3 * a3) / 65536.0;
            c->rhol[i][6] = -107.0 / 105.0;
            c->rho[i][7] = (-3859374457.0 * a) / 1159065600.0 - (55169.0 * a3) / 16384.0 + (18603.0 * a2 * a3) / 65536.0 -
                           (72171.0 * a2 * a2 * a3) / 262144.0;
            c->rhol[i][7] = 107.0 * a / 140.0;
            c->rho[i][8] = -1168617463883.0 / 911303737344.0;
            c->rhol[i][8] = 6313.0 / 5880.0;
            c->rho[i][10] = -63735873771463.0 / 16569158860800.0;
            c->rhol[i][10] = 5029963.0 / 5927040.0;
            c->fre[i][1] = (-3.0 * (chiS + chiA / dM)) / 2.0;
            c->fre[i][3] = (chiS * dM * (427.0 + 79.0 * eta) + chiA * (147.0 + 280.0 * dM * dM + 1251.0 * eta)) / 84.0 / dM;
            if (use_hm) {
                c->fre[i][4] = (-3.0 - 2.0 * eta) * chiA2 + (-3.0 + eta / 2.0) * chiS2 + (-6.0 + 21.0 * eta / 2.0) * chiS * chiA / dM;
                c->fre[i][5] = (3.0 / 4.0 - 3.0 * eta) * chiA3 / dM +
                               (-81.0 / 16.0 + 1709.0 * eta / 1008.0 + 613.0 * eta2 / 1008.0 + (9.0 / 4.0 - 3 * eta) * chiA2) * chiS +
                               3.0 / 4.0 * chiS3 +
                               (-81.0 / 16.0 - 703.0 * eta2 / 112.0 + 8797.0 * eta / 1008.0 + (9.0 / 4.0 - 6.0 * eta) * chiS2) * chiA / dM;
                c->fre[i][6] = (4163.0 / 252.0 - 9287.0 * eta / 1008.0 - 85.0 * eta2 / 112.0) * chiA2 +
                               (4163.0 / 252.0 - 2633.0 * eta / 1008.0 + 461.0 * eta2 / 1008.0) * chiS2 +
                               (4163.0 / 126.0 - 1636.0 * eta / 21.0 + 1088.0 * eta2 / 63.0) * chiS * chiA / dM;
            }
        } else {
            c->fre[i][1] = -3.0 * chiA / 2.0;
            c->fre[i][3] = (chiS * dM * (427.0 + 79.0 * eta) + chiA * (147.0 + 280.0 * dM * dM + 1251.0 * eta)) / 84.0;
            if (use_hm) {
                c->fre[i][4] = (-6 + 21 * eta / 2.0) * chiS * chiA;
                c->fre[i][5] = (3.0 / 4.0 - 3.0 * eta) * chiA3 +
                               (-81.0 / 16.0 - 703.0 * eta2 / 112.0 + 8797.0 * eta / 1008.0 + (9.0 / 4.0 - 6.0 * eta) * chiS2) * chiA;
                c->fre[i][6] = (4163.0 / 126.0 - 1636.0 * eta / 21.0 + 1088.0 * eta2 / 63.0) * chiS * chiA;
            }
        }
    }

    // ---- (3,3)
    {
        const int i = lm_index(3, 3);
        c->dvh[i][3] = 13.0 / 10.0;
        c->dvh[i][6] = (39.0 * pi) / 7.0;
        c->dvh[i][9] = -227827.0 / 3000.0 + (78.0 * pi * pi) / 7.0;
        c->dv[i][5] = -80897.0 * eta / 2430.0;
        if (neq) {
            c->rho[i][2] = -7.0 / 6.0 + (2.0 * eta) / 3.0;
            c->rho[i][4] = -6719.0 / 3960.0 + a2 / 2.0 - (1861.0 * eta) / 990.0 + (149.0 * eta2) / 330.0;
            c->rho[i][5] = (-4.0 * a) / 3.0;
            c->rho[i][6] = 3203101567.0 / 227026800.0 + (5.0 * a2) / 36.0;
            c->rhol[i][6] = -26.0 / 7.0;
            c->rho[i][7] = (5297.0 * a) / 2970.0 + a * a2 / 3.0;
            c->rho[i][8] = -57566572157.0 / 8562153600.0;
            c->rhol[i][8] = 13.0 / 3.0;
            if (use_hm) {
                c->rho[i][6] = 3203101567.0 / 227026800.0 + (5.0 * a2) / 36.0 +
                               (-129509.0 / 25740.0 + 41.0 / 192.0 * pi * pi) * eta - 274621.0 / 154440.0 * eta2 +
                               12011.0 / 46332.0 * eta3;
                c->rho[i][10] = -903823148417327.0 / 30566888352000.0;
                c->rhol[i][10] = 87347.0 / 13860.0;
            }
            c->fre[i][3] = (chiS * dM * (-4.0 + 5.0 * eta) + chiA * (-4.0 + 19.0 * eta)) / (2.0 * dM);
            if (use_hm) {
                c->fre[i][4] = (3.0 / 2.0 * chiS2 * dM + (3.0 - 12 * eta) * chiA * chiS + dM * (3.0 / 2.0 - 6.0 * eta) * chiA2) / dM;
                c->fre[i][5] = (dM * (241.0 / 30.0 * eta2 + 11.0 / 20.0 * eta + 2.0 / 3.0) * chiS +
                                (407.0 / 30.0 * eta2 - 593.0 / 60.0 * eta + 2.0 / 3.0) * chiA) / dM;
                c->fre[i][6] = (dM * (6.0 * eta2 - 27.0 / 2.0 * eta - 7.0 / 4.0) * chiS2 +
                                (44.0 * eta2 - 1.0 * eta - 7.0 / 2.0) * chiA * chiS +
                                dM * (-12 * eta2 + 11.0 / 2.0 * eta - 7.0 / 4.0) * chiA2) / dM;
                c->fim_vh6[i] = (dM * (593.0 / 108.0 * eta - 81.0 / 20.0) * chiS + (7339.0 / 540.0 * eta - 81.0 / 20.0) * chiA) / dM;
            }
        } else {
            c->fre[i][3] = chiA * 3.0 / 8.0;
            if (use_hm) {
                c->fre[i][4] = (3.0 - 12 * eta) * chiA * chiS;
                c->fre[i][5] = (407.0 / 30.0 * eta2 - 593.0 / 60.0 * eta + 2.0 / 3.0) * chiA;
                c->fre[i][6] = (44.0 * eta2 - 1.0 * eta - 7.0 / 2.0) * chiA * chiS;
                c->fim_vh6[i] = (7339.0 / 540.0 * eta - 81.0 / 20.0) * chiA;
            }
        }
    }

    // ---- (3,2)
    {
        const int i = lm_index(3, 2);
        c->dvh[i][3] = (10.0 + 33.0 * eta) / (-15.0 * p3);
        c->dvh[i][6] = (52.0 * pi) / 21.0;
        c->dvh[i][9] = -9112.0 / 405.0 + (208.0 * pi * pi) / 63.0;
        c->rho[i][1] = (4.0 * chiS * eta) / (-3.0 * p3);
        c->rho[i][2] = (328.0 - 1115.0 * eta + 320.0 * eta2) / (270.0 * p3);
        c->rho[i][3] = 2.0 / 9.0 * a;
        c->rho[i][4] = a2 / 3.0 + (-1444528.0 + 8050045.0 * eta - 4725605.0 * eta2 - 20338960.0 * eta3 +
                                   3085640.0 * eta2 * eta2) / (1603800.0 * p3sq);
        c->rho[i][5] = (-2788.0 * a) / 1215.0;
        c->rho[i][6] = 5849948554.0 / 940355325.0 + (488.0 * a2) / 405.0;
        c->rhol[i][6] = -104.0 / 63.0;
        c->rho[i][8] = -10607269449358.0 / 3072140846775.0;
        c->rhol[i][8] = 17056.0 / 8505.0;
        (void)p3cu;
    }

    // ---- (3,1)
    {
        const int i = lm_index(3, 1);
        c->dvh[i][3] = 13.0 / 30.0;
        c->dvh[i][6] = (13.0 * pi) / 21.0;
        c->dvh[i][9] = -227827.0 / 81000.0 + (26.0 * pi * pi) / 63.0;
        c->dv[i][5] = -17.0 * eta / 10.0;
        if (neq) {
            c->rho[i][2] = -13.0 / 18.0 - (2.0 * eta) / 9.0;
            c->rho[i][4] = 101.0 / 7128.0 - (5.0 * a2) / 6.0 - (1685.0 * eta) / 1782.0 - (829.0 * eta2) / 1782.0;
            c->rho[i][5] = (4.0 * a) / 9.0;
            c->rho[i][6] = 11706720301.0 / 6129723600.0 - (49.0 * a2) / 108.0;
            c->rhol[i][6] = -26.0 / 63.0;
            c->rho[i][7] = (-2579.0 * a) / 5346.0 + a * a2 / 9.0;
            c->rho[i][8] = 2606097992581.0 / 4854741091200.0;
            c->rhol[i][8] = 169.0 / 567.0;
            c->fre[i][3] = (chiA * (-4.0 + 11.0 * eta) + chiS * dM * (-4.0 + 13.0 * eta)) / (2.0 * dM);
        } else {
            c->fre[i][3] = -chiA * 5.0 / 8.0;
        }
    }

    // ---- (4,4)
    {
        const int i = lm_index(4, 4);
        c->dvh[i][3] = (112.0 + 219.0 * eta) / (-120.0 * p3);
        c->dvh[i][6] = (25136.0 * pi) / 3465.0;
        if (use_hm) c->dvh[i][9] = -55144.0 / 375.0 + 201088.0 * pi * pi / 10395.0;
        c->rho[i][2] = (1614.0 - 5870.0 * eta + 2625.0 * eta2) / (1320.0 * p3);
        c->rho[i][3] = (chiA * (10.0 - 39.0 * eta) * dM + chiS * (10.0 - 41.0 * eta + 42.0 * eta2)) / (15.0 * p3);
        c->rho[i][4] = a2 / 2.0 + (-511573572.0 + 2338945704.0 * eta - 313857376.0 * eta2 - 6733146000.0 * eta3 +
                                   1252563795.0 * eta2 * eta2) / (317116800.0 * p3sq);
        c->rho[i][5] = (-69.0 * a) / 55.0;
        if (use_hm) {
            c->rho[i][4] = (-511573572.0 + 2338945704.0 * eta - 313857376.0 * eta2 - 6733146000.0 * eta3 +
                            1252563795.0 * eta2 * eta2) / (317116800.0 * p3sq) +
                           chiS2 / 2.0 + dM * chiS * chiA + dM2 * chiA2 / 2.0;
            c->rho[i][5] = chiA * dM * (-8280.0 + 42716.0 * eta - 57990.0 * eta2 + 8955 * eta3) / (6600.0 * p3sq) +
                           chiS * (-8280.0 + 66284.0 * eta - 176418.0 * eta2 + 128085.0 * eta3 + 88650 * eta2 * eta2) /
                               (6600.0 * p3sq);
            c->rho[i][8] = -172066910136202271.0 / 19426955708160000.0;
            c->rhol[i][8] = 845198.0 / 190575.0;
            c->rho[i][10] = -17154485653213713419357.0 / 568432724020761600000.0;
            c->rhol[i][10] = 22324502267.0 / 3815311500.0;
        }
        c->rho[i][6] = 16600939332793.0 / 1098809712000.0 + (217.0 * a2) / 3960.0;
        c->rhol[i][6] = -12568.0 / 3465.0;
    }

    // ---- (4,3)
    {
        const int i = lm_index(4, 3);
        c->dvh[i][3] = (486.0 + 4961.0 * eta) / (810.0 * (1.0 - 2.0 * eta));
        c->dvh[i][6] = 1571.0 * pi / 385.0;
        if (neq) {
            c->rho[i][2] = (222.0 - 547.0 * eta + 160.0 * eta2) / (176.0 * e12);
            c->rho[i][4] = -6894273.0 / 7047040.0 + (3.0 * a2) / 8.0;
            c->rho[i][5] = (-12113.0 * a) / 6160.0;
            c->rho[i][6] = 1664224207351.0 / 195343948800.0;
            c->rhol[i][6] = -1571.0 / 770.0;
            c->fre[i][1] = (5.0 * (chiA - chiS * dM) * eta) / (2.0 * dM * e12);
        } else {
            c->fre[i][1] = -5.0 * chiA / 4.0;
        }
    }

    // ---- (4,2)
    {
        const int i = lm_index(4, 2);
        c->dvh[i][3] = (7.0 * (1.0 + 6.0 * eta)) / (-15.0 * p3);
        c->dvh[i][6] = (6284.0 * pi) / 3465.0;
        c->rho[i][2] = (1146.0 - 3530.0 * eta + 285.0 * eta2) / (1320.0 * p3);
        c->rho[i][3] = (chiA * (10.0 - 21.0 * eta) * dM + chiS * (10.0 - 59.0 * eta + 78.0 * eta2)) / (15.0 * p3);
        c->rho[i][4] = a2 / 2.0 + (-114859044.0 + 295834536.0 * eta + 1204388696.0 * eta2 - 3047981160.0 * eta3 -
                                   379526805.0 * eta2 * eta2) / (317116800.0 * p3sq);
        c->rho[i][5] = (-7.0 * a) / 110.0;
        c->rho[i][6] = 848238724511.0 / 219761942400.0 + (2323.0 * a2) / 3960.0;
        c->rhol[i][6] = -3142.0 / 3465.0;
    }

    // ---- (4,1)
    {
        const int i = lm_index(4, 1);
        c->dvh[i][3] = (2.0 + 507.0 * eta) / (10.0 * (1.0 - 2.0 * eta));
        c->dvh[i][6] = 1571.0 * pi / 3465.0;
        if (neq) {
            c->rho[i][2] = (602.0 - 1385.0 * eta + 288.0 * eta2) / (528.0 * e12);
            c->rho[i][4] = -7775491.0 / 21141120.0 + (3.0 * a2) / 8.0;
            c->rho[i][5] = (-20033.0 * a) / 55440.0 - (5 * a * a2) / 6.0;
            c->rho[i][6] = 1227423222031.0 / 1758095539200.0;
            c->rhol[i][6] = -1571.0 / 6930.0;
            c->fre[i][1] = (5.0 * (chiA - chiS * dM) * eta) / (2.0 * dM * e12);
        } else {
            c->fre[i][1] = -5.0 * chiA / 4.0;
        }
    }

    // ---- (5,5)
    {
        const int i = lm_index(5, 5);
        c->dvh[i][3] = (96875.0 + 857528.0 * eta) / (131250.0 * (1 - 2 * eta));
        if (use_hm) {
            c->dvh[i][6] = 3865.0 / 429.0 * pi;
            c->dvh[i][9] = (-7686949127.0 + 954500400.0 * pi * pi) / 31783752.0;
        }
        if (neq) {
            c->rho[i][2] = (487.0 - 1298.0 * eta + 512.0 * eta2) / (390.0 * e12);
            c->rho[i][3] = (-2.0 * a) / 3.0;
            c->rho[i][4] = -3353747.0 / 2129400.0 + a2 / 2.0;
            c->rho[i][5] = -241.0 * a / 195.0;
            if (use_hm) {
                c->rho[i][6] = 190606537999247.0 / 11957879934000.0;
                c->rhol[i][6] = -1546.0 / 429.0;
                c->rho[i][8] = -1213641959949291437.0 / 118143853747920000.0;
                c->rhol[i][8] = 376451.0 / 83655.0;
                c->rho[i][10] = -150082616449726042201261.0 / 4837990810977324000000.0;
                c->rhol[i][10] = 2592446431.0 / 456756300.0;
                c->fre[i][3] = chiA / dM * (10.0 / (3.0 * e12) - 70.0 * eta / (3.0 * e12) + 110.0 * eta2 / (3.0 * e12)) +
                               chiS * (10.0 / (3.0 * e12) - 10.0 * eta / e12 + 10 * eta2 / e12);
                c->fre[i][4] = chiS2 * (-5.0 / (2.0 * e12) + 5.0 * eta / e12) +
                               chiA * chiS / dM * (-5.0 / e12 + 30.0 * eta / e12 - 40.0 * eta2 / e12) +
                               chiA2 * (-5.0 / (2.0 * e12) + 15.0 * eta / e12 - 20.0 * eta2 / e12);
            }
        } else if (use_hm) {
            c->fre[i][3] = chiA * (10.0 / (3.0 * e12) - 70.0 * eta / (3.0 * e12) + 110.0 * eta2 / (3.0 * e12));
            c->fre[i][4] = chiA * chiS * (-5.0 / e12 + 30.0 * eta / e12 - 40.0 * eta2 / e12);
        }
    }

    // ---- (5,4), (5,3), (5,2), (5,1)
    {
        int i = lm_index(5, 4);
        c->dvh[i][3] = 8.0 / 15.0;
        c->rho[i][2] = (-17448.0 + 96019.0 * eta - 127610.0 * eta2 + 33320.0 * eta3) / (13650.0 * e155);
        c->rho[i][3] = (-2.0 * a) / 15.0;
        c->rho[i][4] = -16213384.0 / 15526875.0 + (2.0 * a2) / 5.0;
        i = lm_index(5, 3);
        c->dvh[i][3] = 31.0 / 70.0;
        if (neq) {
            c->rho[i][2] = (375.0 - 850.0 * eta + 176.0 * eta2) / (390.0 * e12);
            c->rho[i][3] = (-2.0 * a) / 3.0;
            c->rho[i][4] = -410833.0 / 709800.0 + a2 / 2.0;
            c->rho[i][5] = -103.0 * a / 325.0;
        }
        i = lm_index(5, 2);
        c->dvh[i][3] = 4.0 / 15.0;
        c->rho[i][2] = (-15828.0 + 84679.0 * eta - 104930.0 * eta2 + 21980.0 * eta3) / (13650.0 * e155);
        c->rho[i][3] = (-2.0 * a) / 15.0;
        c->rho[i][4] = -7187914.0 / 15526875.0 + (2.0 * a2) / 5.0;
        i = lm_index(5, 1);
        c->dvh[i][3] = 31.0 / 210.0;
        if (neq) {
            c->rho[i][2] = (319.0 - 626.0 * eta + 8.0 * eta2) / (390.0 * e12);
            c->rho[i][3] = (-2.0 * a) / 3.0;
            c->rho[i][4] = -31877.0 / 304200.0 + a2 / 2.0;
            c->rho[i][5] = 139.0 * a / 975.0;
        }
    }

    // ---- l = 6
    {
        int i = lm_index(6, 6);
        c->dvh[i][3] = 43.0 / 70.0;
        c->rho[i][2] = (-106.0 + 602.0 * eta - 861.0 * eta2 + 273.0 * eta3) / (84.0 * e155);
        c->rho[i][3] = (-2.0 * a) / 3.0;
        c->rho[i][4] = -1025435.0 / 659736.0 + a2 / 2.0;
        i = lm_index(6, 5);
        c->dvh[i][3] = 10.0 / 21.0;
        if (neq) {
            c->rho[i][2] = (-185.0 + 838.0 * eta - 910.0 * eta2 + 220.0 * eta3) / (144.0 * dM2eta);
            c->rho[i][3] = -2.0 * a / 9.0;
        }
        i = lm_index(6, 4);
        c->dvh[i][3] = 43.0 / 105.0;
        c->rho[i][2] = (-86.0 + 462.0 * eta - 581.0 * eta2 + 133.0 * eta3) / (84.0 * e155);
        c->rho[i][3] = (-2.0 * a) / 3.0;
        c->rho[i][4] = -476887.0 / 659736.0 + a2 / 2.0;
        i = lm_index(6, 3);
        c->dvh[i][3] = 2.0 / 7.0;
        if (neq) {
            c->rho[i][2] = (-169.0 + 742.0 * eta - 750.0 * eta2 + 156.0 * eta3) / (144.0 * dM2eta);
            c->rho[i][3] = -2.0 * a / 9.0;
        }
        i = lm_index(6, 2);
        c->dvh[i][3] = 43.0 / 210.0;
        c->rho[i][2] = (-74.0 + 378.0 * eta - 413.0 * eta2 + 49.0 * eta3) / (84.0 * e155);
        c->rho[i][3] = (-2.0 * a) / 3.0;
        c->rho[i][4] = -817991.0 / 3298680.0 + a2 / 2.0;
        i = lm_index(6, 1);
        c->dvh[i][3] = 2.0 / 21.0;
        if (neq) {
            c->rho[i][2] = (-161.0 + 694.0 * eta - 670.0 * eta2 + 124.0 * eta3) / (144.0 * dM2eta);
            c->rho[i][3] = -2.0 * a / 9.0;
        }
    }

    // ---- l = 7
    {
        int i = lm_index(7, 7);
        c->dvh[i][3] = 19.0 / 36.0;
        if (neq) {
            c->rho[i][2] = (-906.0 + 4246.0 * eta - 4963.0 * eta2 + 1380.0 * eta3) / (714.0 * dM2eta);
            c->rho[i][3] = -2.0 * a / 3.0;
        }
        i = lm_index(7, 6);
        c->rho[i][2] = (2144.0 - 16185.0 * eta + 37828.0 * eta2 - 29351.0 * eta3 + 6104.0 * eta2 * eta2) / (1666.0 * e7);
        i = lm_index(7, 5);
        c->dvh[i][3] = 95.0 / 252.0;
        if (neq) {
            c->rho[i][2] = (-762.0 + 3382.0 * eta - 3523.0 * eta2 + 804.0 * eta3) / (714.0 * dM2eta);
            c->rho[i][3] = -2.0 * a / 3.0;
        }
        i = lm_index(7, 4);
        c->rho[i][2] = (17756.0 - 131805.0 * eta + 298872.0 * eta2 - 217959.0 * eta3 + 41076.0 * eta2 * eta2) / (14994.0 * e7);
        i = lm_index(7, 3);
        c->dvh[i][3] = 19.0 / 84.0;
        if (neq) {
            c->rho[i][2] = (-666.0 + 2806.0 * eta - 2563.0 * eta2 + 420.0 * eta3) / (714.0 * dM2eta);
            c->rho[i][3] = -2.0 * a / 3.0;
        }
        i = lm_index(7, 2);
        c->rho[i][2] = (16832.0 - 123489.0 * eta + 273924.0 * eta2 - 190239.0 * eta3 + 32760.0 * eta2 * eta2) / (14994.0 * e7);
        i = lm_index(7, 1);
        c->dvh[i][3] = 19.0 / 252.0;
        if (neq) {
            c->rho[i][2] = (-618.0 + 2518.0 * eta - 2083.0 * eta2 + 228.0 * eta3) / (714.0 * dM2eta);
            c->rho[i][3] = -2.0 * a / 3.0;
        }
    }

    // ---- l = 8
    {
        c->rho[lm_index(8, 8)][2] = (3482.0 - 26778.0 * eta + 64659.0 * eta2 - 53445.0 * eta3 + 12243.0 * eta2 * eta2) / (2736.0 * e7);
        if (neq) c->rho[lm_index(8, 7)][2] = (23478.0 - 154099.0 * eta + 309498.0 * eta2 - 207550.0 * eta3 + 38920 * eta2 * eta2) / (18240.0 * e6);
        c->rho[lm_index(8, 6)][2] = (1002.0 - 7498.0 * eta + 17269.0 * eta2 - 13055.0 * eta3 + 2653.0 * eta2 * eta2) / (912.0 * e7);
        if (neq) c->rho[lm_index(8, 5)][2] = (4350.0 - 28055.0 * eta + 54642.0 * eta2 - 34598.0 * eta3 + 6056.0 * eta2 * eta2) / (3648.0 * e6);
        c->rho[lm_index(8, 4)][2] = (2666.0 - 19434.0 * eta + 42627.0 * eta2 - 28965.0 * eta3 + 4899.0 * eta2 * eta2) / (2736.0 * e7);
        if (neq) c->rho[lm_index(8, 3)][2] = (20598.0 - 131059.0 * eta + 249018.0 * eta2 - 149950.0 * eta3 + 24520.0 * eta2 * eta2) / (18240.0 * e6);
        c->rho[lm_index(8, 2)][2] = (2462.0 - 17598.0 * eta + 37119.0 * eta2 - 22845.0 * eta3 + 3063.0 * eta2 * eta2) / (2736.0 * e7);
        if (neq) c->rho[lm_index(8, 1)][2] = (20022.0 - 126451.0 * eta + 236922.0 * eta2 - 138430.0 * eta3 + 21640.0 * eta2 * eta2) / (18240.0 * e6);
    }

    double eta_m = eta;
    if (eta_m > 0.25 && eta_m < 0.25 + 1e-4) eta_m = 0.25;
    c->eta = eta_m;
    c->equal_mass = (eta_m == 0.25) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Which terms of rho_lm and f_lm the radiation-reaction flux keeps.  The flux
// multipoles (src/EOB.cu:1756-1929) truncate some series relative to the
// waveform multipoles (src/EOB.cu:1303-1592):
//   (3,3) rho stops at v^8; (4,4) rho stops at v^6; (5,5) rho stops at v^6 and
//   drops its eulerlog v^6 term; f_lm keeps only v^1 and v^3 terms.
EOB_HD int flux_rho_maxdeg(int l, int m)
{
    if (l == 2) return 10;
    if (l == 3) return 8;
    if (l == 4) return 6;
    if (l == 5) return (m == 5 || m == 3 || m == 1) ? ((m == 5) ? 6 : 5) : 4;
    if (l == 6) return (m % 2 == 0) ? 4 : 3;
    if (l == 7) return (m % 2 == 1) ? 3 : 2;
    return 2;
}
EOB_HD bool flux_keeps_rhol(int l, int m, int k) { return !(l == 5 && m == 5) && k <= flux_rho_maxdeg(l, m); }
EOB_HD bool flux_keeps_f(int l, int m, int k)
{
    if (l == 5) return false;  // f55 enters only the waveform multipole
    return k == 1 || k == 3;
}

// ---------------------------------------------------------------------------
// Newtonian multipole prefactors n_lm * c_lm * eta (Damour-Iyer-Nagar 2008,
// eqs. 5-7), restating eob/seobnrv4phm.py:1703-1776 for one (l, m).
// m1, m2 in units of the total mass.
EOB_HD double double_factorial(int n)
{
    double r = 1.0;
    for (int k = n; k > 1; k -= 2) r *= (double)k;
    return r;
}

EOB_HD void newton_prefix(double m1, double m2, int l, int m, double *re, double *im)
{
    const double tot = m1 + m2;
    const int eps = (l + m) % 2;
    const double x1 = m1 / tot, x2 = m2 / tot;
    const double eta = m1 * m2 / (tot * tot);
    const double sign = (m % 2 == 0) ? 1.0 : -1.0;
    double cval;
    if (m1 != m2 || sign == 1.0) {
        cval = pow(x2, (double)(l + eps - 1)) + sign * pow(x1, (double)(l + eps - 1));
    } else {
        cval = (l == 2 || l == 3) ? -1.0 : ((l == 4 || l == 5) ? -0.5 : 0.0);
    }
    // (i m)^l = m^l * i^l
    const double ml = pow((double)m, (double)l);
    const int q = l % 4;  // i^l
    double nr = (q == 0) ? ml : ((q == 2) ? -ml : 0.0);
    double ni = (q == 1) ? ml : ((q == 3) ? -ml : 0.0);
    const double dl = (double)l, dm = (double)m;
    if (eps == 0) {
        const double mult1 = 8.0 * kPi / double_factorial(2 * l + 1);
        const double mult2 = sqrt(((dl + 1) * (dl + 2)) / (dl * (dl - 1)));
        nr *= mult1 * mult2;
        ni *= mult1 * mult2;
    } else {
        nr = -nr;
        ni = -ni;
        const double mult1 = 16.0 * kPi / double_factorial(2 * l + 1);
        const double mult2 = sqrt(((2. * dl + 1) * (dl + 2) * (dl * dl - dm * dm)) /
                                  ((2. * dl - 1) * (dl + 1) * dl * (dl - 1)));
        // multiply by i * mult1 * mult2
        const double t = nr;
        nr = -ni * mult1 * mult2;
        ni = t * mult1 * mult2;
    }
    *re = nr * eta * cval;
    *im = ni * eta * cval;
}

// Y_n^m(theta = pi/2, phi = 0) with the Condon-Shortley phase, n + m even:
// sqrt((2n+1)/(4 pi) (n-m)!/(n+m)!) * (-1)^((n+m)/2) (n+m-1)!!/(n-m)!!.
EOB_HD double ylm_equator(int n, int m)
{
    if ((n + m) % 2 != 0) return 0.0;
    double ratio = 1.0;  // (n-m)!/(n+m)!
    for (int k = n - m + 1; k <= n + m; ++k) ratio /= (double)k;
    const double norm = sqrt((2.0 * n + 1.0) / (4.0 * kPi) * ratio);
    const double p = double_factorial(n + m - 1) / double_factorial(n - m);
    const double sgn = (((n + m) / 2) % 2 == 0) ? 1.0 : -1.0;
    return norm * sgn * p;
}

}  // namespace eob
