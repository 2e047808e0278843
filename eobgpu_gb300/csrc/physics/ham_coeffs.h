// Aligned-spin SEOBNRv5 effective Hamiltonian ("Ham_align", analytic),
// restated as per-binary coefficient tables in u = 1/r.
//
// The reference evaluates the expression of EOBGPU src/EOB.cu:16-107
// (evaluate_Ham_align_AD) from the masses and spins at every call, with
// generated derivatives (src/EOB.cu:139-222, 254-371).  Every coefficient that
// depends only on (nu, X1, X2, chi1, chi2, K, d5, dSO, dSS) is folded here
// once per binary; what remains per call is a few polynomials in u, log r and
// sqrt(u).  The PN coefficients are physics constants and are kept identical
// to the reference's.
//
//   H      = M sqrt(1 + 2 nu (Heff - 1)) / nu
//   Heff   = sqrt(A W) + L u^3 N(u, pr^2) / Dc(u)
//   W      = 1 + pr^2 (1 + Bnp) + L^2 c(u) + pr^4 q4 + pr^6 q6 + pr^8 q8
//   A      = (AK0 + AKa) Fa AS / Dc
//   Bnp    = AK0 Dbpm (1 + kb u) + bs3 u^3 + bs4 u^4 - 1 + ap2 u^2
//   c(u)   = u^2 (1 - apsq u^2 (1 + 2u) / Dc)
//   Dc     = 1 + ap2 u^2 + 2 ap2 u^3
// with the odd (spin-orbit) numerator N = sum_j pr^(2j) N_j(u).
#pragma once
#include <math.h>
#include "fac_coeffs.h"

namespace eob {

struct HamCoeffs {
    double M, nu;
    // AK0(u) = sum_k (ak0[k] + ak0l[k] log r) u^k + ak0h u^6 sqrt(u)
    double ak0[7], ak0l[7], ak0h;
    double aka[7];           // AKa(u), plain polynomial (calibration K terms and spin terms)
    double fa1, fa2;         // Fa(u) = 1 + fa1 u + fa2 u^2
    double as4, as5, as6;    // AS(u) = 1 + as4 u^4 + as5 u^5 + as6 u^6
    double ap2;              // chi1^2 X1^2 + 2 chi1 chi2 nu + chi2^2 X2^2
    double apsq;             // (chi1 X1 + chi2 X2)^2
    // Dbpm(u) = sum_k (db[k] + dbl[k] log r) u^k + dbh u^5 sqrt(u)
    double db[6], dbl[6], dbh;
    double kb;               // Bnp factor (1 + kb u)
    double bs3, bs4;
    // q4 = sum_k q4c[k] u^k + q4l u^4 log r + q4h u^4 sqrt(u)   (k = 2..4, includes QSalign2)
    double q4c[5], q4l, q4h;
    // q6 = q6c[2] u^2 + q6c[3] u^3 + q6h u^3 sqrt(u)
    double q6c[4], q6h;
    // q8 = q8c[1] u + q8c[2] u^2 + q8h u^2 sqrt(u)
    double q8c[3], q8h;
    // N_j(u) = sum_k (nc[j][k] + ncl[j][k] log r) u^k,  j = 0..4 (power of pr^2), k = 0..4
    double nc[5][5], ncl[5][5];
    // the coefficients of the u-derivatives (k c_k) and the doubled
    // constants, formed once per binary: the same products ham_eval formed
    // at every call
    struct Derived {
        double ak0l6, ak0l5, ak0h, fa2, as6, as5, as4, dbl5, dbl4, dbh, bs4, bs3, two_ap2;
        double q4c4, q4c3, q4c2, q4h, q6h, q6c3, q6c2, q8h, q8c2;
        double nc02, nc03, nc04, nc12, nc13, four_n4, two_nu;
    } d;
};

// m_1, m_2 as stored in the reference's additionalArgs (scaled to M = 1 by
// the waveform class, but any total mass works).
EOB_HD void ham_coeffs_build(HamCoeffs *h, double m_1, double m_2, double chi_1, double chi_2, double K, double d5,
                             double dSO, double dSS)
{
    const double pi = kPi, pi2 = kPi * kPi, eg = kEulerGamma;
    const double l2 = log(2.0), l3 = log(3.0), l5 = log(5.0), l7 = log(7.0);
    const double M = m_1 + m_2;
    const double mu = m_1 * m_2 / (m_1 + m_2);
    const double nu = mu / M;
    const double X1 = m_1 / M, X2 = m_2 / M;
    const double c1 = chi_1, c2 = chi_2;
    const double n2 = nu * nu, n3 = n2 * nu, n4 = n3 * nu, n5 = n4 * nu;
    const double s11 = c1 * c1 * X1 * X1, s22 = c2 * c2 * X2 * X2, s12 = c1 * c2 * nu;
    const double ap2 = s11 + 2.0 * s12 + s22;
    const double Kn = K * nu;
    h->M = M;
    h->nu = nu;
    h->ap2 = ap2;
    h->apsq = (c1 * X1 + c2 * X2) * (c1 * X1 + c2 * X2);

    // ---- AK0 (src/EOB.cu:70)
    for (int k = 0; k < 7; ++k) { h->ak0[k] = 0.0; h->ak0l[k] = 0.0; h->aka[k] = 0.0; }
    h->ak0[0] = 1.0;
    h->ak0[1] = -2.0 * Kn;
    h->ak0[2] = 4.0 * Kn * (Kn - 1.0);
    h->ak0[3] = 2.0 * nu * (-4.0 * K * K * K * n2 + 8.0 * K * K * nu - 4.0 * K + 1.0);
    h->ak0[4] = nu * (16.0 * pow(K, 4) * n3 - 48.0 * K * K * K * n2 + 48.0 * K * K * nu - 4.0 * K * (nu + 4.0) -
                      41.0 * pi2 / 32.0 + 106.0 / 3.0);
    h->ak0[5] = -32.0 * pow(K, 5) * n5 + 128.0 * pow(K, 4) * n4 + K * K * n3 * (8.0 - 192.0 * K) +
                n2 * (12288.0 * K * K - 7552.0 * K + 246.0 * pi2 * K - 3536.0 + 123.0 * pi2) / 96.0 +
                nu * (-32.0 * K + 1.0 / 20.0 + 128.0 * eg / 5.0 + 963.0 * pi2 / 512.0 + 256.0 * l2 / 5.0);
    h->ak0l[5] = -64.0 * nu / 5.0;
    h->ak0l[6] = 4.0 * nu * (nu * (672.0 * K + 756.0) + 1079.0) / 105.0;
    h->ak0h = 13696.0 * pi * nu / 525.0;

    // ---- AKa (src/EOB.cu:90)
    const double km1 = Kn - 1.0;
    h->aka[2] = Kn * (-Kn + 2.0) * ap2;
    h->aka[3] = 2.0 * Kn * ap2 * (2.0 * K * K * n2 - 5.0 * Kn + 3.0);
    h->aka[4] = Kn * (Kn - 2.0) * km1 * km1 * ap2 * ap2 - 4.0 * Kn * km1 * km1 * (3.0 * Kn - 4.0) * ap2;
    h->aka[5] = -2.0 * Kn * km1 * km1 * km1 * (3.0 * Kn - 5.0) * ap2 * ap2 +
                2.0 * nu * km1 * km1 * ap2 * (16.0 * K * K * K * n2 - 36.0 * K * K * nu + 20.0 * K - 1.0);
    h->aka[6] = -Kn * (Kn - 2.0) * km1 * km1 * km1 * km1 * ap2 * ap2 * ap2 -
                nu * km1 * km1 * ap2 *
                    (7680.0 * pow(K, 4) * n3 - 24576.0 * K * K * K * n2 + 26112.0 * K * K * nu - 768.0 * K * (nu + 12.0) -
                     123.0 * pi2 + 3776.0) / 96.0;

    // ---- A factors (src/EOB.cu:92)
    h->fa1 = -(-2.0 * Kn + 2.0);
    h->fa2 = (-Kn + 1.0) * (-Kn + 1.0) * ap2;
    h->as4 = s11 * (5.0 * X2 + nu) / 2.0 + s12 * (2.0 - nu) + s22 * (-5.0 * X2 + nu + 5.0) / 2.0;
    h->as5 = s11 * (-X2 * (294.0 * nu + 85.0) + 428.0 * X2 - 21.0 * n2 + 987.0 * nu) / 56.0 +
             s12 * (6.0 * n2 + 145.0 * nu + 68.0) / 8.0 +
             s22 * (X2 * (294.0 * nu + 85.0) - 428.0 * X2 - 21.0 * n2 + 693.0 * nu + 343.0) / 56.0;
    h->as6 = dSS * (s11 + c1 * c2 * (1.0 - 2.0 * nu) + s22);

    // ---- Dbpm (src/EOB.cu:68)
    for (int k = 0; k < 6; ++k) { h->db[k] = 0.0; h->dbl[k] = 0.0; }
    h->db[0] = 1.0;
    h->db[2] = 6.0 * nu;
    h->db[3] = -6.0 * n2 + 52.0 * nu;
    h->db[4] = n2 * (-260.0 + 123.0 * pi2 / 16.0) +
               nu * (-6496.0 * l2 / 15.0 - 23761.0 * pi2 / 1536.0 - 533.0 / 45.0 + 1184.0 * eg / 15.0 + 2916.0 * l3 / 5.0);
    h->dbl[4] = -592.0 * nu / 15.0;
    h->db[5] = d5;
    h->dbl[5] = 3392.0 * n2 / 15.0 + 1420.0 * nu / 7.0;
    h->dbh = 264932.0 * pi * nu / 1575.0;

    // ---- Bnp (src/EOB.cu:72, 66)
    h->kb = h->fa1;
    h->bs3 = 3.0 * s11 * (7.0 * X2 + 5.0 * nu) / 4.0 + s12 * (9.0 * nu / 2.0 + 6.0) + 3.0 * s22 * (-7.0 * X2 + 5.0 * nu + 7.0) / 4.0;
    h->bs4 = s11 * (1.0 * X2 * (38.0 - 48.0 * nu) - X2 * (80.0 * nu + 49.0) - 20.0 * n2 + 214.0 * nu) / 4.0 +
             s12 * (10.0 * n2 + 29.0 * nu + 8.0) +
             s22 * (1.0 * X2 * (48.0 * nu - 38.0) + X2 * (80.0 * nu + 49.0) - 20.0 * n2 + 86.0 * nu - 11.0) / 4.0;

    // ---- Q = QSalign2 + Qpm (src/EOB.cu:54-58)
    for (int k = 0; k < 5; ++k) h->q4c[k] = 0.0;
    for (int k = 0; k < 4; ++k) h->q6c[k] = 0.0;
    for (int k = 0; k < 3; ++k) h->q8c[k] = 0.0;
    const double qs = -5.0 * s11 * (X2 * (18.0 * nu - 1.0) + nu * (11.0 * nu - 21.0)) / 8.0 -
                      5.0 * s12 * (10.0 * n2 - 9.0 * nu - 4.0) / 8.0 -
                      5.0 * s22 * (-18.0 * X2 * nu + X2 + 11.0 * n2 - 3.0 * nu - 1.0) / 8.0;
    h->q8c[1] = nu * (-693359375.0 * l5 - 643896.0 + 59326749.0 * l3 + 1516829440.0 * l2) / 3150.0;
    h->q8h = 5994461.0 * pi * nu / 12700800.0;
    h->q8c[2] = -6.0 * n4 + 24.0 * n3 / 7.0 +
                n2 * (-11712255859375.0 * l5 - 3391115364245.0 * l7 + 1755887616.0 + 8965819883403.0 * l3 +
                      22502063927296.0 * l2) / 1058400.0 +
                nu * (-43480265170944.0 * l2 - 10632236726043.0 * l3 + 10005778368.0 + 3391115364245.0 * l7 +
                      21877274609375.0 * l5) / 4233600.0;
    h->q6h = -2723471.0 * pi * nu / 756000.0;
    h->q6c[2] = 6.0 * n3 - 27.0 * n2 / 5.0 +
                nu * (-2358912.0 * l2 / 25.0 - 827.0 / 3.0 + 1399437.0 * l3 / 50.0 + 390625.0 * l5 / 18.0);
    h->q6c[3] = -14.0 * n4 + 116.0 * n3 +
                n2 * (-9996617728.0 * l2 - 408682503.0 * l3 + 6681738.0 + 4580078125.0 * l5) / 3150.0 +
                nu * (-5084375000.0 * l5 - 1249161912.0 * l3 + 23517747.0 + 13751491072.0 * l2) / 9450.0;
    h->q4h = 88703.0 * pi * nu / 1890.0;
    h->q4c[2] = -6.0 * n2 + 8.0 * nu;
    h->q4c[3] = 10.0 * n3 - 83.0 * n2 + 4.0 * nu * (-74358.0 * l3 - 3981.0 + 124064.0 * l2) / 45.0 + qs;
    h->q4c[4] = n3 * (640.0 - 615.0 * pi2 / 32.0) +
                n2 * (-9765625.0 * l5 / 126.0 - 6396489.0 * l3 / 70.0 - 1184.0 * eg / 5.0 + 31633.0 * pi2 / 512.0 +
                      150683.0 / 105.0 + 33693536.0 * l2 / 105.0) +
                nu * (-40979464.0 * l2 / 315.0 - 93031.0 * pi2 / 1536.0 + 10856.0 * eg / 105.0 + 1295219.0 / 350.0 +
                      9765625.0 * l5 / 504.0 + 14203593.0 * l3 / 280.0);
    h->q4l = 592.0 * n2 / 5.0 - 5428.0 * nu / 105.0;

    // ---- odd part: N = cS gS + nus gSstr + (chi1 X1 g31 + chi2 X2 g32) u^2 + soc u^4  (src/EOB.cu:98-104)
    const double cS = c1 * X1 * X1 + c2 * X2 * X2;
    const double nus = nu * (c1 + c2);
    const double g32 = s11 * (-4.0 * X2 - 1.0) / 12.0 + s12 * (0.166666666666667 * X2 - 0.583333333333333) +
                       s22 * (2.0 * X2 - 2.0) / 4.0;
    const double g31 = -0.5 * s11 * X2 + s12 * (-2.0 * X2 - 5.0) / 12.0 + s22 * (4.0 * X2 - 5.0) / 12.0;
    const double soc = dSO * (c1 * X1 + c2 * X2) +
                       (X1 - X2) * (c1 * X1 - c2 * X2) *
                           (7.0 * n4 / 512.0 + 31.0 * n3 / 512.0 + n2 * (208493.0 - 5136.0 * pi2) / 4608.0 -
                            nu * (-13288125.0 * pi2 + 13762560.0 * eg + 26542080.0 * l2 + 168816592.0) / 921600.0 +
                            1701.0 / 512.0);
    // gS[j][k] and gSs[j][k]: coefficient of pr^(2j) u^k; *_l: of pr^(2j) u^k log r
    double gS[5][5] = {{0}}, gSl[5][5] = {{0}}, gT[5][5] = {{0}}, gTl[5][5] = {{0}};
    gS[0][0] = 2.0;
    gS[0][1] = -5.0 * nu / 8.0;
    gS[0][2] = (-n2 - 102.0 * nu) / 8.0;
    gS[0][3] = (-63.0 * n3 + 13644.0 * n2 - 80399.0 * nu + 1446.0 * pi2 * nu) / 1152.0;
    gSl[0][4] = 584.0 * nu / 15.0;
    gS[1][0] = -27.0 * nu / 8.0;
    gS[1][1] = (23.0 * n2 - 84.0 * nu) / 8.0;
    gS[1][2] = (69.0 * n3 + 6228.0 * n2 - 5283.0 * nu) / 64.0;
    gS[1][3] = (14400.0 * n4 - 2477700.0 * n3 - 326100.0 * pi2 * n2 + 19813300.0 * n2 - 89579520.0 * nu * l3 -
                1672575.0 * pi2 * nu - 3993600.0 * eg * nu + 54396338.0 * nu + 83824640.0 * nu * l2) / 19200.0;
    gSl[1][3] = 1996800.0 * nu / 19200.0;
    gS[2][0] = (35.0 * n2 + 5.0 * nu) / 8.0;
    gS[2][1] = (-771.0 * n3 + 3324.0 * n2 + 781.0 * nu) / 128.0;
    gS[2][2] = (-38520.0 * n4 - 3309615.0 * n3 + 2872170.0 * n2 - 1626767360.0 * nu * l2 + 19954938.0 * nu +
                1008889344.0 * nu * l3) / 11520.0;
    gS[3][0] = -(665.0 * n3 + 252.0 * n2 - 7.0 * nu) / 128.0;
    gS[3][1] = (567720.0 * n4 - 2564325.0 * n3 - 1148850.0 * n2 - 28998570240.0 * nu * l3 - 19300000000.0 * nu * l5 +
                175835718.0 * nu + 90521206784.0 * nu * l2) / 57600.0;
    gS[4][0] = (7144200.0 * n4 + 4465125.0 * n3 + 935550.0 * n2 - 11506980454400.0 * nu * l2 -
                188268367392.0 * nu * l3 + 3476909988.0 * nu + 5082137500000.0 * nu * l5) / 1209600.0;

    gT[0][0] = 3.0 / 2.0;
    gT[0][1] = 3.0 * (-2.0 * nu - 3.0) / 8.0;
    gT[0][2] = 3.0 * (-n2 - 52.0 * nu - 9.0) / 16.0;
    gT[0][3] = (-36.0 * n3 + 4266.0 * n2 - 15254.0 * nu + 492.0 * pi2 * nu - 1215.0) / 384.0;
    gTl[0][4] = 24.0 * nu;
    gT[1][0] = 3.0 * (-6.0 * nu - 5.0) / 8.0;
    gT[1][1] = 3.0 * (19.0 * n2 - 12.0 * nu + 23.0) / 16.0;
    gT[1][2] = 3.0 * (36.0 * n3 + 1574.0 * n2 - 558.0 * nu - 15.0) / 64.0;
    gT[1][3] = (5130.0 * n4 - 469440.0 * n3 - 59040.0 * pi2 * n2 + 2316030.0 * n2 - 12317184.0 * nu * l3 -
                72435.0 * pi2 * nu - 393216.0 * eg * nu + 5731444.0 * nu + 12025856.0 * nu * l2 - 3240.0) / 3840.0;
    gTl[1][3] = 196608.0 * nu / 3840.0;
    gT[2][0] = (45.0 * n2 + 40.0 * nu + 35.0) / 16.0;
    gT[2][1] = (-972.0 * n3 + 702.0 * n2 - 106.0 * nu - 1105.0) / 128.0;
    gT[2][2] = (-20655.0 * n4 - 834300.0 * n3 + 182025.0 * n2 - 381263872.0 * nu * l2 + 3596448.0 * nu +
                237385728.0 * nu * l3 + 37875.0) / 3840.0;
    gT[3][0] = -(420.0 * n3 + 462.0 * n2 + 350.0 * nu + 315.0) / 128.0;
    gT[3][1] = (2170395.0 * n4 - 1291140.0 * n3 - 593325.0 * n2 - 62204578560.0 * nu * l3 - 40300000000.0 * nu * l5 +
                343473264.0 * nu + 191671894016.0 * nu * l2 + 2399625.0) / 172800.0;
    gT[4][0] = (4465125.0 * n4 + 5953500.0 * n3 + 4975425.0 * n2 - 8132450787328.0 * nu * l2 - 90415828800.0 * nu * l3 +
                2254036356.0 * nu + 3562775000000.0 * nu * l5 + 3274425.0) / 1209600.0;
    for (int j = 0; j < 5; ++j)
        for (int k = 0; k < 5; ++k) {
            h->nc[j][k] = cS * gS[j][k] + nus * gT[j][k];
            h->ncl[j][k] = cS * gSl[j][k] + nus * gTl[j][k];
        }
    h->nc[0][2] += c1 * X1 * g31 + c2 * X2 * g32;
    h->nc[0][4] += soc;
    HamCoeffs::Derived &d = h->d;
    d.ak0l6 = 6.0 * h->ak0l[6];
    d.ak0l5 = 5.0 * h->ak0l[5];
    d.ak0h = 6.5 * h->ak0h;
    d.fa2 = 2.0 * h->fa2;
    d.as6 = 6.0 * h->as6;
    d.as5 = 5.0 * h->as5;
    d.as4 = 4.0 * h->as4;
    d.dbl5 = 5.0 * h->dbl[5];
    d.dbl4 = 4.0 * h->dbl[4];
    d.dbh = 5.5 * h->dbh;
    d.bs4 = 4.0 * h->bs4;
    d.bs3 = 3.0 * h->bs3;
    d.two_ap2 = 2.0 * h->ap2;
    d.q4c4 = 4.0 * h->q4c[4];
    d.q4c3 = 3.0 * h->q4c[3];
    d.q4c2 = 2.0 * h->q4c[2];
    d.q4h = 4.5 * h->q4h;
    d.q6h = 3.5 * h->q6h;
    d.q6c3 = 3.0 * h->q6c[3];
    d.q6c2 = 2.0 * h->q6c[2];
    d.q8h = 2.5 * h->q8h;
    d.q8c2 = 2.0 * h->q8c[2];
    d.nc02 = 2.0 * h->nc[0][2];
    d.nc03 = 3.0 * h->nc[0][3];
    d.nc04 = 4.0 * h->nc[0][4];
    d.nc12 = 2.0 * h->nc[1][2];
    d.nc13 = 3.0 * h->nc[1][3];
    d.four_n4 = 4.0 * h->nc[4][0];
    d.two_nu = 2.0 * h->nu;
}

// ---------------------------------------------------------------------------
// Generic evaluation, templated on the scalar type so that the oracle and the
// initial-condition solver can differentiate it with dual numbers.
// Returns Heff; H follows from ham_H_from_heff.
template <class T>
EOB_HD T ham_heff(const HamCoeffs &h, const T &r, const T &pr, const T &L)
{
    const T u = 1.0 / r;
    const T lr = log(r);
    const T su = sqrt(u);
    const T u2 = u * u, u3 = u2 * u, u4 = u3 * u, u5 = u4 * u, u6 = u5 * u;
    const T upow[7] = {T(1.0), u, u2, u3, u4, u5, u6};
    T ak0 = T(h.ak0h) * u6 * su, aka = T(0.0), db = T(h.dbh) * u5 * su;
    for (int k = 0; k < 7; ++k) {
        ak0 = ak0 + (h.ak0[k] + h.ak0l[k] * lr) * upow[k];
        aka = aka + h.aka[k] * upow[k];
    }
    for (int k = 0; k < 6; ++k) db = db + (h.db[k] + h.dbl[k] * lr) * upow[k];
    const T dc = 1.0 + h.ap2 * u2 + 2.0 * h.ap2 * u3;
    const T fa = 1.0 + h.fa1 * u + h.fa2 * u2;
    const T as = 1.0 + h.as4 * u4 + h.as5 * u5 + h.as6 * u6;
    const T A = (ak0 + aka) * fa * as / dc;
    const T bnp = ak0 * db * (1.0 + h.kb * u) + h.bs3 * u3 + h.bs4 * u4 - 1.0 + h.ap2 * u2;
    const T bnpa = -u2 * (1.0 + 2.0 * u) / dc;
    const T cu = u2 * (1.0 + h.apsq * bnpa);
    const T q4 = h.q4c[2] * u2 + h.q4c[3] * u3 + h.q4c[4] * u4 + h.q4l * u4 * lr + h.q4h * u4 * su;
    const T q6 = h.q6c[2] * u2 + h.q6c[3] * u3 + h.q6h * u3 * su;
    const T q8 = h.q8c[1] * u + h.q8c[2] * u2 + h.q8h * u2 * su;
    const T p2 = pr * pr;
    const T W = 1.0 + p2 * (1.0 + bnp) + L * L * cu + p2 * p2 * (q4 + p2 * (q6 + p2 * q8));
    T N = T(0.0);
    for (int j = 4; j >= 0; --j) {
        T nj = T(0.0);
        for (int k = 0; k < 5; ++k) nj = nj + (h.nc[j][k] + h.ncl[j][k] * lr) * upow[k];
        N = N * p2 + nj;
    }
    const T hodd = L * u3 * N / dc;
    return sqrt(A * W) + hodd;
}

template <class T>
EOB_HD T ham_H_from_heff(const HamCoeffs &h, const T &heff)
{
    return h.M * sqrt(1.0 + 2.0 * h.nu * (heff - 1.0)) / h.nu;
}

}  // namespace eob
