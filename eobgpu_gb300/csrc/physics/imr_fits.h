// Fits of the merger-ringdown completion of the SEOBNRv4HM waveform, shared
// by the CUDA kernels and the host oracle.
//
// * NR fits of the modes at their attachment point (the reference's
//   eob/seobnrv4phm.py:878-1463; Bohe et al. 2017, PRD 95, 044028, and Cotesta
//   et al. 2018, PRD 98, 084028, App. B): time of the (2,2) attachment
//   relative to the peak of the orbital frequency, |h_lm|, its first and
//   second time derivatives, the mode frequency and its derivative.
// * Ringdown ansatz coefficients (eob/eobstuff.py:44-342; Cotesta et al.
//   2018, App. C): the free amplitude and phase coefficients.
// * Remnant: final mass (the SEOBNRv4 formula of eob/eobstuff.py:6-20 with the
//   Kerr ISCO of Bardeen, Press & Teukolsky 1972), final spin (Hofmann,
//   Barausse & Rezzolla 2016, ApJL 825, L19, the nM = 3, nJ = 4 fit), and the
//   fundamental Kerr quasi-normal modes from a table of Leaver's continued
//   fractions (qnm_table.h).
//
// The fit coefficients are the published ones, identical to the reference's;
// the layout (one function per quantity, switch on the mode) is ours.
// Masses m1, m2 need not be normalised; spins are aligned components.
#pragma once
#include "fac_coeffs.h"
#include "qnm_table.h"

namespace eob {

// Time of the (2,2) attachment before the peak of the orbital frequency
// [M]; the (5,5) mode attaches 10 M earlier (the caller adds 10).
EOB_HD double nr_delta_t22(double m1, double m2, double chi1, double chi2)
{
    const double eta = m1 * m2 / (m1 + m2) / (m1 + m2);
    const double chi = 0.5 * (chi1 + chi2) + 0.5 * (chi1 - chi2) * (m1 - m2) / (m1 + m2) / (1.0 - 2.0 * eta);
    const double e2 = eta * eta, e3 = e2 * eta, c2 = chi * chi, c3 = c2 * chi;
    return 2.50499 + 13.0064 * chi + 11.5435 * c2 + 45.8838 * eta - 40.3183 * eta * chi - 19.0538 * eta * c3 +
           13.0879 * e2 + 0.192775 * e2 * c3 - 716.044 * e3;
}

// the combination of a test-particle fit fTPL, an equal-mass fit fEQ and a
// global coefficient A1 that recovers both limits exactly
EOB_HD double tpl_eqm_combine(double eta, double A1, double fEQ, double fTPL)
{
    const double A0 = -0.00099601593625498 * A1 - 0.00001600025600409607 * fEQ + 1.000016000256004 * fTPL;
    const double A2 = -3.984063745019967 * A1 + 16.00025600409607 * fEQ - 16.0002560041612 * fTPL;
    return A0 + A1 * eta + A2 * (eta * eta);
}

struct NrSpins {
    double eta, dM, chi, chiS, chiA;
};

// the fits assume m1 >= m2: otherwise the bodies are swapped (chiA changes sign)
EOB_HD NrSpins nr_spins(double m1, double m2, double chiS, double chiA)
{
    NrSpins s;
    s.eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
    s.dM = sqrt(1.0 - 4.0 * s.eta);
    if (m1 < m2) {
        const double t = m1;
        m1 = m2;
        m2 = t;
        chiA = -chiA;
    }
    s.chiS = chiS;
    s.chiA = chiA;
    s.chi = chiS + chiA * (m1 - m2) / (m1 + m2) / (1.0 - 2.0 * s.eta);
    return s;
}

// |h_lm| / M at the attachment point (the caller takes the absolute value)
EOB_HD double nr_peak_amp(int l, int m, double m1, double m2, double chiS, double chiA)
{
    const NrSpins s = nr_spins(m1, m2, chiS, chiA);
    const double eta = s.eta, dM = s.dM, chi = s.chi, e2 = eta * eta;
    const double chi21 = s.chiS * dM / (1.0 - 1.3 * eta) + s.chiA;
    const double chi33 = s.chiS * dM + s.chiA;
    const double chi44 = s.chiS * (1 - 5 * eta) + s.chiA * dM;
    const double c2 = chi * chi, c3 = chi * c2;
    if (l == 2 && m == 2) {
        const double fTPL = 1.4528573105413543 + 0.16613449160880395 * chi + 0.027355646661735258 * c2 -
                            0.020072844926136438 * c3;
        const double fEQ = 1.577457498227 - 0.0076949474494639085 * chi + 0.02188705616693344 * c2 +
                           0.023268366492696667 * c3;
        const double A1 = -0.03442402416125921 + -1.218066264419839 * chi + -0.5683726304811634 * c2 +
                          0.4011143761465342 * c3;
        return eta * tpl_eqm_combine(eta, A1, fEQ, fTPL);
    }
    if (l == 2 && m == 1)
        return -((0.29256703361640224 - 0.19710255145276584 * eta) * eta * chi21 +
                 dM * eta *
                     (-0.42817941710649793 + 0.11378918021042442 * eta - 0.7736772957051212 * e2 +
                      chi21 * chi21 * (0.047004057952214004 - eta * 0.09326128322462478)) +
                 dM * eta * chi21 * (-0.010195081244587765 + 0.016876911550777807 * chi21 * chi21));
    if (l == 3 && m == 3)
        return (0.10109183988848384 * eta - 0.4704095462146807 * e2 + 1.0735457779890183 * e2 * eta) * chi33 +
               dM * (0.5636580081367962 * eta - 0.054609013952480856 * e2 + 2.3093699480319234 * e2 * eta +
                     chi33 * chi33 * (0.029812986680919126 * eta - 0.09688097244145283 * e2));
    if (l == 4 && m == 4)
        return eta * (0.2646580063832686 + 0.067584186955327 * chi44 + 0.02925102905737779 * chi44 * chi44) +
               e2 * (-0.5658246076387973 - 0.8667455348964268 * chi44 + 0.005234192027729502 * chi44 * chi44) +
               eta * e2 * (-2.5008294352355405 + 6.880772754797872 * chi44 - 1.0234651570264885 * chi44 * chi44) +
               e2 * e2 * (7.6974501716202735 - 16.551524307203252 * chi44);
    if (l == 5 && m == 5)
        return 0.128621 * dM * eta - 0.474201 * dM * eta * eta + 1.0833 * dM * eta * eta * eta +
               0.0322784 * eta * chi33 - 0.134511 * chi33 * eta * eta + 0.0990202 * chi33 * eta * eta * eta;
    return 0.0;
}

// d|h_lm|/dt at the attachment point
EOB_HD double nr_peak_adot(int l, int m, double m1, double m2, double chiS, double chiA)
{
    const NrSpins s = nr_spins(m1, m2, chiS, chiA);
    const double eta = s.eta, dM = s.dM, dM2 = dM * dM, e2 = eta * eta;
    const double chi21 = s.chiS * dM / (1.0 - 2.0 * eta) + s.chiA;
    const double chi33 = s.chiS * dM + s.chiA;
    const double chi44 = s.chiS * (1 - 7 * eta) + s.chiA * dM;
    if (l == 2 && m == 2) return 0.0;
    if (l == 2 && m == 1)
        return dM * eta * (0.007147528020812309 - eta * 0.035644027582499495) +
               dM * eta * chi21 * (-0.0087785131749995 + eta * 0.03054672006241107) +
               eta * 0.00801714459112299 *
                   fabs(-dM * (0.7875612917853588 + eta * 1.161274164728927 + e2 * 11.306060006923605) + chi21);
    if (l == 3 && m == 3)
        return dM * eta * (-0.00309943555972098 + eta * 0.010076527264663805) * chi33 * chi33 +
               eta * 0.0016309606446766923 *
                   sqrt(dM2 * (8.811660714437027 + 104.47752236009688 * eta) +
                        dM * chi33 * (-5.352043503655119 + eta * 49.68621807460999) + chi33 * chi33);
    if (l == 4 && m == 4)
        return eta * (0.004347588211099233 - 0.0014612210699052148 * chi44 - 0.002428047910361957 * chi44 * chi44) +
               e2 * (0.023320670701084355 - 0.02240684127113227 * chi44 + 0.011427087840231389 * chi44 * chi44) +
               eta * e2 * (-0.46054477257132803 + 0.433526632115367 * chi44) +
               e2 * e2 * (1.2796262150829425 - 1.2400051122897835 * chi44);
    if (l == 5 && m == 5)
        return eta * (dM * (-0.008389798844109389 + 0.04678354680410954 * eta) +
                      dM * chi33 * (-0.0013605616383929452 + 0.004302712487297126 * eta) +
                      dM * chi33 * chi33 * (-0.0011412109287400596 + 0.0018590391891716925 * eta) +
                      0.0002944221308683548 * fabs(dM * (37.11125499129578 - 157.79906814398277 * eta) + chi33));
    return 0.0;
}

// d^2|h_lm|/dt^2 at the attachment point
EOB_HD double nr_peak_addot(int l, int m, double m1, double m2, double chiS, double chiA)
{
    const NrSpins s = nr_spins(m1, m2, chiS, chiA);
    const double eta = s.eta, dM = s.dM, chi = s.chi, e2 = eta * eta;
    const double chi21 = s.chiS * dM / (1.0 - 2.0 * eta) + s.chiA;
    const double chi33 = s.chiS * dM + s.chiA;
    const double cm1 = -1.0 + chi;
    if (l == 2 && m == 2) {
        const double fTPL = 0.002395610769995033 * cm1 - 0.00019273850675004356 * cm1 * cm1 -
                            0.00029666193167435337 * cm1 * cm1 * cm1;
        const double fEQ = -0.004126509071377509 + 0.002223999138735809 * chi;
        const double A1 = -0.005776537350356959 + 0.001030857482885267 * chi;
        return eta * tpl_eqm_combine(eta, A1, fEQ, fTPL);
    }
    if (l == 2 && m == 1)
        return eta * dM * 0.00037132201959950333 -
               fabs(dM * eta * (-0.0003650874948532221 - eta * 0.003054168419880019) +
                    dM * eta * chi21 * chi21 *
                        (-0.0006306232037821514 - eta * 0.000868047918883389 + e2 * 0.022306229435339213) +
                    eta * chi21 * chi21 * chi21 * 0.0003402427901204342 + dM * eta * chi21 * 0.00028398490492743);
    if (l == 3 && m == 3)
        return dM * eta * (0.0009605689249339088 - 0.00019080678283595965 * eta) * chi33 -
               0.00015623760412359145 * eta *
                   fabs(dM * (4.676662024170895 + 79.20189790272218 * eta - 1097.405480250759 * e2 +
                              6512.959044311574 * eta * e2 - 13263.36920919937 * e2 * e2) +
                        chi33);
    if (l == 4 && m == 4)
        return eta * (-0.000301722928925693 + 0.0003215952388023551 * chi) +
               e2 * (0.006283048344165004 + 0.0011598784110553046 * chi) +
               e2 * eta * (-0.08143521096050622 - 0.013819464720298994 * chi) +
               e2 * e2 * (0.22684871200570564 + 0.03275749240408555 * chi);
    if (l == 5 && m == 5)
        return eta * (dM * (0.00012727220842255978 + 0.0003211670856771251 * eta) +
                      dM * chi33 * (-0.00006621677859895541 + 0.000328855327605536 * eta) +
                      chi33 * chi33 * (-0.00005824622885648688 + 0.00013944293760663706 * eta));
    return 0.0;
}

// mode frequency at the attachment point (chi = the caller's effective spin)
EOB_HD double nr_peak_omega(int l, int m, double eta, double chi)
{
    const double e2 = eta * eta;
    if (l == 2 && m == 2) {
        const double c0 = 0.5626787200433265, c1 = -0.08706198756945482, cc2 = 25.81979479453255,
                     cc3 = 25.85037751197443, d2 = 7.629921628648589, d3 = 10.26207326082448,
                     c4 = 0.00174345193125868;
        const double A4 = d2 + 4 * (d2 - cc2) * (eta - 0.25);
        const double A3 = d3 + 4 * (d3 - cc3) * (eta - 0.25);
        return c0 + (c1 + c4 * chi) * log(A3 - A4 * chi);
    }
    if (l == 2 && m == 1)
        return 0.1743194440996283 + eta * 0.1938944514123048 + 0.1670063050527942 * e2 +
               0.053508705425291826 * chi - eta * chi * 0.18460213023455802 + e2 * chi * 0.2187305149636044 +
               chi * chi * 0.030228846150378793 - eta * chi * chi * 0.11222178038468673;
    if (l == 3 && m == 3)
        return 0.3973947703114506 + 0.16419332207671075 * chi + 0.1635531186118689 * chi * chi +
               0.06140164491786984 * chi * chi * chi +
               eta * (0.6995063984915486 - 0.3626744855912085 * chi - 0.9775469868881651 * chi * chi) +
               e2 * (-0.3455328417046369 + 0.31952307610699876 * chi + 1.9334166149686984 * chi * chi);
    if (l == 4 && m == 4)
        return 0.5389359134370971 + 0.16635177426821202 * chi + 0.2075386047689103 * chi * chi +
               0.15268115749910835 * chi * chi * chi +
               eta * (0.7617423831337586 + 0.009587856087825369 * chi - 1.302303785053009 * chi * chi -
                      0.5562751887042064 * chi * chi * chi) +
               e2 * (0.9675153069365782 - 0.22059322127958586 * chi + 2.678097398558074 * chi * chi) -
               e2 * eta * 4.895381222514275;
    if (l == 5 && m == 5)
        return 0.6437545281817488 + 0.22315530037902315 * chi + 0.2956893357624277 * chi * chi +
               0.17327819169083758 * chi * chi * chi +
               eta * (-0.47017798518175785 - 0.3929010618358481 * chi - 2.2653368626130654 * chi * chi -
                      0.5512998466154311 * chi * chi * chi) +
               e2 * (2.311483807604238 + 0.8829339243493562 * chi + 5.817595866020152 * chi * chi);
    return 0.0;
}

// time derivative of the mode frequency at the attachment point
EOB_HD double nr_peak_omegadot(int l, int m, double eta, double chi)
{
    const double e2 = eta * eta;
    if (l == 2 && m == 2) {
        const double fTPL = -0.011209791668428353 +
                            (0.0040867958978563915 + 0.0006333925136134493 * chi) *
                                log(68.47466578100956 - 58.301487557007206 * chi);
        const double fEQ = 0.01128156666995859 + 0.0002869276768158971 * chi;
        const double A1 = 0.01574321112717377 + 0.02244178140869133 * chi;
        return tpl_eqm_combine(eta, A1, fEQ, fTPL);
    }
    if (l == 2 && m == 1)
        return 0.0070987396362959514 + eta * 0.024816844694685373 - e2 * 0.050428973182277494 +
               eta * e2 * 0.03442040062259341 - chi * 0.0017751850002442097 + eta * chi * 0.004244058872768811 -
               e2 * chi * 0.031996494883796855 - chi * chi * 0.0035627260615894584 +
               eta * chi * chi * 0.01471807973618255 - chi * chi * chi * 0.0019020967877681962;
    if (l == 3 && m == 3)
        return 0.010337157192240338 - 0.0053067782526697764 * chi * chi - 0.005087932726777773 * chi * chi * chi +
               eta * (0.027735564986787684 + 0.018864151181629343 * chi + 0.021754491131531044 * chi * chi +
                      0.01785477515931398 * chi * chi * chi) +
               e2 * (0.018084233854540898 - 0.08204268775495138 * chi);
    if (l == 4 && m == 4)
        return 0.013997911323773867 - 0.0051178205260273574 * chi - 0.0073874256262988 * chi * chi +
               eta * (0.0528489379269367 + 0.01632304766334543 * chi + 0.02539072293029433 * chi * chi) +
               e2 * (-0.06529992724396189 + 0.05782894076431308 * chi);
    if (l == 5 && m == 5)
        return 0.01763430670755021 - 0.00024925743340389135 * chi - 0.009240404217656968 * chi * chi -
               0.007907831334704586 * chi * chi * chi +
               eta * (-0.1366002854361568 + 0.0561378177186783 * chi + 0.16406275673019852 * chi * chi +
                      0.07736232247880881 * chi * chi * chi) +
               e2 * (0.9875890632901151 - 0.31392112794887855 * chi - 0.5926145463423832 * chi * chi) -
               1.6943356548192614 * e2 * eta;
    return 0.0;
}

// ---- ringdown ansatz: the free coefficients c1f, c2f (amplitude) and d1f,
// d2f (phase), each a sum of k_ij eta^i chi^j over the terms the fit has, in
// the reference's order of summation
struct RdTerms {
    double k00, k01, k02, k12, k10, k11, k20, k21, k31;  // k12: eta chi^2
};

EOB_HD double rd_eval(const RdTerms &k, double eta, double chi)
{
    return k.k00 + k.k01 * chi + k.k02 * chi * chi + k.k12 * chi * chi * eta + k.k10 * eta + k.k11 * eta * chi +
           k.k20 * eta * eta + k.k21 * eta * eta * chi + k.k31 * eta * eta * eta * chi;
}

EOB_HD int rd_mode(int l, int m) { return (l == 2 && m == 2) ? 0 : (l == 2 && m == 1) ? 1 : (l == 3) ? 2 : (l == 4) ? 3 : 4; }

// which = 0: c1f, 1: c2f, 2: d1f, 3: d2f
EOB_HD RdTerms rd_terms(int which, int l, int m)
{
    const int q = rd_mode(l, m);
    // rows: k00, k01, k02, k12, k10, k11, k20, k21, k31
    const double c1[5][9] = {
        {0.0830664, -0.0196758, -0.0136459, 0.0, 0.0612892, 0.00146142, -0.0893454, 0.0, 0.0},
        {0.07780330893915006, -0.05070638166864379, 0.0, 0.0, 0.24091006920322164, 0.38582622780596576,
         -0.7456327888190485, -0.9695534075470388, 0.0},
        {0.07638733045623343, -0.030993441267953236, 0.0, 0.0, 0.2543447497371546, 0.2516879591102584,
         -1.0892686061231245, -0.7980907313033606, 0.0},
        {-0.06392710223439678, -0.03646167590514318, 0.0, 0.0, 0.345195277237925, 1.2777441574118558,
         -1.764352185878576, -14.825262897834696, 40.67135475479875},
        {-0.06704614393611373, 0.021905949257025503, 0.0, 0.0, -0.24754936787743445, -0.0943771022698497,
         0.7588042862093705, 0.4357768883690394, 0.0}};
    const double c2[5][9] = {
        {-0.623953, -0.371365, 0.0, 0.0, 1.39777, 2.40203, -1.82173, -5.25339, 0.0},
        {-1.2451852641667298, -1.195786238319961, 0.0, 0.0, 6.134202504312409, 15.66696619631313,
         -14.67251127485556, -44.41982201432511, 0.0},
        {-0.8325292359346013, -0.598880303198448, 0.0, 0.0, 2.767989795032018, 5.904371617277156,
         -7.028151926115957, -18.232606706124482, 0.0},
        {0.7813275473485185, 0.8094706044462984, 0.0, 0.0, -5.18689829943586, -5.38343327318501,
         14.026415859369477, 0.1051625997942299, 46.978434956814006},
        {1.6763424265367357, 0.4925695499534606, 0.0, 0.0, -5.604559311983177, -6.209095657439377,
         16.751319143123386, 16.778452555342554, 0.0}};
    const double d1[5][9] = {
        {0.147584, 0.00779176, -0.0244358, 0.0, 0.263456, -0.120853, -0.808987, 0.0, 0.0},
        {0.15601401627613815, 0.10219957917717622, 0.0, 0.0, 0.023346852452720928, -0.9435308286367039,
         0.15326558178697175, 1.7979082057513565, 0.0},
        {0.11085299117493969, 0.018959099261813613, 0.0, 0.0, 0.9999800463662053, -0.729149797691242,
         -3.3983315694441125, 2.5192011762934037, 0.0},
        {0.11498976343440313, 0.008389519706605305, 0.0, 0.0, 1.6126522800609633, -0.8069979888526699,
         -6.255895564079467, 7.595651881827078, -19.32367406125053},
        {0.16465380962882128, -0.026574817803812007, 0.0, 0.0, -0.19184523794508765, -0.05519618962738479,
         0.33328424135336965, 0.3194274548351241, 0.0}};
    const double d2[5][9] = {
        {2.46654, 3.13067, 0.581626, 0.0, -6.99396, -9.61861, 17.5646, 0.0, 0.0},
        {2.7886287922318105, 4.29290053494256, 2.5582321247274726, -10.232928498772893, -0.8145406685320334,
         -15.93796979597706, 5.549338798935832, 12.649775582333442, 0.0},
        {2.7825237371542735, 2.8796835808075003, 0.0, 0.0, -7.844741660437831, -34.7670039322078,
         27.181024362399302, 127.13948436435182, 0.0},
        {3.111817347262856, 5.399341180960216, 2.3832321567874686, -9.532928476043567, 15.885333959709488,
         -87.92421137153823, -79.64931908155609, 657.7156442271963, -1555.2968529739226},
        {11.102447263357977, 6.015112119742853, 0.0, 0.0, -58.605776859097084, -81.68032025902797,
         176.60643662729498, 266.47345742836745, 0.0}};
    const double(*t)[9] = which == 0 ? c1 : which == 1 ? c2 : which == 2 ? d1 : d2;
    return {t[q][0], t[q][1], t[q][2], t[q][3], t[q][4], t[q][5], t[q][6], t[q][7], t[q][8]};
}

EOB_HD double rd_coeff(int which, int l, int m, double eta, double chi) { return rd_eval(rd_terms(which, l, m), eta, chi); }

// ---- remnant
// Kerr ISCO radius [M] for dimensionless spin a (prograde for a > 0)
EOB_HD double kerr_isco_radius(double a)
{
    const double z1 = 1.0 + cbrt(1.0 - a * a) * (cbrt(1.0 + a) + cbrt(1.0 - a));
    const double z2 = sqrt(3.0 * a * a + z1 * z1);
    const double sg = (a > 0.0) ? 1.0 : (a < 0.0 ? -1.0 : 0.0);
    return 3.0 + z2 - sg * sqrt((3.0 - z1) * (3.0 + z1 + 2.0 * z2));
}

// specific energy of the ISCO at radius r: sqrt(1 - 2 / (3 r))
EOB_HD double kerr_isco_energy(double r) { return sqrt(1.0 - 2.0 / (3.0 * r)); }

// final mass / M (eob/eobstuff.py:6-20): masses, aligned spins a1 (of m1), a2
EOB_HD double final_mass_seobnrv4(double m1, double m2, double a1, double a2)
{
    const double q = m1 / m2;
    const double eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
    const double iq = 1.0 / q, opiq = 1.0 + iq, iq2 = iq * iq;
    const double atl = (a1 + a2 * iq2) / (opiq * opiq);
    const double eisco = kerr_isco_energy(kerr_isco_radius(atl));
    return 1.0 - ((1.0 - eisco) * eta +
                  16.0 * eta * eta *
                      (0.00258 - 0.0773 / (1.0 / ((1.0 + iq2) / (opiq * opiq)) * atl - 1.6939) - 0.25 * (1.0 - eisco)));
}

// final spin of an aligned-spin binary (Hofmann, Barausse & Rezzolla 2016,
// eqs. 13-16, nM = 3, nJ = 4 coefficients of their Table 1):
// a_f = a_tot + eta l(a_eff), l = L_isco(a_eff) - 2 a_tot (E_isco(a_eff) - 1)
// + sum_ij k_ij eta^(1 + i) a_eff^j, a_tot = (a1 + a2 q^2) / (1 + q)^2 with
// q = m2 / m1 <= 1, a_eff = a_tot + xi eta (a1 + a2).
EOB_HD double final_spin_hbr2016(double m1, double m2, double a1, double a2)
{
    if (m2 > m1) {
        double t = m1; m1 = m2; m2 = t;
        t = a1; a1 = a2; a2 = t;
    }
    const double k[4][5] = {{-5.97723, 3.39221, 4.48865, -5.77101, -13.0459},
                            {35.1278, -72.9336, -86.0036, 93.7371, 200.975},
                            {-146.822, 387.184, 447.009, -467.383, -884.339},
                            {223.911, -648.502, -697.177, 753.738, 1166.89}};
    const double xi = 0.474046;
    const double q = m2 / m1;
    const double eta = m1 * m2 / ((m1 + m2) * (m1 + m2));
    const double atot = (a1 + a2 * q * q) / ((1.0 + q) * (1.0 + q));
    const double aeff = atot + xi * eta * (a1 + a2);
    const double r = kerr_isco_radius(aeff);
    const double Lisco = 2.0 / (3.0 * sqrt(3.0)) * (1.0 + 2.0 * sqrt(3.0 * r - 2.0));
    const double Eisco = kerr_isco_energy(r);
    double sum = 0.0, ei = eta;
    for (int i = 0; i < 4; ++i) {
        double aj = 1.0;
        for (int j = 0; j < 5; ++j) {
            sum += k[i][j] * ei * aj;
            aj *= aeff;
        }
        ei *= eta;
    }
    const double ell = Lisco - 2.0 * atot * (Eisco - 1.0) + sum;
    return atot + eta * ell;
}

static constexpr double kQnmTabH[5][kQnmN][2] = EOB_QNM_INIT;
#ifdef __CUDACC__
__device__ const double kQnmTabD[5][kQnmN][2] = EOB_QNM_INIT;
#endif

EOB_HD double qnm_node(int q, int i, int c)
{
#ifdef __CUDA_ARCH__
    return kQnmTabD[q][i][c];
#else
    return kQnmTabH[q][i][c];
#endif
}

// fundamental QNM M_f omega_lm at spin af (for unit remnant mass), four-point
// Lagrange interpolation of the Leaver table in sqrt(1 - af); e^{-i omega t},
// im < 0
EOB_HD void qnm_lookup(int l, int m, double af, double *re, double *im)
{
    const int q = rd_mode(l, m);
    const double x = (sqrt(1.0 - af) - kQnmX0) / kQnmDx;
    int i = (int)floor(x) - 1;
    if (i < 0) i = 0;
    if (i > kQnmN - 4) i = kQnmN - 4;
    const double u = x - i;  // position among the four points i .. i + 3
    const double w0 = -(u - 1) * (u - 2) * (u - 3) / 6.0, w1 = u * (u - 2) * (u - 3) / 2.0,
                 w2 = -u * (u - 1) * (u - 3) / 2.0, w3 = u * (u - 1) * (u - 2) / 6.0;
    *re = w0 * qnm_node(q, i, 0) + w1 * qnm_node(q, i + 1, 0) + w2 * qnm_node(q, i + 2, 0) + w3 * qnm_node(q, i + 3, 0);
    *im = w0 * qnm_node(q, i, 1) + w1 * qnm_node(q, i + 1, 1) + w2 * qnm_node(q, i + 2, 1) + w3 * qnm_node(q, i + 3, 1);
}

}  // namespace eob
