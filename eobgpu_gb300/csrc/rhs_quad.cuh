// One binary on four warps (a warp quad, one warp on each SM sub-partition):
// the right-hand side of the EOB equations in pieces that four FP64 pipes
// evaluate side by side.  It extends the warp pair (rhs_pair.cuh) for the few
// binaries whose sequential chains set a batch's time:
//
//   stage           warp 0              warp 1              warp 2              warp 3
//   jets            log r               polynomial parts    sqrt(u) polynomials log polynomials
//                                                           and sqrt(u)
//   combination a   1/Dc, A(u)          1/Dc, c(u),         B_np, q, W - L^2 c  N(u, p_r^2)
//                                       q part of dW/dp_r
//   combination b   even part sqrt(AW)  odd part            --                  y_2/y_3, 1/(8 pi nu)
//   H, flux set-up  H and gradient,     m factors from      omega, v = omega    omega, log v,
//                   v_phi^2             H_real omega = M^2 D r_omega^2, v^12, S_o H_real, S_even
//   multipoles      series part 0..15   m-factor and v_phi  series part 16..34  m-factor and v_phi
//                   (two lanes each)    part 0..31                              part 32..34
//   (then each multipole's two parts multiplied and summed)
//
// Values cross through shared memory at six barriers per right-hand side
// (an mbarrier of 128 arrivals with the pair's time limit).  As for the pair,
// every value more than one warp uses afterwards is read by all of them from
// shared memory, so the four warps' results and control decisions agree bit
// for bit.
#pragma once
#include "rhs_pair.cuh"

namespace eob {

struct QuadXchg {
    double jet[3][2][32];  // jets: [log polynomial, polynomial, sqrt part][v, d][lane]
    double lr;             // warp 0: log r
    double su[2];          // warp 2: sqrt(u) = 1/sqrt(r), r sqrt(u) / 2
    double pa[2][32];      // warp 0: A, dA/du
    double pc[2][32];      // warp 1: c, dc/du
    double pw[3][32];      // warp 2: W - L^2 c and its u-derivative, the B_np part of dW/dp_r
    double pwq[32];        // warp 1: the q part of dW/dp_r
    double pn[3][32];      // warp 3: N, dN/du, dN/dp_r^2
    double ev[4][32];      // warp 0: even part of H_eff and its derivatives
    double od[4][32];      // warp 1: odd part
    double ham[3];         // warp 0: dH/dr, dH/dp_r, dH/dL at the state
    double fl[16];         // v, log v, v^12, S_e^2, S_o^2, v_phi^2, v^5, v^2
    double T[8], k4[8];    // warp 1: m factors, m = 1..8
    double b[40];          // m-factor parts of the multipoles (sorted positions)
    double part[2];        // flux partial sums (warps 0 and 2)
    double aux[2];         // warp 3: y_2 / y_3, 1 / (8 pi nu)
    unsigned long long slot;
};

constexpr int kQuadMax = 2;  // quads per block (256 threads)

// k = f(y) for the binary of this quad; the four warps call it with the same y
// and return the same k.  q: warp of the quad (0..3); lane: 0..31.
__device__ __forceinline__ void eob_rhs_quad(const HamJets &J, const FluxTable &t, const double y[4], double k[4],
                                             int lane, int q, QuadXchg &x, PairSync &ps)
{
    const double r = y[0], L = y[3];
    const int j = lane & 15;
    const double u = eob_rcp(r);

    // ---- jets (lanes 16..31 repeat lanes 0..15)
    if (q == 0) {
        const double lr = eob_log(r);
        if (lane == 0) x.lr = lr;
    } else if (q == 1) {
        const Jet p = jet_half(J, j, false, u, r, 1.0);
        x.jet[1][0][lane] = p.v;
        x.jet[1][1][lane] = p.d;
    } else if (q == 2) {
        // sqrt(u) = 1/sqrt(r), beside the division u = 1/r
        const double su = eob_rsqrt(r);
        const Jet p = jet_poly_s(J, j, upow(u));
        x.jet[2][0][lane] = p.v;
        x.jet[2][1][lane] = p.d;
        if (lane == 0) {
            x.su[0] = su;
            x.su[1] = 0.5 * r * su;
        }
    } else {
        const Jet p = jet_poly_l(J, j, upow(u));
        x.jet[0][0][lane] = p.v;
        x.jet[0][1][lane] = p.d;
    }
    pair_sync(ps);  // 1: jets
    // poly + sqrt(u) poly + log r * log poly, the same expression on every
    // warp; each warp gathers only the jets its pieces read
    const Jet jn = jet_join_s({x.jet[1][0][lane], x.jet[1][1][lane]}, {x.jet[2][0][lane], x.jet[2][1][lane]},
                              {x.jet[0][0][lane], x.jet[0][1][lane]}, x.su[0], x.su[1], x.lr, r);
    const double jv = jn.v, jd = jn.d;
    Jet jt[kNumJets];
    auto gather = [&](int s) {
        jt[s].v = __shfl_sync(0xffffffffu, jv, s);
        jt[s].d = __shfl_sync(0xffffffffu, jd, s);
    };
    if (q == 0) {
        gather(J_AK0); gather(J_AKA); gather(J_FA); gather(J_AS); gather(J_DC);
    } else if (q == 1) {
        gather(J_DC); gather(J_BNN);
        // values only
        jt[J_Q4].v = __shfl_sync(0xffffffffu, jv, J_Q4);
        jt[J_Q6].v = __shfl_sync(0xffffffffu, jv, J_Q6);
        jt[J_Q8].v = __shfl_sync(0xffffffffu, jv, J_Q8);
    } else if (q == 2) {
        gather(J_AK0); gather(J_DB); gather(J_G); gather(J_BX); gather(J_Q4); gather(J_Q6); gather(J_Q8);
    } else {
        gather(J_N0); gather(J_N1); gather(J_N2); gather(J_N3);
    }

    // ---- combination (odd lanes at p_r = 0: the circular frequency)
    const double pr = (lane & 1) ? 0.0 : y[2];
    double idc = 0.0;
    if (q == 0) {
        idc = eob_rcp(jt[J_DC].v);
        const PartA a = comb_A(jt, idc);
        x.pa[0][lane] = a.Av;
        x.pa[1][lane] = a.Ad;
    } else if (q == 1) {
        idc = eob_rcp(jt[J_DC].v);
        const PartC c = comb_C(J, jt, u, idc);
        x.pc[0][lane] = c.cuv;
        x.pc[1][lane] = c.cud;
        x.pwq[lane] = comb_Wp_q(jt, pr);
    } else if (q == 2) {
        const PartW w = comb_W_b(comb_b(jt, pr * pr), pr);
        x.pw[0][lane] = w.W;
        x.pw[1][lane] = w.Wu;
        x.pw[2][lane] = w.Wp;
    } else {
        const PartN n = comb_N(J, jt, pr * pr);
        x.pn[0][lane] = n.Nv;
        x.pn[1][lane] = n.Nu;
        x.pn[2][lane] = n.Np;
    }
    pair_sync(ps);  // 2: A, c, W, N
    if (q == 0) {
        const PartA a{x.pa[0][lane], x.pa[1][lane]};
        const PartC c{x.pc[0][lane], x.pc[1][lane]};
        const PartW w{x.pw[0][lane], x.pw[1][lane], x.pw[2][lane] + x.pwq[lane]};
        const HeffPart e = comb_even_parts(a, c, w, L);
        x.ev[0][lane] = e.v;
        x.ev[1][lane] = e.du;
        x.ev[2][lane] = e.dp;
        x.ev[3][lane] = e.dL;
    } else if (q == 1) {
        const PartN n{x.pn[0][lane], x.pn[1][lane], x.pn[2][lane]};
        const HeffPart o = comb_odd_parts(jt, u, idc, n, pr, L);
        x.od[0][lane] = o.v;
        x.od[1][lane] = o.du;
        x.od[2][lane] = o.dp;
        x.od[3][lane] = o.dL;
    } else if (q == 3 && lane == 0) {
        // written after barrier 1 of this right-hand side, so no warp still
        // reads the previous values (they are read after barrier 6)
        x.aux[0] = y[2] / y[3];
        x.aux[1] = 1.0 / (8.0 * kPi * J.nu);
    }
    pair_sync(ps);  // 3: even and odd parts

    // ---- H and the flux set-up
    // lane 0's (state) parts: D = dH_eff/dL
    const double D = x.ev[3][0] + x.od[3][0];
    if (q == 0) {
        HeffPart ev, od;
        ev.v = x.ev[0][lane];
        ev.du = x.ev[1][lane];
        ev.dp = x.ev[2][lane];
        ev.dL = x.ev[3][lane];
        od.v = x.od[0][lane];
        od.du = x.od[1][lane];
        od.dp = x.od[2][lane];
        od.dL = x.od[3][lane];
        const HamPart hp = comb_final(J, u, ev, od);
        const double omega = __shfl_sync(0xffffffffu, hp.dHdL, 0);
        const double omega_c = __shfl_sync(0xffffffffu, hp.dHdL, 1);
        if (lane == 0) {
            x.ham[0] = hp.dHdr;
            x.ham[1] = hp.dHdpr;
            x.ham[2] = hp.dHdL;
        }
        // v_phi^2 = (omega omega_c^(-2/3))^2 (its powers are taken by the
        // m-factor warps, which wait longer)
        const double rc = eob_rcbrt(omega_c);
        const double vphi = omega * (rc * rc);
        if (lane == 0) x.fl[5] = vphi * vphi;
    } else if (q == 1) {
        // H_real omega = M^2 D (H_real = M s, omega = M D / s)
        const double hw = (J.M * J.M) * D;
        double Tm, k4m;
        flux_m_factors((lane & 7) + 1, 4.0 * kPi * hw, hw, &Tm, &k4m);
        if (lane < 8) {
            x.T[lane] = Tm;
            x.k4[lane] = k4m;
        }
    } else {
        // s = sqrt(s2) and omega = M D / s from the state's parts
        const double heff = x.ev[0][0] + x.od[0][0];
        const double s2 = fma(2.0 * J.nu, heff - 1.0, 1.0);
        const double rs = eob_rsqrt(s2);
        const double omega = (J.M * D) * rs;
        if (q == 2) {
            // v = omega^(1/3) = omega r^2, v^12, S_odd = v p_phi
            const double ro = eob_rcbrt(omega);
            const double v = omega * (ro * ro);
            const double v2 = v * v, v4 = v2 * v2;
            const double So = v * L;
            if (lane == 0) {
                x.fl[0] = v;
                x.fl[2] = v4 * v4 * v4;
                x.fl[4] = So * So;
                x.fl[6] = v4 * v;
                x.fl[7] = v2;
            }
        } else {
            // log v = log(omega) / 3, and S_even from H_real^2 = M^2 s^2
            // (no square root on that branch)
            const double Se = fma(fma(J.M * J.M, s2, -1.0), t.inv2eta, 1.0);
            const double lv = eob_log(omega) * (1.0 / 3.0);
            if (lane == 0) {
                x.fl[1] = lv;
                x.fl[3] = Se * Se;
            }
        }
    }
    pair_sync(ps);  // 4: flux set-up and m factors

    // ---- multipoles: series parts on warps 0 and 2, m-factor parts on 1 and 3
    FluxLane f;
    f.v = x.fl[0];
    f.v2 = x.fl[7];
    f.lv = x.fl[1];
    f.v12 = x.fl[2];
    f.S2e = x.fl[3];
    f.S2o = x.fl[4];
    f.Se = 0.0;
    f.Sodd = 0.0;
    double a_part = 0.0;
    if (q == 0) {
        // positions 0..15 (degree 10 .. 4): lanes j and j + 16 take the two
        // halves of rho's series of position j
        const int i = kFluxOrder[lane & 15];
        const double hv = flux_rho_half(t, i, f, lane >> 4);
        const double hi = __shfl_xor_sync(0xffffffffu, hv, 16);
        const double rho = fma(fma(x.fl[6], hi, hv), f.v, 1.0);
        a_part = flux_mode_s_rho(t, i, f, rho);
    } else if (q == 2) {
        // positions 16..34 (degree 4 .. 2)
        const int pos = 16 + lane;
        a_part = flux_mode_s<kFluxDegSorted[16]>(t, kFluxOrder[pos < kNumLM ? pos : kNumLM - 1], f);
    } else {
        const int pos = (q == 1) ? lane : 32 + lane;
        if (pos < kNumLM) {
            const int i = kFluxOrder[pos];
            const int m = lm_packed(i) & 15;
            x.b[pos] = flux_mode_b(t, i, x.T[m - 1], x.k4[m - 1]) * flux_mode_vp_sq(i, x.fl[5]);
        }
    }
    pair_sync(ps);  // 5: m-factor parts
    // F / omega = total c1 with F = total omega^2 / (8 pi) / nu, and
    // (y_2 / y_3) F / omega = total c2: the factors are taken here, beside
    // the reduction below, so that only two products follow the last barrier
    const double omega = x.ham[2];
    const double c1 = omega * x.aux[1], c2 = x.aux[0] * c1;
    if (q == 0 || q == 2) {
        const int pos = (q == 0) ? lane : 16 + lane;
        double part = (q == 0 ? lane < 16 : pos < kNumLM) ? x.b[pos] * a_part : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
        if (lane == 0) x.part[q >> 1] = part;
    }
    pair_sync(ps);  // 6: flux partial sums
    const double total = x.part[0] + x.part[1];
    k[0] = x.ham[1];
    k[1] = omega;
    k[2] = -fma(c2, total, x.ham[0]);
    k[3] = -(total * c1);
}

}  // namespace eob
