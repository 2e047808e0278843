// One binary on four warps (a warp quad, one warp on each SM sub-partition):
// the right-hand side of the EOB equations in pieces that four FP64 pipes
// evaluate side by side.  It extends the warp pair (rhs_pair.cuh) for the few
// binaries whose sequential chains set a batch's time:
//
//   stage           warp 0              warp 1              warp 2              warp 3
//   jets            log r               polynomial parts    sqrt(u) polynomials log polynomials
//                                                                               and sqrt(u)
//   combination a   1/Dc, A(u)          1/Dc, c(u),         B_np, q, W - L^2 c  N(u, p_r^2)
//                                       q part of dW/dp_r
//   combination b   even part sqrt(AW)  odd part            H_eff's value,      y_2/y_3
//                   and derivatives     and derivatives     s^2, 1/s
//   H, flux set-up  H and gradient,     m x/(1-e^{-m x})    omega, v = omega    omega, log v,
//                   v_phi^2, 4 k^2      from H_real omega   r_omega^2, v^12, S_o H_real, S_even
//                                       = M^2 D
//   multipoles      series part 0..15   m-factor and v_phi  series part 16..34  m-factor and v_phi
//                   (two lanes each)    part 0..31                              part 32..34
//   (then each multipole's two parts multiplied and summed by every warp)
//
// Values cross through shared memory at five barriers per right-hand side
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
    double su;             // warp 3: sqrt(u) = 1/sqrt(r)
    double pa[2][32];      // warp 0: A, dA/du
    double pc[2][32];      // warp 1: c, dc/du
    double pw[3][32];      // warp 2: W - L^2 c and its u-derivative, the B_np part of dW/dp_r
    double pwq[32];        // warp 1: the q part of dW/dp_r
    double pn[3][32];      // warp 3: N, dN/du, dN/dp_r^2
    double idc[32];        // warp 0: 1 / D_c
    double hs[2][32];      // warp 2: s^2 = 1 + 2 nu (H_eff - 1) and 1/s
    double ev[4][32];      // warp 0: derivatives of the even part of H_eff ([0] unused)
    double od[4][32];      // warp 1: derivatives of the odd part ([0] unused)
    double ham[3];         // warp 0: dH/dr, dH/dp_r, dH/dL at the state
    double fl[16];         // v, log v, v^12, S_e^2, S_o^2, v_phi^2, v^5, v^2
    double T[8], k4[8];    // warps 1, 0: m factors, m = 1..8
    double elm[8];         // warp 3: eulerlog_m(v) = elog[m] + log v, m = 1..8
    double b[64];          // warps 1, 3: m-factor parts of the multipoles (sorted positions 0..34)
    double a[64];          // warps 0, 2: series parts (positions 0..34)
    double aux[1];         // warp 3: y_2 / y_3
    unsigned long long slot;
};

constexpr int kQuadMax = 2;  // quads per block (256 threads)

// Per-lane constants of a four-warp group, set once per launch: the
// multipole whose series part (warps 0, 2) or m-factor part (warps 1, 3) the
// lane evaluates, and m as a double for the m-factor lanes (lanes 0..7 give
// m = 1..8).  Kept in registers: the lookups would otherwise be chained
// global loads at the start of every multipole phase.
struct QuadLane {
    int i, lm;  // kFluxOrder at the lane's sorted position, lm_packed(i)
    double md;  // (lane & 7) + 1
};

__device__ __forceinline__ QuadLane quad_lane(int q, int lane)
{
    int pos = (q == 0) ? (lane & 15) : (q == 2) ? 16 + lane : (q == 1) ? lane : 32 + lane;
    pos = pos < kNumLM ? pos : kNumLM - 1;
    QuadLane o;
    o.i = kFluxOrder[pos];
    o.lm = lm_packed(o.i);
    o.md = (double)((lane & 7) + 1);
    return o;
}

// k = f(y) for the binary of this quad; the four warps call it with the same y
// and return the same k.  q: warp of the quad (0..3); lane: 0..31.
__device__ __forceinline__ void eob_rhs_quad(const HamJets &J, const FluxTable &t, const QuadLane &ql, const double y[4],
                                             double k[4], int lane, int q, QuadXchg &x, PairSync &ps)
{
    const double r = y[0], L = y[3];
    const int j = lane & 15;
    const double u = eob_rcp(r);
    double u3 = 0.0;  // warp 2: u^3 from the jets' powers, for its H_eff value
    // p_r and p_r^2 of the combination (odd lanes: p_r = 0, the circular frequency)
    const double pr = (lane & 1) ? 0.0 : y[2];
    const double p2 = pr * pr;

    // ---- jets (lanes 16..31 repeat lanes 0..15)
    if (q == 0) {
        const double lr = eob_log(r);
        if (lane == 0) x.lr = lr;
    } else if (q == 1) {
        const Jet p = jet_half(J, j, false, u, r, 1.0);
        x.jet[1][0][lane] = p.v;
        x.jet[1][1][lane] = p.d;
    } else if (q == 2) {
        const UPow up = upow(u);
        const Jet p = jet_poly_s_t(J, j, up, r);
        x.jet[2][0][lane] = p.v;
        x.jet[2][1][lane] = p.d;
        u3 = up.u3;
    } else {
        // sqrt(u) = 1/sqrt(r) beside the log polynomials
        const double su = eob_rsqrt(r);
        const Jet p = jet_poly_l(J, j, upow(u));
        x.jet[0][0][lane] = p.v;
        x.jet[0][1][lane] = p.d;
        if (lane == 0) x.su = su;
    }
    pair_sync(ps);  // 1: jets
    // poly + sqrt(u) poly + log r * log poly, the same expression on every
    // warp; each warp gathers only the jets its pieces read
    const Jet jn = jet_join_t({x.jet[1][0][lane], x.jet[1][1][lane]}, {x.jet[2][0][lane], x.jet[2][1][lane]},
                              {x.jet[0][0][lane], x.jet[0][1][lane]}, x.su, x.lr, r);
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
        jt[J_DC].v = __shfl_sync(0xffffffffu, jv, J_DC);
    } else {
        gather(J_N0); gather(J_N1); gather(J_N2); gather(J_N3);
    }

    // ---- combination (odd lanes at p_r = 0: the circular frequency)
    double idc = 0.0;
    if (q == 0) {
        idc = eob_rcp(jt[J_DC].v);
        const PartA a = comb_A(jt, idc);
        x.pa[0][lane] = a.Av;
        x.pa[1][lane] = a.Ad;
        x.idc[lane] = idc;
    } else if (q == 1) {
        idc = eob_rcp(jt[J_DC].v);
        const PartC c = comb_C(J, jt, u, idc);
        x.pc[0][lane] = c.cuv;
        x.pc[1][lane] = c.cud;
        x.pwq[lane] = comb_Wp_q_p2(jt, pr, p2);
    } else if (q == 2) {
        const PartW w = comb_W_b_p2(comb_b(jt, p2), pr, p2);
        x.pw[0][lane] = w.W;
        x.pw[1][lane] = w.Wu;
        x.pw[2][lane] = w.Wp;
    } else {
        const PartN n = comb_N(J, jt, p2);
        x.pn[0][lane] = n.Nv;
        x.pn[1][lane] = n.Nu;
        x.pn[2][lane] = n.Np;
    }
    pair_sync(ps);  // 2: A, c, W, N
    if (q == 0) {
        const PartA a{x.pa[0][lane], x.pa[1][lane]};
        const PartC c{x.pc[0][lane], x.pc[1][lane]};
        const PartW w{x.pw[0][lane], x.pw[1][lane], x.pw[2][lane] + x.pwq[lane]};
        const HeffPart e = comb_even_parts(a, c, w, L);  // its value: warp 2
        x.ev[1][lane] = e.du;
        x.ev[2][lane] = e.dp;
        x.ev[3][lane] = e.dL;
    } else if (q == 1) {
        const PartN n{x.pn[0][lane], x.pn[1][lane], x.pn[2][lane]};
        const HeffPart o = comb_odd_parts(jt, u, idc, n, pr, L);  // its value: warp 2
        x.od[1][lane] = o.du;
        x.od[2][lane] = o.dp;
        x.od[3][lane] = o.dL;
    } else if (q == 2) {
        // H_eff's value from the same pieces as warps 0 and 1 (even part
        // sqrt(A W), odd part L u^3 N / D_c), then s^2 and 1/s, which the
        // H and flux set-up of every warp needs after barrier 3
        const double W = fma(L * L, x.pc[0][lane], x.pw[0][lane]);
        const double AW = x.pa[0][lane] * W;
        const double u3i = u3 * x.idc[lane];
        const double od = L * u3i * x.pn[0][lane];
        const double s2 = fma(J.two_nu, fma(AW, eob_rsqrt(AW), od) - 1.0, 1.0);
        x.hs[0][lane] = s2;
        x.hs[1][lane] = eob_rsqrt(s2);
    } else if (lane == 0) {
        // written after barrier 2 of this right-hand side, so no warp still
        // reads the previous value (it is read between barriers 5 and 6)
        x.aux[0] = y[2] * eob_rcp(y[3]);
    }
    pair_sync(ps);  // 3: even and odd parts, s^2 and 1/s

    // ---- H and the flux set-up
    // lane 0's (state) parts: D = dH_eff/dL
    const double D = x.ev[3][0] + x.od[3][0];
    if (q == 0) {
        HeffPart ev, od;
        ev.v = 0.0;  // H_eff's value enters through s^2 and 1/s
        ev.du = x.ev[1][lane];
        ev.dp = x.ev[2][lane];
        ev.dL = x.ev[3][lane];
        od.v = 0.0;
        od.du = x.od[1][lane];
        od.dp = x.od[2][lane];
        od.dL = x.od[3][lane];
        const HamPart hp = comb_final_s(J, u, ev, od, x.hs[0][lane], x.hs[1][lane]);
        // 4 k^2 = 4 (m H_real omega)^2 of the m factors, H_real omega = M^2 D
        const double k4m = flux_m_factor_k4(ql.md, J.M2 * D);
        if (lane < 8) x.k4[lane] = k4m;
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
        // m x / (1 - e^{-m x}), x = 4 pi H_real omega = 4 pi M^2 D
        // (H_real = M s, omega = M D / s)
        const double Tm = flux_m_factor_T(ql.md, 4.0 * kPi * (J.M2 * D));
        if (lane < 8) x.T[lane] = Tm;
    } else {
        // omega = M D / s at the state
        const double s2 = x.hs[0][0];
        const double omega = (J.M * D) * x.hs[1][0];
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
            const double Se = fma(fma(J.M2, s2, -1.0), t.inv2eta, 1.0);
            const double lv = eob_log(omega) * (1.0 / 3.0);
            const double elm = t.elog[(lane & 7) + 1] + lv;
            if (lane < 8) x.elm[lane] = elm;
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
        const double hv = flux_rho_half_e(t, ql.i, x.elm[(ql.lm & 15) - 1], f, lane >> 4);
        const double hi = __shfl_xor_sync(0xffffffffu, hv, 16);
        const double rho = fma(fma(x.fl[6], hi, hv), f.v, 1.0);
        const double a_part = flux_mode_s_rho_lm<flux_lmax(0, 16), flux_lmin(0, 16)>(t, ql.i, ql.lm, f, rho);
        if (lane < 16) x.a[lane] = a_part;
    } else if (q == 2) {
        // positions 16..34 (degree 4 .. 2)
        const int pos = 16 + lane;
        const double a_part = flux_mode_s_e<kFluxDegSorted[16], kLMax, flux_lmin(16, kNumLM - 16)>(
            t, ql.i, ql.lm, x.elm[(ql.lm & 15) - 1], f);
        if (pos < kNumLM) x.a[pos] = a_part;
    } else {
        const int pos = (q == 1) ? lane : 32 + lane;
        if (pos < kNumLM) {
            // times F / (omega total) = omega / (8 pi nu): the sum below is F / omega
            const int m = ql.lm & 15;
            const double c1 = x.ham[2] * J.inv8pinu;
            x.b[pos] = (flux_mode_b_l(t, ql.i, ql.lm >> 4, x.T[m - 1], x.k4[m - 1]) * flux_mode_vp_sq_lm(ql.lm, x.fl[5])) * c1;
        }
    }
    pair_sync(ps);  // 5: series and m-factor parts
    // F / omega (the m-factor parts carry omega / (8 pi nu)); every warp
    // forms it itself -- the same products and butterfly
    // on the same shared values, so the same bits on every warp -- and no
    // barrier follows: lane l takes positions l and (l < 3) 32 + l
    const bool hi3 = lane < kNumLM - 32;
    double total = fma(hi3 ? x.b[32 + lane] : 0.0, hi3 ? x.a[32 + lane] : 0.0, x.b[lane] * x.a[lane]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) total += __shfl_xor_sync(0xffffffffu, total, off);
    k[0] = x.ham[1];
    k[1] = x.ham[2];
    k[2] = -fma(x.aux[0], total, x.ham[0]);  // (y_2 / y_3) F / omega
    k[3] = -total;
}

}  // namespace eob
