// One binary on two warps (a warp pair): the right-hand side of the EOB
// equations split into pieces that the two warps evaluate side by side.
//
// On GB300 each SM sub-partition issues one FP64 warp-instruction per 64
// cycles, so a lane group's right-hand side costs as many issue slots as it
// has FP64 instructions, however many lanes share them.  A binary whose
// trajectory is the batch's critical path therefore gets shorter only if its
// instruction stream gets shorter.  The two warps of a pair sit on two
// sub-partitions of one SM (warps 2p and 2p + 1 of the block), each with its
// own FP64 pipe, and split every stage whose pieces are independent:
//
//   stage        role 0 (warp 2p)                 role 1 (warp 2p + 1)
//   jets         log r, the log(r) parts          sqrt(u), the polynomial and
//                                                 sqrt(u) parts (halves of the warp)
//   combination  A(u), c(u)  -> even part         B_np, q  -> odd part
//   H, flux      H and its gradient;              m factors (m x/(1-e^{-m x}), 4k^2),
//                v = omega^(1/3), v_phi powers;   log v, y_2/y_3, 1/(8 pi nu); multipoles 32..34
//                multipoles 0..31
//
// Values cross between the warps through shared memory at five pair
// barriers per right-hand side (an mbarrier of 64 arrivals, waited on with a
// time limit: if the partner does not arrive within kPairTimeoutNs the pair
// reports failure and the integrator ends that binary with EOB_ST_SYNC).
// Every value both warps go on to use is read by both from shared memory
// (never one warp's register copy, which the compiler could fuse into a later
// fma differently), so their results -- and every later control decision of
// the integrator, which both warps run redundantly -- are bitwise identical.
#pragma once
#include "physics/flux_eval.h"

namespace eob {

constexpr int kPairMax = 4;                                  // pairs per block (256 threads)
constexpr unsigned long long kPairTimeoutNs = 2000000000ull;  // 2 s per barrier wait
constexpr int kPairMaxPolls = 1 << 28;                        // and at most this many polls

// shared-memory exchange of one pair
struct PairXchg {
    double jet[2][2][32];  // [part: 0 log, 1 poly+sqrt][v, d][lane]
    double b[4][32];       // role 1 -> 0: bnpv, bnpd, qa, qad
    double ev[4][32];      // role 0 -> both: even part of H_eff and its derivatives
    double od[4][32];      // role 1 -> both: odd part
    double T[8], k4[8];    // role 1 -> 0: m factors, m = 1..8
    double fl[13];         // v, log v (role 1 -> 0), v^12, S_even, S_odd, v_phi^(2e) e = 2..9 (role 0 -> 1)
    double part[2];        // flux partial sums of the two warps
    double aux[2];         // role 1 -> both: y_2 / y_3, 1 / (8 pi nu)
    double ham[3];         // role 0 -> both: dH/dr, dH/dp_r, dH/dL at the state
    unsigned long long slot;
};

struct PairSync {
    unsigned bar;     // shared-memory address of the pair's mbarrier
    unsigned parity;  // parity of the phase this warp waits for next
    bool ok;          // false once a wait ran out of time
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Both warps of the pair arrive (all 64 lanes: each lane's shared and global
// writes before the barrier are released to the other warp) and wait, with a
// time limit of limit_ns, for the phase to complete.  A warp whose wait runs
// out marks itself failed (ps.ok = false) and skips every later barrier, so a
// group in which one warp stopped arriving ends after one limit per warp.
__device__ __forceinline__ void pair_sync_limit(PairSync &ps, unsigned long long limit_ns)
{
    if (!ps.ok) return;
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(ps.bar) : "memory");
    unsigned done = 0;
    unsigned long long t0 = 0;
    for (int i = 0;; ++i) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(ps.bar), "r"(ps.parity)
            : "memory");
        if (done) break;
        if (i == 0) t0 = global_ns();
        else if (global_ns() - t0 > limit_ns || i >= kPairMaxPolls) break;
    }
    ps.parity ^= 1u;
    if (!__all_sync(0xffffffffu, done)) ps.ok = false;
}

// The integrator's barrier: the fixed limit kPairTimeoutNs.
__device__ __forceinline__ void pair_sync(PairSync &ps) { pair_sync_limit(ps, kPairTimeoutNs); }

// Set-up by the block's first thread, before any group barrier is used:
// ngroups barriers of `arrivals` threads each (64 for a pair, 128 for four warps).
__device__ __forceinline__ void group_init(unsigned long long *bars, int ngroups, int arrivals)
{
    if (threadIdx.x == 0) {
        for (int p = 0; p < ngroups; ++p) {
            const unsigned a = (unsigned)__cvta_generic_to_shared(&bars[p]);
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(arrivals) : "memory");
        }
    }
    __syncthreads();
}

__device__ __forceinline__ void pair_init(unsigned long long *bars, int npairs) { group_init(bars, npairs, 64); }

// multipoles at sorted positions [FIRST, FIRST + 32) of one warp, m factors
// from shared memory
template <int FIRST>
__device__ __forceinline__ double flux_warp_modes(const FluxTable &t, const FluxLane &f, const PairXchg &x, int lane)
{
    constexpr int KM = kFluxDegSorted[FIRST];
    const int pos = FIRST + lane;
    const int i = kFluxOrder[pos < kNumLM ? pos : kNumLM - 1];
    const int m = lm_packed(i) & 15;
    const double here =
        flux_mode_lane<KM, flux_lmax(FIRST, 32), flux_lmin(FIRST, 32)>(t, i, f, x.T[m - 1], x.k4[m - 1]);
    return (pos < kNumLM) ? here : 0.0;
}

// k = f(y) for the binary of this pair; both warps call it with the same y
// and return the same k.  role: 0 or 1; lane: 0..31.
__device__ __forceinline__ void eob_rhs_pair(const HamJets &J, const FluxTable &t, const double y[4], double k[4],
                                             int lane, int role, PairXchg &x, PairSync &ps)
{
    const double r = y[0], L = y[3];
    const int j = lane & 15;
    const double u = eob_rcp(r);

    // ---- jets: role 0 the log(r) parts; role 1 the polynomial parts on
    // lanes 0..15 and the sqrt(u) parts on lanes 16..31
    if (role == 0) {
        const double lr = eob_log(r);
        const Jet p = jet_part_l(J, j, u, r, lr);
        x.jet[0][0][lane] = p.v;
        x.jet[0][1][lane] = p.d;
    } else {
        const bool sq = lane >= 16;
        // sqrt(u) = 1/sqrt(r), independent of the division u = 1/r
        const Jet hj = jet_half(J, j, sq, u, r, sq ? eob_rsqrt(r) : 1.0);
        const double ov = __shfl_xor_sync(0xffffffffu, hj.v, 16);
        const double od = __shfl_xor_sync(0xffffffffu, hj.d, 16);
        // lanes j and j + 16 hold the two halves; add them in one order
        x.jet[1][0][lane] = sq ? ov + hj.v : hj.v + ov;
        x.jet[1][1][lane] = sq ? od + hj.d : hj.d + od;
    }
    pair_sync(ps);  // 1: jets
    const double jv = x.jet[1][0][lane] + x.jet[0][0][lane];
    const double jd = x.jet[1][1][lane] + x.jet[0][1][lane];
    Jet jt[kNumJets];
#pragma unroll
    for (int q = 0; q < kNumJets; ++q) {
        jt[q].v = __shfl_sync(0xffffffffu, jv, q);
        jt[q].d = __shfl_sync(0xffffffffu, jd, q);
    }

    // ---- combination (odd lanes at p_r = 0: the circular frequency)
    const double pr = (lane & 1) ? 0.0 : y[2];
    if (role == 0) {
        const CombA a = comb_a(J, jt, u);
        pair_sync(ps);  // 2: B_np, q
        CombB b;
        b.bnpv = x.b[0][lane];
        b.bnpd = x.b[1][lane];
        b.qa = x.b[2][lane];
        b.qad = x.b[3][lane];
        const HeffPart e = comb_even(jt, a, b, pr, L);
        x.ev[0][lane] = e.v;
        x.ev[1][lane] = e.du;
        x.ev[2][lane] = e.dp;
        x.ev[3][lane] = e.dL;
        pair_sync(ps);  // 3: even and odd parts
    } else {
        const CombB b = comb_b(jt, pr * pr);
        x.b[0][lane] = b.bnpv;
        x.b[1][lane] = b.bnpd;
        x.b[2][lane] = b.qa;
        x.b[3][lane] = b.qad;
        if (lane == 0) {
            x.aux[0] = y[2] * eob_rcp(y[3]);
            x.aux[1] = J.inv8pinu;
        }
        pair_sync(ps);  // 2
        const HeffPart o = comb_odd(J, jt, u, eob_rcp(jt[J_DC].v), pr, L);
        x.od[0][lane] = o.v;
        x.od[1][lane] = o.du;
        x.od[2][lane] = o.dp;
        x.od[3][lane] = o.dL;
        pair_sync(ps);  // 3
    }
    HeffPart ev, od;
    ev.v = x.ev[0][lane];
    ev.du = x.ev[1][lane];
    ev.dp = x.ev[2][lane];
    ev.dL = x.ev[3][lane];
    od.v = x.od[0][lane];
    od.du = x.od[1][lane];
    od.dp = x.od[2][lane];
    od.dL = x.od[3][lane];
    // ---- H and the flux set-up
    double part;
    if (role == 0) {
        const HamPart hp = comb_final(J, u, ev, od);
        const double Hreal = __shfl_sync(0xffffffffu, hp.Hreal, 0);
        const double omega = __shfl_sync(0xffffffffu, hp.dHdL, 0);
        const double omega_c = __shfl_sync(0xffffffffu, hp.dHdL, 1);
        if (lane == 0) {
            x.ham[0] = hp.dHdr;
            x.ham[1] = hp.dHdpr;
            x.ham[2] = hp.dHdL;
        }
        // reciprocal cube roots of omega (even lanes) and omega_c (odd lanes)
        // in one instruction stream: v = omega r_omega^2 and
        // v_phi = omega / omega_c^(2/3) = omega r_c^2 without a division
        const double rc = eob_rcbrt((lane & 1) ? omega_c : omega);
        const double r0 = __shfl_sync(0xffffffffu, rc, 0), r1 = __shfl_sync(0xffffffffu, rc, 1);
        FluxLane f = flux_lane_make_rv(t, L, omega, Hreal, omega * (r0 * r0), omega * (r1 * r1), 0.0);
        if (lane == 0) {
            x.fl[0] = f.v;
            x.fl[2] = f.v12;
            x.fl[3] = f.Se;
            x.fl[4] = f.Sodd;
#pragma unroll
            for (int q = 0; q < 8; ++q) x.fl[5 + q] = f.vp[q];
        }
        pair_sync(ps);  // 4: FluxLane, log v and m factors
        f.lv = x.fl[1];
        part = flux_warp_modes<0>(t, f, x, lane);
    } else {
        // this warp needs H_real omega and omega, not the whole combination:
        // with D = dH_eff/dL, H_real omega = M^2 D exactly (H_real = M s,
        // omega = M D / s), and omega = M D / s with s from the same square root
        const double D = x.ev[3][0] + x.od[3][0];
        const double hw = J.M2 * D;
        double Tm, k4m;
        flux_m_factors((lane & 7) + 1, 4.0 * kPi * hw, hw, &Tm, &k4m);
        if (lane < 8) {
            x.T[lane] = Tm;
            x.k4[lane] = k4m;
        }
        // log v = log(omega) / 3, here rather than after the cube root on the
        // other warp, whose flux set-up is the longer of the two
        const double heff = x.ev[0][0] + x.od[0][0];
        const double s2 = fma(J.two_nu, heff - 1.0, 1.0);
        const double omega = (J.M * D) * eob_rsqrt(s2);
        const double lv = eob_log(omega) * (1.0 / 3.0);
        if (lane == 0) x.fl[1] = lv;
        pair_sync(ps);  // 4
        FluxLane f;
        f.v = x.fl[0];
        f.v2 = f.v * f.v;
        f.lv = x.fl[1];
        f.v12 = x.fl[2];
        f.Se = x.fl[3];
        f.Sodd = x.fl[4];
        f.S2e = f.Se * f.Se;
        f.S2o = f.Sodd * f.Sodd;
#pragma unroll
        for (int q = 0; q < 8; ++q) f.vp[q] = x.fl[5 + q];
        part = flux_warp_modes<32>(t, f, x, lane);
    }
    // F / omega = total c1 with F = total omega^2 / (8 pi) / nu, and
    // (y_2 / y_3) F / omega = total c2, beside the reduction
    const double omega = x.ham[2];
    const double c1 = omega * x.aux[1], c2 = x.aux[0] * c1;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if (lane == 0) x.part[role] = part;
    pair_sync(ps);  // 5: flux partial sums
    const double total = x.part[0] + x.part[1];
    k[0] = x.ham[1];
    k[1] = omega;
    k[2] = -fma(c2, total, x.ham[0]);
    k[3] = -(total * c1);
}

}  // namespace eob
