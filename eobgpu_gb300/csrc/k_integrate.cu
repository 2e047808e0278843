// Persistent DOPR853 integrator over the EOB equations of motion.
//
// Replaces the reference's Python-driven loop (eob/new_Dormand_horiz.py:
// 424-778) and its ~90 synchronous launches per step (src/DOPR853.cu:357-798,
// src/EOB.cu:3046-3145) with one launch for the whole batch:
//
//  * one lane per binary for large batches, or G lanes per binary (lane
//    groups) when the longest binary's chain sets the time: GB300 issues one
//    FP64 warp-instruction per 64 cycles per SM sub-partition whatever the
//    active mask, so every lane must carry a binary or a distinct piece of
//    one binary's arithmetic;
//  * a flat per-lane state machine: each pass through the main loop evaluates
//    exactly one right-hand side on every lane, whether that lane is in stage
//    s of a step, in the stopping test, or starting a new pass or binary --
//    the expensive RHS never diverges;
//  * binaries are taken from a device work queue (atomicAdd) in a caller
//    given order (longest first), so ragged step counts (13 .. 8676 steps)
//    refill lanes instead of idling them;
//  * the stopping test's RHS at the accepted state is reused as the next
//    step's first stage (the reference evaluates the same function twice);
//  * both passes of run_trajectory (eob/seobnrv4phm.py:2072-2136) run in the
//    same thread: adaptive pass, step back 10 M, fixed 0.05 M pass;
//  * the stopping rule is StoppingCriterion (eob/seobnrv4phm.py:82-150) read
//    for one binary; its omega history restarts at zero at every pass.
//
// All loops are bounded: a pass ends after max_tries step attempts, on a
// non-finite error estimate or step, or at the row capacity.
#include "eob_device.cuh"
#include "rhs_pair.cuh"
#include "rhs_quad.cuh"

namespace eob {
namespace dp {
// Tableau of Hairer's DOP853 as used by the reference (src/DOPR853.cu:10-192).
// For stage s (2..12) the weights a[s][*] on the stored slopes, listed in the
// reference's accumulation order; slot numbering k1..k10, stage 11 writes k2
// and stage 12 writes k3 (src/DOPR853.cu:498, 516).
struct Term {
    signed char slot;
    double a;
};
#define EOB_DOPR_STAGES \
{ \
    {}, {}, \
    {{1, 5.26001519587677318785587544488e-2}}, \
    {{1, 1.97250569845378994544595329183e-2}, {2, 5.91751709536136983633785987549e-2}}, \
    {{1, 2.95875854768068491816892993775e-2}, {3, 8.87627564304205475450678981324e-2}}, \
    {{1, 2.41365134159266685502369798665e-1}, {3, -8.84549479328286085344864962717e-1}, \
    {4, 9.24834003261792003115737966543e-1}}, \
    {{1, 3.7037037037037037037037037037e-2}, {4, 1.70828608729473871279604482173e-1}, \
    {5, 1.25467687566822425016691814123e-1}}, \
    {{1, 3.7109375e-2}, {4, 1.70252211019544039314978060272e-1}, {5, 6.02165389804559606850219397283e-2}, \
    {6, -1.7578125e-2}}, \
    {{1, 3.70920001185047927108779319836e-2}, {4, 1.70383925712239993810214054705e-1}, \
    {5, 1.07262030446373284651809199168e-1}, {6, -1.53194377486244017527936158236e-2}, \
    {7, 8.27378916381402288758473766002e-3}}, \
    {{1, 6.24110958716075717114429577812e-1}, {4, -3.36089262944694129406857109825e0}, \
    {5, -8.68219346841726006818189891453e-1}, {6, 2.75920996994467083049415600797e1}, \
    {7, 2.01540675504778934086186788979e1}, {8, -4.34898841810699588477366255144e1}}, \
    {{1, 4.77662536438264365890433908527e-1}, {4, -2.48811461997166764192642586468e0}, \
    {5, -5.90290826836842996371446475743e-1}, {6, 2.12300514481811942347288949897e1}, \
    {7, 1.52792336328824235832596922938e1}, {8, -3.32882109689848629194453265587e1}, \
    {9, -2.03312017085086261358222928593e-2}}, \
    {{1, -9.3714243008598732571704021658e-1}, {4, 5.18637242884406370830023853209e0}, \
    {5, 1.09143734899672957818500254654e0}, {6, -8.14978701074692612513997267357e0}, \
    {7, -1.85200656599969598641566180701e1}, {8, 2.27394870993505042818970056734e1}, \
    {9, 2.49360555267965238987089396762e0}, {10, -3.0467644718982195003823669022e0}}, \
    {{1, 2.27331014751653820792359768449e0}, {4, -1.05344954667372501984066689879e1}, \
    {5, -2.00087205822486249909675718444e0}, {6, -1.79589318631187989172765950534e1}, \
    {7, 2.79488845294199600508499808837e1}, {8, -2.85899827713502369474065508674e0}, \
    {9, -8.87285693353062954433549289258e0}, {10, 1.23605671757943030647266201528e1}, \
    {2, 6.43392746015763530355970484046e-1}}, \
    }
__constant__ Term kStage[13][9] = EOB_DOPR_STAGES;
constexpr Term kStageC[13][9] = EOB_DOPR_STAGES;
__constant__ signed char kNTerms[13] = {0, 0, 1, 2, 2, 3, 3, 4, 5, 6, 7, 8, 9};
constexpr int kNTermsC[13] = {0, 0, 1, 2, 2, 3, 3, 4, 5, 6, 7, 8, 9};
__constant__ signed char kOutSlot[13] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 2, 3};

constexpr double b1 = 5.42937341165687622380535766363e-2, b6 = 4.45031289275240888144113950566e0,
                 b7 = 1.89151789931450038304281599044e0, b8 = -5.8012039600105847814672114227e0,
                 b9 = 3.1116436695781989440891606237e-1, b10 = -1.52160949662516078556178806805e-1,
                 b11 = 2.01365400804030348374776537501e-1, b12 = 4.47106157277725905176885569043e-2;
constexpr double bhh1 = 0.244094488188976377952755905512e+00, bhh2 = 0.733846688281611857341361741547e+00,
                 bhh3 = 0.220588235294117647058823529412e-01;
constexpr double er1 = 0.1312004499419488073250102996e-01, er6 = -0.1225156446376204440720569753e+01,
                 er7 = -0.4957589496572501915214079952e+00, er8 = 0.1664377182454986536961530415e+01,
                 er9 = -0.3503288487499736816886487290e+00, er10 = 0.3341791187130174790297318841e+00,
                 er11 = 0.8192320648511571246570742613e-01, er12 = -0.2235530786388629525884427845e-01;
constexpr double safe = 0.9, minscale = 1.0 / 3.0, maxscale = 6.0;

// Running sums spread over the 32 lanes of a warp that carries one binary:
// lane l holds component l & 3 of two sums, selected by its slot group
// g = l >> 2: the argument sum of stage g + 2 (stages 2..9) and, for
// g = 0, 1, 2, that of stage g + 10, or for g = 3, 4, 5 the increment sum
// b_s k_s, the error sum er_s k_s and the correction sum -bhh_s k_s.  When
// the slope of stage p exists, every lane adds its weights w[p][g][*] times
// that slope (zero where stage p does not enter), so each sum is accumulated
// in the reference's order (its term lists run over ascending stages) while
// the lanes work on different sums in the same instruction.
struct LaneWeights {
    double w[13][8][2];
};

constexpr LaneWeights make_lane_weights()
{
    LaneWeights L{};
    for (int s = 2; s <= 12; ++s) {
        const int g = (s <= 9) ? s - 2 : s - 10, k = (s <= 9) ? 0 : 1;
        for (int t = 0; t < kNTermsC[s]; ++t) {
            const int slot = kStageC[s][t].slot;
            const int p = (s == 12 && slot == 2) ? 11 : slot;  // stage 11 overwrote slot 2
            L.w[p][g][k] = kStageC[s][t].a;
        }
    }
    const double bw[13] = {0, b1, 0, 0, 0, 0, b6, b7, b8, b9, b10, b11, b12};
    const double ew[13] = {0, er1, 0, 0, 0, 0, er6, er7, er8, er9, er10, er11, er12};
    for (int p = 1; p <= 12; ++p) {
        L.w[p][3][1] = bw[p];
        L.w[p][4][1] = ew[p];
    }
    L.w[1][5][1] = -bhh1;
    L.w[9][5][1] = -bhh2;
    L.w[12][5][1] = -bhh3;
    return L;
}

__device__ const LaneWeights kLaneW = make_lane_weights();
}  // namespace dp


__device__ __forceinline__ double pow4(double x)
{
    const double x2 = x * x;
    return x2 * x2;
}

// weights of stage s (2..12) in the three running sums (zero where a stage
// does not enter); selects on compile-time constants, no table lookups
__device__ __forceinline__ void stage_weights(int s, double *wb, double *we, double *wh)
{
    double b = 0.0, e = 0.0, hh = 0.0;
    b = (s == 6) ? dp::b6 : b;     e = (s == 6) ? dp::er6 : e;
    b = (s == 7) ? dp::b7 : b;     e = (s == 7) ? dp::er7 : e;
    b = (s == 8) ? dp::b8 : b;     e = (s == 8) ? dp::er8 : e;
    b = (s == 9) ? dp::b9 : b;     e = (s == 9) ? dp::er9 : e;     hh = (s == 9) ? -dp::bhh2 : hh;
    b = (s == 10) ? dp::b10 : b;   e = (s == 10) ? dp::er10 : e;
    b = (s == 11) ? dp::b11 : b;   e = (s == 11) ? dp::er11 : e;
    b = (s == 12) ? dp::b12 : b;   e = (s == 12) ? dp::er12 : e;   hh = (s == 12) ? -dp::bhh3 : hh;
    *wb = b;
    *we = e;
    *wh = hh;
}

// Lane state
enum Phase : int { kIdle = 0, kStartPass = 1, kStage = 2, kStopTest = 3 };

struct IntArgs {
    const BinaryRec *bins;
    const int *order;
    int B;
    double *traj;
    int cap;
    int *nsteps;
    int *status;
    int *rhs;
    unsigned long long *queue;
    unsigned long long *qslot;  // the work-queue counter (queue[0], or queue[7] for a head of four-warp groups)
    int base;                   // first entry of `order` this queue hands out
    double rtol, atol, h_init, fine_step, step_back, tmax;
    long long max_tries;
};

// component q of a 4-vector held in registers (selects, no local memory)
__device__ __forceinline__ double pick4(const double v[4], int q)
{
    return q == 0 ? v[0] : (q == 1 ? v[1] : (q == 2 ? v[2] : v[3]));
}

template <int G, class X = PairXchg>
__device__ __forceinline__ void integrate_body(const IntArgs &a, X *xch_all, unsigned long long *bars)
{
    // G consecutive lanes carry one binary; every lane of the group keeps the
    // same control state, the Hamiltonian jets and flux multipoles are split
    // over the group, and only the group leader writes scalar results.
    //
    // Groups of 4 or more lanes also split the DOPR853 state: lane q (mod 4)
    // of the group holds component q of y, of the slopes and of the running
    // stage sums, so the stage arguments, the sums and the per-component
    // part of the error norm cost one lane's arithmetic instead of four (on
    // GB300 an FP64 instruction costs the same issue slot whatever the number
    // of active lanes).  The components are gathered by shuffles where the
    // right-hand side or the stopping rule needs all four; the error norm
    // adds the four components by a butterfly that gives every lane the same
    // bits, so all lanes reach the same accept/reject decision.
    //
    // G = 64 / 128: two / four warps per binary (rhs_pair.cuh, rhs_quad.cuh);
    // each warp runs the control state of a 32-lane group, role 0 writes the
    // results.
    constexpr bool kPair = (G >= 64);
    constexpr int NW = G / 32;          // warps per binary (groups of several warps)
    constexpr int GW = kPair ? 32 : G;  // lanes of the group inside one warp
    constexpr bool kDist = (G >= 4);
    constexpr int NC = kDist ? 1 : 4;  // state components held by one lane
    // every lane of a warp on the same stage: the stage sums spread over the
    // lanes (dp::LaneWeights) instead of slopes in local memory
    constexpr bool kReg = (GW == 32);
    const int lane = threadIdx.x & 31;
    const int sub = lane & (GW - 1);
    const int role = kPair ? (int)((threadIdx.x >> 5) % NW) : 0;
    const int cq = kDist ? (sub & 3) : 0;  // the component a distributing lane holds
    const bool leader = (sub == 0) && role == 0;
    const bool writer = kDist ? (sub < 4 && role == 0) : leader;  // writes trajectory components
    const unsigned gmask = (GW == 32) ? 0xffffffffu : (((1u << GW) - 1u) << (lane - sub));
    X *xch = nullptr;
    PairSync ps{0u, 0u, true};
    QuadLane ql{};
    if constexpr (G == 128) ql = quad_lane(role, lane);
    if constexpr (kPair) {
        const int grp = (int)(threadIdx.x / G);
        xch = &xch_all[grp];
        ps.bar = (unsigned)__cvta_generic_to_shared(&bars[grp]);
    }
    // per-lane DOPR853 state (components comp(c) = kDist ? cq : c)
    double k[11][NC];  // slopes k1..k10 (slot 0 unused)
    double y[NC], argl[NC];
    // running sums over the stages of the current attempt: the 8th-order
    // increment sum b_s k_s, the 5th-order error sum er_s k_s and the 3rd-order
    // correction -bhh_s k_s; each stage adds its own term as soon as its slope
    // exists, so the end of a step is short (lanes of one warp reach it at
    // different iterations, and that code runs for the whole warp)
    double acc_b[NC], acc_e[NC], acc_h[NC];
    // kReg: this lane's two running sums (slot group lane >> 2), its weights
    // for the slope the coming right-hand side produces, its component of k1
    double SA = 0.0, SB = 0.0, wA = 0.0, wB = 0.0, k1c = 0.0;
    const int lg = lane >> 2;
    double x = 0.0, h = 0.0, hfix = 0.0, errOld = 1e-4;
    // omega at the last four stopping tests of this pass, newest first (zero
    // before the pass's first row: the reference's omega array restarts per pass)
    double om1 = 0.0, om2 = 0.0, om3 = 0.0, om4 = 0.0;
    int step = 0, first_row = 1, stage = 0, pass = 0, phase = kIdle, b = -1, st = 0;
    bool prevReject = false, fix = false;
    bool nan_seen = false;  // this pass met a NaN error estimate (reported if the pass then fails)
    long long tries = 0;
    unsigned long long n_useful = 0, n_all = 0;  // RHS evaluations (census for the roofline)
    int n_bin = 0;                               // RHS evaluations of the current binary
    const BinaryRec *rec = nullptr;
    double *tr = nullptr;
    bool queue_empty = false;
    int cyc = 0;  // iterations of this warp (the same on every lane)

    for (;;) {
        // ------------------------------------------------ bookkeeping
        if (phase == kIdle && !queue_empty) {
            unsigned long long slot = 0;
            if (leader) slot = atomicAdd(a.qslot, 1ull);
            if constexpr (kPair) {
                if (leader) xch->slot = slot;
                pair_sync(ps);
                const unsigned long long got = slot;
                slot = xch->slot;
                if (!ps.ok) {
                    // the partner warp stopped answering: record the binary
                    // this warp took (if any) and leave
                    if (leader && got < (unsigned long long)a.B) {
                        const int bb = a.order ? a.order[a.base + (int)got] : a.base + (int)got;
                        a.nsteps[bb] = 1;
                        a.status[bb] |= EOB_ST_SYNC | EOB_ST_SHORT;
                    }
                    break;
                }
            } else if (G > 1) {
                slot = __shfl_sync(gmask, slot, lane - sub);
            }
            if (slot >= (unsigned long long)a.B) {
                queue_empty = true;
            } else {
                b = a.order ? a.order[a.base + (int)slot] : a.base + (int)slot;
                rec = &a.bins[b];
                tr = a.traj + (size_t)b * (size_t)a.cap * kTrajStride;
                st = 0;
                pass = 1;
                step = 0;
                n_bin = 0;
                x = 0.0;
                for (int c = 0; c < NC; ++c) y[c] = rec->y0[kDist ? cq : c];
                if (leader) tr[0] = 0.0;
                if (writer)
                    for (int c = 0; c < NC; ++c) tr[1 + (kDist ? cq : c)] = y[c];
                h = a.h_init;
                hfix = a.h_init;
                fix = false;
                phase = kStartPass;
            }
        }
        const bool live = (phase != kIdle);
        // all lanes of the warp idle and the queue exhausted: done
        if (__all_sync(0xffffffffu, !live)) break;
        // Several binaries per warp keep their steps in phase: a step starts
        // (stage 2) only at iteration 0 of the warp's 12-iteration cycle and
        // a pass (its first slope) only at iteration 11, so the end-of-step
        // and stopping blocks, which the whole warp issues whenever any lane
        // needs them, run once per cycle instead of nearly every iteration.
        // A lane that would start off-cycle waits (its right-hand side is
        // evaluated at its own state and discarded): about six iterations
        // per pass and one per rejected step.
        bool wait = false;
        if constexpr (!kReg) {
            const int cpos = cyc % 12;
            wait = (phase == kStage && stage == 2 && cpos != 0) || (phase == kStartPass && cpos != 11);
        }
        ++cyc;
        const bool active = live && !wait;
        n_all += leader ? 1ull : 0ull;
        n_useful += (active && leader) ? 1ull : 0ull;
        n_bin += active ? 1 : 0;

        // ------------------------------------------------ RHS argument
        int out_slot = 1;
        if (phase == kStage) {
            if constexpr (kReg) {
                const double sel = (stage <= 9) ? SA : SB;
                const int src = (((stage <= 9) ? stage - 2 : stage - 10) << 2) | cq;
                argl[0] = y[0] + h * __shfl_sync(0xffffffffu, sel, src);
            } else {
                const int nt = dp::kNTerms[stage];
                for (int c = 0; c < NC; ++c) {
                    double ak = 0.0;
                    for (int t = 0; t < nt; ++t) ak += dp::kStage[stage][t].a * k[dp::kStage[stage][t].slot][c];
                    argl[c] = y[c] + h * ak;
                }
            }
            out_slot = dp::kOutSlot[stage];
        } else if (phase == kStopTest || phase == kStartPass) {
            for (int c = 0; c < NC; ++c) argl[c] = y[c];
        } else {
            // idle lane: evaluate a harmless state of binary 0 (result unused)
            rec = &a.bins[0];
            for (int c = 0; c < NC; ++c) argl[c] = rec->y0[kDist ? cq : c];
        }
        if constexpr (kReg) {
            const int p = (phase == kStage) ? stage : 1;
            wA = dp::kLaneW.w[p][lg][0];
            wB = dp::kLaneW.w[p][lg][1];
        }
        double arg[4];
        if constexpr (kDist) {
#pragma unroll
            for (int q = 0; q < 4; ++q) arg[q] = __shfl_sync(0xffffffffu, argl[0], q, GW);
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) arg[q] = argl[q];
        }

        // ------------------------------------------------ the one RHS per loop
        double kk[4];
        if constexpr (G == 1) eob_rhs(rec->ham, rec->flux, arg, kk);
        else if constexpr (G == 64) eob_rhs_pair(rec->jets, rec->flux, arg, kk, lane, role, *xch, ps);
        else if constexpr (G == 128) eob_rhs_quad(rec->jets, rec->flux, ql, arg, kk, lane, role, *xch, ps);
        else eob_rhs_group<G>(rec->jets, rec->flux, arg, kk, sub);
        if constexpr (kPair) {
            if (!ps.ok) {
                // a pair barrier ran out of time: end this binary with what it has
                if (leader && active) {
                    a.nsteps[b] = step + 1;
                    a.status[b] |= st | EOB_ST_SYNC;
                    a.rhs[b] = n_bin;
                }
                break;
            }
        }
        if (!active) continue;
        double km[NC];  // this lane's components of the new slope
        if constexpr (kDist) km[0] = pick4(kk, cq);
        else
            for (int c = 0; c < NC; ++c) km[c] = kk[c];

        // ------------------------------------------------ advance the lane
        if (phase == kStartPass) {
            if constexpr (kReg) {
                k1c = km[0];
                SA = wA * km[0];
                SB = wB * km[0];
            } else {
                for (int c = 0; c < NC; ++c) {
                    k[1][c] = km[c];
                    acc_b[c] = dp::b1 * km[c];
                    acc_e[c] = dp::er1 * km[c];
                    acc_h[c] = -dp::bhh1 * km[c];
                }
            }
            errOld = 1e-4;
            prevReject = false;
            nan_seen = false;
            tries = 0;
            first_row = step + 1;
            om1 = om2 = om3 = om4 = 0.0;
            stage = 2;
            phase = kStage;
            continue;
        }
        if (phase == kStage) {
            if constexpr (kReg) {
                SA = fma(wA, km[0], SA);
                SB = fma(wB, km[0], SB);
            } else {
                double wb, we, wh;
                stage_weights(stage, &wb, &we, &wh);
                for (int c = 0; c < NC; ++c) {
                    k[out_slot][c] = km[c];
                    acc_b[c] = fma(wb, km[c], acc_b[c]);
                    acc_e[c] = fma(we, km[c], acc_e[c]);
                    acc_h[c] = fma(wh, km[c], acc_h[c]);
                }
            }
            if (stage < 12) {
                ++stage;
                continue;
            }
            if constexpr (kReg) {
                // the increment, error and correction sums of this lane's component
                acc_b[0] = __shfl_sync(0xffffffffu, SB, 12 | cq);
                acc_e[0] = __shfl_sync(0xffffffffu, SB, 16 | cq);
                acc_h[0] = __shfl_sync(0xffffffffu, SB, 20 | cq);
            }
            // error estimate (src/DOPR853.cu:537-618) from the running sums
            double e1 = 0.0, e2 = 0.0, ynew[NC];
            for (int c = 0; c < NC; ++c) {
                const double t = acc_b[c];
                ynew[c] = y[c] + h * t;
                const double mx = (y[c] > ynew[c]) ? y[c] : ynew[c];
                const double sk = eob_rcp(a.atol + a.rtol * mx);
                e2 += pow4((t + acc_h[c]) * sk);
                e1 += pow4(acc_e[c] * sk);
            }
            if constexpr (kDist) {
                // the four components' terms summed by a butterfly over the
                // lanes that hold them, (t0 + t1) + (t2 + t3): addition
                // commutes, so every lane gets the same bits
                e1 += __shfl_xor_sync(gmask, e1, 1, GW);
                e2 += __shfl_xor_sync(gmask, e2, 1, GW);
                e1 += __shfl_xor_sync(gmask, e1, 2, GW);
                e2 += __shfl_xor_sync(gmask, e2, 2, GW);
            }
            double denom = e1 + 0.01 * e2;
            denom = (denom < 0.0) ? 1.0 : denom;
            double err = fabs(h) * e1 * (0.5 * rsqrt(denom));  // |h| e1 sqrt(1 / (4 denom))
            // A NaN error estimate -- a trial stage outside the Hamiltonian's
            // domain, as when too long a step in the plunge carries a stage
            // past the horizon -- counts as +inf: the attempt is rejected with
            // the smallest scale.  (The reference's controller would carry
            // the NaN into h, after which its integration cannot go on.)
            // Tested on the bits: a comparison of doubles takes an FP64 slot.
            const bool err_nan = ((unsigned long long)__double_as_longlong(err) << 1) > (0x7ff0000000000000ull << 1);
            if (err_nan) {
                err = __longlong_as_double(0x7ff0000000000000LL);
                nan_seen = true;
            }
            const double hOld = h;
            // controller (src/DOPR853.cu:674-762), beta = 0
            bool ok;
            if (err <= 1.0) {
                double scale;
                if (err == 0.0) {
                    scale = dp::maxscale;
                } else {
                    scale = dp::safe * eob_inv_eighth_root(err);
                    if (scale > dp::maxscale) scale = dp::maxscale;
                    else if (scale < dp::minscale) scale = dp::minscale;
                }
                if (prevReject && scale > 1.0) scale = 1.0;
                h = h * scale;
                double eo = err;
                if (eo < 1e-4) eo = 1e-4; else if (eo > 1e300) eo = 1e300;
                errOld = eo;
                prevReject = false;
                ok = true;
            } else {
                prevReject = true;
                double t = dp::safe * eob_inv_eighth_root(err);
                if (t < dp::minscale) t = dp::minscale; else if (t > 1e300) t = 1e300;
                h = h * t;
                ok = false;
            }
            (void)errOld;
            if (fix && !ok) hfix /= 2.0;
            if (fix) h = hfix;
            ++tries;
            const bool bad = !(h == h) || h == 0.0;
            if (ok) {
                for (int c = 0; c < NC; ++c) y[c] = ynew[c];
                x = x + hOld;
                ++step;
                double *row = tr + (size_t)step * kTrajStride;
                if (leader) row[0] = x;
                if (writer)
                    for (int c = 0; c < NC; ++c) row[1 + (kDist ? cq : c)] = y[c];
                phase = kStopTest;  // next RHS: f(y_new) for the stopping rule and the next k1
                if (bad) st |= EOB_ST_NAN;
            } else {
                // first attempt of the pass rejected: the reference's stop flags
                // start true, so the pass ends here (new_Dormand_horiz.py:623-761)
                bool end = (step == first_row - 1);
                if (end) st |= EOB_ST_STOP_REJECT;
                if (bad) { st |= EOB_ST_NAN; end = true; }
                if (tries >= a.max_tries) { st |= EOB_ST_TRIES | (nan_seen ? EOB_ST_NAN : 0); end = true; }
                if (!end) {
                    stage = 2;  // retry with the new h; k1 unchanged
                    if constexpr (kReg) {
                        SA = dp::kLaneW.w[1][lg][0] * k1c;
                        SB = dp::kLaneW.w[1][lg][1] * k1c;
                    } else {
                        for (int c = 0; c < NC; ++c) {
                            acc_b[c] = dp::b1 * k[1][c];
                            acc_e[c] = dp::er1 * k[1][c];
                            acc_h[c] = -dp::bhh1 * k[1][c];
                        }
                    }
                    continue;
                }
                phase = -1;  // fall through to end-of-pass handling
            }
            if (phase == kStopTest && !bad) continue;
            if (phase == kStopTest && bad) phase = -1;
        }
        bool end_pass = false;
        if (phase == kStopTest) {
            // stopping rule on the accepted state (kk = f(y))
            if constexpr (kReg) {
                k1c = km[0];
                SA = wA * km[0];
                SB = wB * km[0];
            } else {
                for (int c = 0; c < NC; ++c) {
                    k[1][c] = km[c];
                    acc_b[c] = dp::b1 * km[c];
                    acc_e[c] = dp::er1 * km[c];
                    acc_h[c] = -dp::bhh1 * km[c];
                }
            }
            const double r = arg[0], drdt = kk[0], omega = kk[1], dprdt = kk[2];  // arg = y here
            int code = 0;
            if (r < 1.0) code = 2;
            else if (r < 6.0 && drdt > 0.0) code = 3;
            else if (r < 6.0 && dprdt > 0.0) code = 4;
            else if (step > 5) {
                // history rows written in this pass, zero before (omega array restarts per pass)
                const bool c2 = omega < om1;
                // the reference's differences om_j - om_(j+1) < 0, as comparisons
                // (equal for finite values: a nonzero difference is exact in sign)
                const bool c3 = (om3 < om4) && (om2 < om3) && (om1 < om2);
                if (r < 6.0 && c2 && c3) code = 5;
            }
            om4 = om3;
            om3 = om2;
            om2 = om1;
            om1 = omega;
            end_pass = (code != 0) || (x >= a.tmax) || (step >= a.cap - 1) || (tries >= a.max_tries);
            if (step >= a.cap - 1) st |= EOB_ST_MAXSTEP;
            if (tries >= a.max_tries && code == 0) st |= EOB_ST_TRIES;
            if (!end_pass) {
                stage = 2;
                phase = kStage;
                continue;
            }
        } else {
            end_pass = true;  // rejected first attempt, non-finite state or attempt limit
        }
        // ------------------------------------------------ end of a pass
        if (pass == 1 && end_pass) {
            // step back (eob/seobnrv4phm.py:2096-2114): t_stop is the time of
            // the second-to-last stored row; restart from the row before the one
            // closest to t_stop - step_back
            const int S1 = step;
            if (S1 < 2 || (st & (EOB_ST_NAN | EOB_ST_TRIES))) {
                st |= EOB_ST_SHORT;
                if (leader) {
                    a.nsteps[b] = S1 + 1;
                    a.status[b] |= st;
                    a.rhs[b] = n_bin;
                }
                phase = kIdle;
                continue;
            }
            // the rows were written by other lanes of the group: make them visible
            __syncwarp(gmask);
            const double t_stop = tr[(size_t)(S1 - 1) * kTrajStride];
            const double t_des = t_stop - a.step_back;
            int idx = 0;
            double best = fabs(tr[0] - t_des);
            for (int i = 1; i <= S1; ++i) {
                const double d = fabs(tr[(size_t)i * kTrajStride] - t_des);
                if (d < best) { best = d; idx = i; }
            }
            if (idx < 1) { idx = 1; st |= EOB_ST_SHORT; }
            step = idx - 1;
            const double *row = tr + (size_t)step * kTrajStride;
            x = row[0];
            for (int c = 0; c < NC; ++c) y[c] = row[1 + (kDist ? cq : c)];
            pass = 2;
            h = a.fine_step;
            hfix = a.fine_step;
            fix = true;
            st &= ~EOB_ST_STOP_REJECT;
            phase = kStartPass;
            continue;
        }
        // pass 2 finished: binary done
        if (leader) {
            a.nsteps[b] = step + 1;
            a.status[b] |= st;
            a.rhs[b] = n_bin;
        }
        phase = kIdle;
    }
    if (leader) {
        atomicAdd(&a.queue[4], n_useful);
        atomicAdd(&a.queue[5], n_all);
    }
}

// One kernel per group size.  Groups of 4+ lanes hold little per-lane state
// and may use up to 255 registers (one or two warps per SM sub-partition are
// resident); one- and two-lane groups keep the compiler's default budget so
// that several warps share each sub-partition.
template <int G>
__global__ void __launch_bounds__(256, 1) k_integrate(IntArgs a)
{
    integrate_body<G>(a, (PairXchg *)nullptr, nullptr);
}

template <int G>
__global__ void __launch_bounds__(256) k_integrate_lane(IntArgs a)
{
    integrate_body<G>(a, (PairXchg *)nullptr, nullptr);
}

// warp pairs: blockDim.x a multiple of 64, at most kPairMax pairs
__global__ void __launch_bounds__(256, 1) k_integrate_pair(IntArgs a)
{
    __shared__ PairXchg xch[kPairMax];
    __shared__ unsigned long long bars[kPairMax];
    pair_init(bars, (int)(blockDim.x / 64));
    integrate_body<64>(a, xch, bars);
}

// The longest binaries on four warps, the rest on groups of GB lanes (warp
// pairs for GB = 64), in one launch of 128-thread blocks: blocks [0, nq)
// first run four-warp groups over the first `head` binaries of the order
// (their own queue counter, queue[7]), then join the other blocks over the
// remaining binaries.
template <int GB>
__global__ void __launch_bounds__(128, 1) k_integrate_mixed(IntArgs a, int nq, int head)
{
    __shared__ QuadXchg xq;
    __shared__ PairXchg xp[2];
    __shared__ unsigned long long bq[1], bp[2];
    if (threadIdx.x == 0) {
        const unsigned aq = (unsigned)__cvta_generic_to_shared(&bq[0]);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(aq), "r"(128) : "memory");
        for (int p = 0; p < 2; ++p) {
            const unsigned ap = (unsigned)__cvta_generic_to_shared(&bp[p]);
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(ap), "r"(64) : "memory");
        }
    }
    __syncthreads();
    if ((int)blockIdx.x < nq) {
        IntArgs aq = a;
        aq.B = head;
        aq.qslot = &a.queue[7];
        integrate_body<128, QuadXchg>(aq, &xq, bq);
        __syncthreads();  // the block leaves the four-warp queue together
    }
    IntArgs ap = a;
    ap.base = a.base + head;
    ap.B = a.B - head;
    if constexpr (GB == 64) integrate_body<64>(ap, xp, bp);
    else integrate_body<GB>(ap, (PairXchg *)nullptr, nullptr);
}

// warp quads: blockDim.x a multiple of 128, at most kQuadMax quads
__global__ void __launch_bounds__(256, 1) k_integrate_quad(IntArgs a)
{
    __shared__ QuadXchg xch[kQuadMax];
    __shared__ unsigned long long bars[kQuadMax];
    group_init(bars, (int)(blockDim.x / 128), 128);
    integrate_body<128, QuadXchg>(a, xch, bars);
}

template <int G>
cudaError_t launch_g(const IntArgs &a, int bs, int grid, cudaStream_t s)
{
    // little or no shared memory: give the SM's unified L1/shared storage to
    // L1, where the lanes' coefficient tables and slope arrays live
    void (*kern)(IntArgs);
    if constexpr (G == 128) kern = k_integrate_quad;
    else if constexpr (G == 64) kern = k_integrate_pair;
    else if constexpr (G >= 4) kern = k_integrate<G>;
    else kern = k_integrate_lane<G>;
    static bool carveout_set = false;
    if (!carveout_set) {
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        carveout_set = true;
    }
    if (grid <= 0) {
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, bs, 0);
        if (per_sm < 1) per_sm = 1;
        // at most one warp per SM sub-partition, so that no binary's chain
        // shares an FP64 pipe (a warp alone on a sub-partition keeps its FP64
        // pipe ~80 % busy); later binaries wait in the queue instead, which
        // hands out the longest first.  With three warps per sub-partition a
        // ragged batch's longest binaries run three times slower (65 536
        // one-lane binaries: 22 s in chunks at three warps, 11 s in one launch
        // at one warp)
        {
            const int cap = (4 * 32 + bs - 1) / bs;
            if (per_sm > cap) per_sm = cap;
        }
        const long long lanes = (long long)a.B * G;
        const long long need = (lanes + bs - 1) / bs;
        grid = (int)(need < (long long)nsm * per_sm ? need : (long long)nsm * per_sm);
        if (grid < 1) grid = 1;
    }
    kern<<<grid, bs, 0, s>>>(a);
    return cudaGetLastError();
}

// Lanes per binary chosen from the batch size: a power of two in [1, 64]
// (64: a warp pair, with a head of four-warp groups; 128 only on request).  One lane
// per binary is the most efficient use of the FP64 pipe; more lanes per
// binary shorten each binary's critical path when the batch cannot fill the
// device.
int auto_lanes_per_binary(int B)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // up to two warps' worth of lanes per SM sub-partition: the grid keeps one
    // warp per sub-partition resident and the work queue feeds it the rest,
    // longest binaries first, so a batch bound by its longest binary gets the
    // shortest chain (e.g. B = 4096 -> 8 lanes)
    const long long target = (long long)nsm * 4 * 32 * 2;
    int G = 1;
    while (G < 32 && (long long)B * (G * 2) <= target) G *= 2;
    // warp pairs cost about 1.3x the issue slots of a 32-lane group per
    // right-hand side but shorten the chain 1.5x: worth it while the batch's
    // total work stays below its longest binary's chain (up to four warps'
    // worth of lanes per sub-partition, e.g. B = 1024 -> 64)
    if (G == 32 && (long long)B * 64 <= 2 * target) G = 64;
    return G;
}

cudaError_t launch_integrate(const Ws &w, const RunArgs &ra, cudaStream_t s)
{
    IntArgs a;
    a.bins = w.bins;
    a.order = ra.order;
    a.B = ra.B;
    a.traj = w.traj;
    a.cap = w.L.Lc;
    a.nsteps = w.nsteps;
    a.status = w.status;
    a.rhs = w.rhs;
    a.queue = w.queue;
    a.rtol = ra.opt.rtol;
    a.atol = ra.opt.atol;
    a.h_init = ra.opt.h_init;
    a.fine_step = ra.opt.fine_step;
    a.step_back = ra.opt.step_back;
    a.tmax = 1e7 * 1e6;
    a.max_tries = ra.opt.max_tries > 0 ? ra.opt.max_tries : 2LL * w.L.Lc + 100;
    const int bs = (ra.opt.block > 0 && ra.opt.block <= 256 && ra.opt.block % 32 == 0) ? ra.opt.block : 128;
    int G = ra.opt.lanes_per_binary;
    if (G != 1 && G != 2 && G != 4 && G != 8 && G != 16 && G != 32 && G != 64 && G != 128)
        G = auto_lanes_per_binary(ra.B);
    a.qslot = &w.queue[0];
    a.base = 0;
    cudaError_t e = cudaMemsetAsync(w.queue, 0, sizeof(unsigned long long) * 8, s);
    if (e != cudaSuccess) return e;
    // a head of the longest binaries on four warps, the rest on warp pairs
    // (automatic: the 16 longest, at most B / 64) or, when asked for, on
    // lane groups of 8 .. 32
    if ((G == 64 || (G >= 8 && G <= 32)) && ra.opt.head_quads != 0) {
        int dev = 0, nsm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        int head = ra.opt.head_quads;
        if (head < 0) head = (G == 64 && ra.B >= 64) ? (ra.B / 64 < 16 ? ra.B / 64 : 16) : 0;
        if (head > ra.B) head = ra.B;
        if (head > 0) {
            void (*kern)(IntArgs, int, int) = G == 64 ? k_integrate_mixed<64>
                                              : G == 32 ? k_integrate_mixed<32>
                                              : G == 16 ? k_integrate_mixed<16>
                                                        : k_integrate_mixed<8>;
            static bool carve[4] = {false, false, false, false};
            const int ci = G == 64 ? 0 : G == 32 ? 1 : G == 16 ? 2 : 3;
            if (!carve[ci]) {
                cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
                carve[ci] = true;
            }
            const int nq = head < nsm ? head : nsm;
            const long long need = nq + ((long long)(ra.B - head) * G + 127) / 128;
            const int grid = (int)(need < nsm ? need : nsm);
            kern<<<grid > nq ? grid : nq, 128, 0, s>>>(a, nq, head);
            return cudaGetLastError();
        }
    }
    switch (G) {
        case 1: return launch_g<1>(a, bs, ra.opt.grid, s);
        case 2: return launch_g<2>(a, bs, ra.opt.grid, s);
        case 4: return launch_g<4>(a, bs, ra.opt.grid, s);
        case 8: return launch_g<8>(a, bs, ra.opt.grid, s);
        case 16: return launch_g<16>(a, bs, ra.opt.grid, s);
        case 32: return launch_g<32>(a, bs, ra.opt.grid, s);
        case 64: return launch_g<64>(a, bs % 64 == 0 ? bs : 128, ra.opt.grid, s);
        default: return launch_g<128>(a, bs % 128 == 0 ? bs : 128, ra.opt.grid, s);
    }
}

}  // namespace eob
