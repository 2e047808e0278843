// Shared device-side definitions of the GB300 EOB pipeline: per-binary
// record, status bits, and the workspace layout carved out of one
// caller-provided device buffer (the library never allocates).
#pragma once
#include <cstddef>
#include <cstdint>
#include "physics/fac_coeffs.h"
#include "physics/ham_coeffs.h"
#include "physics/ham_eval.h"
#include "physics/flux_eval.h"
#include "physics/mode_eval.h"
#include "../../include/eobgb300.h"

namespace eob {

// Everything the integrator needs for one binary (built once by the setup
// kernel; read-only afterwards).
struct BinaryRec {
    HamCoeffs ham;
    HamJets jets;      // the same Hamiltonian as 16 jets for lane groups
    FluxTable flux;
    double pre_re[kNumLM], pre_im[kNumLM];
    double m1s, m2s, chi1, chi2, Mt, omega0, nu;
    double y0[4];      // initial state (r0, 0, pr0, pphi0)
    int ic_iters, pad;
};

constexpr int kMaxModes = 5;
constexpr int kChunk = 1024;   // samples per synthesis work item
constexpr int kTrajStride = 5; // t, r, phi, pr, pphi per trajectory row

struct WsLayout {
    size_t bins, fac, traj, nsteps, status, rhs, queue, row_off, chunk_off, npts, tin, ys, cA, cB, cC, cD, partial, f32,
        dataf, total;
    // merger-ringdown section (after everything else; present when imr): splines of r
    // and p_r ([2][rows] each), attachment records, per-binary attachment
    size_t imr_ys, imr_cA, imr_cB, imr_cC, imr_cD, imr_rec, imr_bin, imr_total;
    int Bc, Lc, Kc, Nc, nsubs, max_chunks, imr;
};

// Merger-ringdown attachment (eob/seobnrv4phm.py:2374-2557), per binary and
// mode: the NQC coefficients, the ringdown ansatz coefficients and the match
// point.  t_match is on the uniform grid of the inspiral (t_k = k dT + t0, [M]).
struct ImrRec {
    double a1, a2, a3, b1, b2;         // NQC amplitude and phase coefficients
    double c1c, c2c, c1f, c2f;         // ringdown amplitude
    double d1c, d1f, d2f, phi_match;   // ringdown phase
    double om_re, om_im;               // QNM omega_R, 1/tau of the mode (remnant units applied)
    double eta;
};

// per binary: attachment sample, waveform length with the ringdown, flags
struct ImrBin {
    int idx;        // last inspiral sample (nearest the attachment time)
    int npts;       // samples of the IMR waveform (idx + ringdown samples)
    int fail;       // nonzero: a window fell outside the waveform (inspiral only)
    int on;         // 1: the synthesis attaches the ringdown for this binary
};

constexpr int kImrWin = 256;  // longest fit window on the uniform grid [samples]

EOB_HD constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Offsets of every array inside the workspace for capacities (Bc binaries,
// Lc trajectory rows per binary, Kc modes, Nc samples); imr appends the
// merger-ringdown section (the offsets before it do not change).
EOB_HD constexpr WsLayout ws_layout(int Bc, int Lc, int Kc, int Nc, int imr = 0)
{
    WsLayout w{};
    w.Bc = Bc; w.Lc = Lc; w.Kc = Kc; w.Nc = Nc; w.imr = imr;
    w.nsubs = 1 + 2 * Kc;
    w.max_chunks = Bc * ((Nc + kChunk - 1) / kChunk);
    const size_t rows = (size_t)Bc * (size_t)Lc;
    size_t o = 0;
    w.bins = o;      o = align256(o + sizeof(BinaryRec) * (size_t)Bc);
    w.fac = o;       o = align256(o + sizeof(FacCoeffs) * (size_t)Bc);
    w.traj = o;      o = align256(o + sizeof(double) * kTrajStride * rows);
    w.nsteps = o;    o = align256(o + sizeof(int) * (size_t)Bc);
    w.status = o;    o = align256(o + sizeof(int) * (size_t)Bc);
    w.rhs = o;       o = align256(o + sizeof(int) * (size_t)Bc);
    w.queue = o;     o = align256(o + sizeof(unsigned long long) * 8);
    w.row_off = o;   o = align256(o + sizeof(long long) * ((size_t)Bc + 1));
    w.chunk_off = o; o = align256(o + sizeof(long long) * ((size_t)Bc + 1));
    w.npts = o;      o = align256(o + sizeof(int) * (size_t)Bc);
    w.tin = o;       o = align256(o + sizeof(double) * rows);
    w.ys = o;        o = align256(o + sizeof(double) * rows * w.nsubs);
    w.cA = o;        o = align256(o + sizeof(double) * rows * w.nsubs);
    w.cB = o;        o = align256(o + sizeof(double) * rows * w.nsubs);
    w.cC = o;        o = align256(o + sizeof(double) * rows * w.nsubs);
    w.cD = o;        o = align256(o + sizeof(double) * rows * w.nsubs);
    w.partial = o;   o = align256(o + sizeof(double) * (size_t)w.max_chunks);
    w.f32 = o;       o = align256(o + sizeof(float) * 4 * rows * 2 * (size_t)Kc);
    w.dataf = o;     o = align256(o + sizeof(float) * (size_t)Nc);
    w.total = o;
    w.imr_ys = o;    o = align256(o + sizeof(double) * rows * 2);
    w.imr_cA = o;    o = align256(o + sizeof(double) * rows * 2);
    w.imr_cB = o;    o = align256(o + sizeof(double) * rows * 2);
    w.imr_cC = o;    o = align256(o + sizeof(double) * rows * 2);
    w.imr_cD = o;    o = align256(o + sizeof(double) * rows * 2);
    w.imr_rec = o;   o = align256(o + sizeof(ImrRec) * (size_t)Bc * (size_t)Kc);
    w.imr_bin = o;   o = align256(o + sizeof(ImrBin) * (size_t)Bc);
    w.imr_total = o;
    if (imr) w.total = o;
    return w;
}

// Typed views of the workspace.
struct Ws {
    BinaryRec *bins;
    FacCoeffs *fac;
    double *traj;
    int *nsteps, *status;
    int *rhs;                   // right-hand sides evaluated for each binary (both passes, all attempts)
    unsigned long long *queue;  // [0] work queue, [1] total rows, [2] total chunks, [3] sum data^2 (double bits),
                                // [4] RHS evaluations for binaries, [5] RHS evaluations incl. idle lanes,
                                // [6] 1 if the spline build wrote FP32 copies (mixed precision)
    long long *row_off, *chunk_off;
    int *npts;
    double *tin, *ys, *cA, *cB, *cC, *cD, *partial;
    float *f32;    // mixed precision: y, c1, c2, c3 of the mode series, [4][2K][rows]
    float *dataf;  // mixed precision: data in FP32
    // merger-ringdown section (null when the workspace has none)
    double *imr_ys, *imr_cA, *imr_cB, *imr_cC, *imr_cD;  // series 0: r, 1: p_r
    ImrRec *imr_rec;                                     // [b * Kc + q]
    ImrBin *imr_bin;
    WsLayout L;
};

inline Ws ws_views(void *base, const WsLayout &L)
{
    char *b = (char *)base;
    Ws w;
    w.bins = (BinaryRec *)(b + L.bins);
    w.fac = (FacCoeffs *)(b + L.fac);
    w.traj = (double *)(b + L.traj);
    w.nsteps = (int *)(b + L.nsteps);
    w.status = (int *)(b + L.status);
    w.rhs = (int *)(b + L.rhs);
    w.queue = (unsigned long long *)(b + L.queue);
    w.row_off = (long long *)(b + L.row_off);
    w.chunk_off = (long long *)(b + L.chunk_off);
    w.npts = (int *)(b + L.npts);
    w.tin = (double *)(b + L.tin);
    w.ys = (double *)(b + L.ys);
    w.cA = (double *)(b + L.cA);
    w.cB = (double *)(b + L.cB);
    w.cC = (double *)(b + L.cC);
    w.cD = (double *)(b + L.cD);
    w.partial = (double *)(b + L.partial);
    w.f32 = (float *)(b + L.f32);
    w.dataf = (float *)(b + L.dataf);
    const bool imr = L.imr != 0;
    w.imr_ys = imr ? (double *)(b + L.imr_ys) : nullptr;
    w.imr_cA = imr ? (double *)(b + L.imr_cA) : nullptr;
    w.imr_cB = imr ? (double *)(b + L.imr_cB) : nullptr;
    w.imr_cC = imr ? (double *)(b + L.imr_cC) : nullptr;
    w.imr_cD = imr ? (double *)(b + L.imr_cD) : nullptr;
    w.imr_rec = imr ? (ImrRec *)(b + L.imr_rec) : nullptr;
    w.imr_bin = imr ? (ImrBin *)(b + L.imr_bin) : nullptr;
    w.L = L;
    return w;
}

// Kernel launchers (defined in the k_*.cu translation units).
struct RunArgs {
    const double *params;  // [B][5]: m1, m2 [Msun], chi1, chi2, f0 [Hz]
    const int *order;      // work order (longest first) or null
    int B;
    int K;
    int ells[kMaxModes], mms[kMaxModes];
    double dt;
    const double *data;
    int N;
    double amp;
    eob_options opt;
    double *lnl;
    int *status_out;
};

cudaError_t launch_setup(const Ws &w, const RunArgs &a, cudaStream_t s);
cudaError_t launch_integrate(const Ws &w, const RunArgs &a, cudaStream_t s);
cudaError_t launch_prepare_post(const Ws &w, const RunArgs &a, cudaStream_t s);
// merger-ringdown attachment after the splines (a.opt.imr, workspace with the section)
cudaError_t launch_imr(const Ws &w, const RunArgs &a, cudaStream_t s);
// mode 0: lnL (a.data, a.lnl; a.opt.precision 1 = mixed); 1: summed strain out[B][N];
// 2: per-mode out[B][K][N], t clamped to each end
cudaError_t launch_synth(const Ws &w, const RunArgs &a, int mode, double *out, cudaStream_t s);

}  // namespace eob
