/* eobgb300.h -- C ABI of the GB300-native EOB waveform + likelihood path.
 *
 * A drop-in native layer for the batched SEOBNR effective-one-body path of
 * mikekatz04/EOBGPU.  Every entry point takes plain device pointers and
 * sizes, an explicit cudaStream_t, allocates nothing, and returns an int
 * status (0 = success, see EOB_E_* below) instead of exiting the process as the
 * reference's gpuErrchk does (include/global.h:13-20).  Calls are asynchronous
 * on the given stream; the reference synchronises after every launch.
 *
 * Array layouts follow the reference's Cython layer (src/eob.pyx,
 * src/dopr853.pyx, src/tdinterp.pyx): state arg[4][n] = (r, phi, pr, pphi),
 * additionalArgs[80][n] = (m1, m2, chi1, chi2, omega, K, d5, dSO, dSS,
 * h22_calib, then Re/Im of the 35 Newtonian prefixes (l = 2..8, m = 1..l)).
 */
#ifndef EOBGB300_H
#define EOBGB300_H

#include <stddef.h>
#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define EOB_OK 0
#define EOB_E_ARG 1        /* invalid argument / capacity exceeded */
#define EOB_E_CUDA 2       /* a CUDA runtime call failed */
#define EOB_E_CTX 3        /* context not initialised */

/* per-binary status bits of the fused pipeline */
#define EOB_ST_IC_NOCONV 1     /* (r0, pphi0) Newton did not converge */
#define EOB_ST_MAXSTEP 2       /* trajectory hit the row capacity (max_step) */
#define EOB_ST_NAN 4           /* non-finite state or error estimate */
#define EOB_ST_TRIES 8         /* step-attempt limit reached (no progress) */
#define EOB_ST_SHORT 16        /* too few rows for the step-back restart or the spline */
#define EOB_ST_STOP_REJECT 32  /* first step of a pass rejected (reference stops there) */
#define EOB_ST_SYNC 64         /* the warps of a multi-warp group (lanes_per_binary 64 or 128) lost step: a
                                  barrier wait ran out of time and the binary was ended early */
#define EOB_ST_IMR 128         /* merger-ringdown requested but not attached (a fit window fell outside the
                                  inspiral or exceeded 256 samples): the template is the inspiral alone */

typedef struct eob_options {
    double rtol, atol;      /* DOPR853 tolerances; reference: 1e-12, 1e-12 (src/DOPR853.cu:7-8) */
    double h_init;          /* first step [M]; reference 0.01 (eob/new_Dormand_horiz.py:527-531) */
    double step_back;       /* restart offset [M]; reference 10 (eob/seobnrv4phm.py:2072) */
    double fine_step;       /* fixed fine step [M]; reference 0.05 */
    int ic_mode;            /* 0: reference-effective p_r0, 1: physical (exact Hessian) */
    int precision;          /* 0: FP64 synthesis + lnL; 1: mixed -- phase in FP64 and reduced mod 2 pi, amplitude
                               splines, sin/cos and the residual in FP32 with compensated sums (pass the same value
                               to the prepare and synth calls) */
    int block;              /* integrator threads per block (0 = default) */
    int grid;               /* integrator blocks (0 = one wave of resident blocks) */
    long long max_tries;    /* step attempts per pass before giving up (0 = 2 * max_steps + 100) */
    int lanes_per_binary;   /* integrator lanes per binary: 1, 2, 4, 8, 16, 32, 64 (two warps on two SM
                               sub-partitions) or 128 (four warps, one per sub-partition of an SM);
                               0 = chosen from the batch size */
    int spline_tile;        /* spline build: series (one warp each) per block, 1..8 (0 = default 4) */
    int head_quads;         /* with warp pairs or groups of 8, 16 or 32 lanes: the head_quads longest
                               binaries (first in `order`) on four warps each, concurrently with the rest
                               (-1 = chosen from the batch: with warp pairs min(B / 64, 16), otherwise
                               none; 0 = none) */
    int imr;                /* 1: complete each waveform with the NQC correction and the merger-ringdown
                               (eob/seobnrv4phm.py:2374-2557; needs a workspace of eob_workspace_bytes_imr,
                               FP64 synthesis); 0 (default): the inspiral up to the trajectory's end */
} eob_options;

void eob_options_default(eob_options *o);

/* ---------------------------------------------------------------------------
 * Fused path: parameters -> lnL for a batch (no counterpart as one call in the
 * reference; replaces SEOBNRv4PHM.__call__ + BBHWaveformTD's mode sum and its
 * likelihood, eob/seobnrv4phm.py:2628-2726, 636-721).
 * params[B][5] = (m1, m2 [Msun], chi1z, chi2z, f0 [Hz]); data[N];
 * lnl[B] = -1/2 sum_{k<N} (data_k - amp Re sum_lm h_lm(t_k))^2 with h = 0
 * past each binary's last sample; status[B] per-binary EOB_ST_* bits.  A
 * binary left without a template (its trajectory failed: EOB_ST_SHORT with
 * the reason's bit) gets lnl = NaN.
 * order[B] (may be NULL) is the order in which the persistent integrator
 * takes binaries from its queue.
 */
size_t eob_workspace_bytes(int max_batch, int max_steps, int max_modes, int max_samples);
/* the same with the merger-ringdown section (eob_options.imr = 1) appended */
size_t eob_workspace_bytes_imr(int max_batch, int max_steps, int max_modes, int max_samples);
int eob_waveform_lnl(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                     int max_samples, const double *params, const int *order, int B, const int *ells,
                     const int *mms, int K, double dt, const double *data, int N, double amp,
                     const eob_options *opt, double *lnl, int *status, cudaStream_t stream);

/* The same path in two phases, for callers that inspect per-binary results
 * between them (trajectory rows, sample counts; eob_workspace_views):
 * eob_prepare runs setup, initial conditions, the integrator, the multipoles
 * on the trajectory and the splines; eob_synth_lnl / eob_synth_strain then
 * evaluate the splines on the uniform grid t_k = k dt of each binary.  The
 * synth calls must get the same B, K, modes and dt as the prepare call. */
int eob_prepare(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes, int max_samples,
                const double *params, const int *order, int B, const int *ells, const int *mms, int K, double dt,
                const eob_options *opt, int *status, cudaStream_t stream);
/* eob_prepare in parts (for timing each stage): stages bit 1 = setup and
 * initial conditions, 2 = integrator, 4 = multipoles and splines. */
int eob_prepare_stages(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                       int max_samples, const double *params, const int *order, int B, const int *ells, const int *mms,
                       int K, double dt, const eob_options *opt, int stages, cudaStream_t stream);
int eob_synth_lnl(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                  int max_samples, int B, const int *mms, int K, double dt, const double *data, int N, double amp,
                  const eob_options *opt, double *lnl, int *status, cudaStream_t stream);
/* per_mode = 0: out[B][N] complex = sum_lm h_lm(t_k), zero past each binary's last sample;
 * per_mode = 1: out[B][K][N] complex per mode with t_k clamped to each binary's last sample
 * (the uniform-grid modes of SEOBNRv4PHM.__call__, eob/seobnrv4phm.py:2336-2372). */
int eob_synth_strain(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                     int max_samples, int B, const int *mms, int K, double dt, int N, int per_mode, double *out,
                     int *status, cudaStream_t stream);

/* eob_waveform_lnl for callers that cannot allocate device memory (no
 * counterpart in the reference).  Code that runs inside another framework's
 * memory pool, a plugin host without allocator access, or a process that must
 * not call cudaMalloc while other work is in flight passes only its inputs
 * and outputs; the scratch is a fixed __device__ array of
 * eob_noalloc_scratch_bytes() bytes (13 588 736 bytes, 13.6 MB) that every
 * GPU loading the library keeps until exit.  Limits: B <= 16 binaries, K = 1 mode,
 * N <= 8192 samples, at most 4096 trajectory rows per binary (longer
 * trajectories end with EOB_ST_MAXSTEP); larger calls return EOB_E_ARG.
 * Every call looks up the array's device address (cudaGetSymbolAddress, no
 * allocation); the first call on a device also loads the library's device code
 * there and should come before any stream capture.  All calls share the array and it keeps the
 * last call's contents: calls that overlap on the GPU (other streams or
 * threads) race and must be serialised by the caller.  Allocates nothing
 * (no cudaMalloc, cudaFree or allocating library call). */
size_t eob_noalloc_scratch_bytes(void);
int eob_waveform_lnl_noalloc(const double *params, int B, const int *ells, const int *mms, int K, double dt,
                             const double *data, int N, double amp, const eob_options *opt, double *lnl, int *status,
                             cudaStream_t stream);

/* Same pipeline, writing the summed strain instead of the likelihood:
 * strain[B][N] complex (re, im interleaved) = sum_lm h_lm(t_k) on the grid
 * t_k = k dt from each binary's start, zero past its last sample (the
 * mode sum of BBHWaveformTD, eob/seobnrv4phm.py:715-721; "geocenter_td"). */
int eob_waveform_strain(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                        int max_samples, const double *params, const int *order, int B, const int *ells,
                        const int *mms, int K, double dt, int N, const eob_options *opt, double *strain, int *status,
                        cudaStream_t stream);

/* Device pointers into a workspace after eob_waveform_lnl: trajectories
 * traj[b][row][5] = (t [M], r, phi, pr, pphi), nsteps[b] rows each;
 * npts[b] uniform-grid samples of each binary's waveform. */
typedef struct eob_views {
    void *bins;           /* per-binary coefficient records */
    double *traj;
    int *nsteps;
    int *status;
    int *npts;
    long long *row_off;
    double *tin;          /* knot times [M], packed by row_off */
    double *spline_y;     /* [nsubs][rows]: phi, then Re/Im of h_lm e^{i m phi} per mode */
    double *spline_c1, *spline_c2, *spline_c3;
    int row_capacity;     /* max_steps */
    long long rows_capacity;
    int nsubs;
    int *rhs;             /* right-hand sides evaluated per binary (both passes, every attempt) */
} eob_views;
int eob_workspace_views(void *workspace, int max_batch, int max_steps, int max_modes, int max_samples,
                        eob_views *out);

/* Host copy of the pipeline's counters after a run (synchronises the stream):
 * [1] trajectory rows, [2] synthesis chunks, [4] right-hand-side evaluations
 * spent on binaries, [5] right-hand-side evaluations of all integrator lanes. */
int eob_workspace_counters(void *workspace, int max_batch, int max_steps, int max_modes, int max_samples,
                           unsigned long long *out8, cudaStream_t stream);

/* ---------------------------------------------------------------------------
 * Reference-shaped entry points (src/eob.pyx, src/dopr853.pyx, src/tdinterp.pyx)
 */

/* src/eob.pyx:79 evaluate_Ham_align_AD -> src/EOB.cu:127 evaluate_Ham_align_AD_wrap */
int eob_evaluate_ham(double *out, const double *r, const double *phi, const double *pr, const double *pphi,
                     const double *m_1, const double *m_2, const double *chi_1, const double *chi_2, double K,
                     double d5, double dSO, double dSS, int numSys, cudaStream_t stream);
/* src/eob.pyx:61 grad_Ham_align_AD -> src/EOB.cu:242 grad_Ham_align_AD_wrap */
int eob_grad_ham(const double *arg, double *grad_out, const double *additionalArgs, int numSys, cudaStream_t stream);
/* src/eob.pyx:70 hessian_Ham_align_AD -> src/EOB.cu:391 hessian_Ham_align_AD_wrap (exact d2H/dr2) */
int eob_hessian_ham(const double *arg, double *hessian_out, const double *additionalArgs, int numSys,
                    cudaStream_t stream);
/* src/eob.pyx:94 IC_cons -> src/EOB.cu:451 IC_cons_wrap */
int eob_ic_cons(double *res, const double *x, double *args, const double *additionalArgs, double *grad_out,
                int numSys, cudaStream_t stream);
/* src/eob.pyx:51 root_find_all -> src/EOB.cu:3033 root_find_all_wrap (n = 2, num_args = 4) */
int eob_root_find_all(double *xOut, const double *x0In, const double *argsIn, const double *additionalArgsIn,
                      int max_iter, double err, int numBinAll, int n, int num_args, int num_add_args,
                      cudaStream_t stream);

/* SEOBNRv5 class (src/eob.pyx:106-255, src/EOB.cu:3343-3496) as a context:
 * per-binary coefficient tables live in caller memory of
 * eob_ctx_bytes(numSys) bytes. */
size_t eob_ctx_bytes(int numSys);
/* src/eob.pyx:118 update_information -> src/EOB.cu:3355; prefixes (re, im) interleaved, [35][numSys] */
int eob_ctx_update_information(void *ctx, const double *m1, const double *m2, const double *eta, const double *tplspin,
                               const double *chi_S, const double *chi_A, int use_hm, int numSys,
                               cudaStream_t stream);
/* src/eob.pyx:158 ODE_Ham_align_AD -> src/EOB.cu:3486 */
int eob_ctx_ode(const void *ctx, const double *x, const double *arg, double *k, const double *additionalArgs,
                int numSys, const int *hCoeffs_index, cudaStream_t stream);
/* src/eob.pyx:147 RR_force -> src/EOB.cu:3385 */
int eob_ctx_rr_force(const void *ctx, double *force_out, double *grad_out, const double *args,
                     const double *additionalArgs, int numSys, const int *hCoeffs_index, cudaStream_t stream);
/* src/eob.pyx:169 root_find_scalar_all -> src/EOB.cu:3398 (ic_mode as eob_options) */
int eob_ctx_root_find_scalar_all(const void *ctx, double *pr_res, const double *start_bounds, const double *argsIn,
                                 const double *additionalArgsIn, int max_iter, double err, int numBinAll,
                                 int num_args, int num_add_args, int ic_mode, cudaStream_t stream);
/* src/eob.pyx:203 EOBGetSpinFactorizedWaveform -> src/EOB.cu:3423; out and newtonian_prefix complex interleaved */
int eob_ctx_waveform(const void *ctx, double *out, const double *r, const double *phi, const double *pr,
                     const double *pphi, const double *v, const double *Hreal, const double *eta,
                     const double *vPhiInput, int l, int m, const double *newtonian_prefix, double h22_calib,
                     int numSys, int traj_length, const int *hCoeffs_index, cudaStream_t stream);

/* src/eob.pyx:178 SEOBNRv5Class.compute_hlms -> src/EOB.cu:3147-3322.  The
 * reference's kernel computes the modes but never stores them (its store is
 * commented out, :3319) and indexes its per-block shared arrays by trajectory
 * row; this is the function it was written to be:
 * hlms[(b num_modes + k) num_steps_max + i] (complex128) = h_lm, l = ell_arr[k],
 * m = mm_arr[k] (device int arrays), of binary b at row i < num_steps[b] of
 * r/phi/pr/L_arr [num_bin_all][num_steps_max], with H and its gradients at the
 * state and at p_r = 0 from additionalArgs [num_add_args >= 10][num_bin_all]
 * (rows m1, m2, chi1, chi2, omega0, K, d5, dSO, dSS, h22_calib), nu from m1/m2_arr,
 * v = omega^(1/3), the vPhi input 1/(omega_c^2 r^3), ctx's coefficient tables
 * and newtonian_prefixes [num_modes][num_bin_all] (complex128: the array
 * update_information was given).  chi1/chi2_arr are accepted for the argument
 * order and not read (additionalArgs carries the spins). */
int eob_ctx_compute_hlms(const void *ctx, double *hlms, const double *r_arr, const double *phi_arr,
                         const double *pr_arr, const double *L_arr, const double *m1_arr, const double *m2_arr,
                         const double *chi1_arr, const double *chi2_arr, const int *num_steps, int num_steps_max,
                         const int *ell_arr, const int *mm_arr, int num_modes, int num_bin_all,
                         const double *additionalArgs, int num_add_args, const double *newtonian_prefixes,
                         cudaStream_t stream);

/* src/dopr853.pyx:67 dormandPrinceSteps -> src/DOPR853.cu:357 (one fused launch) */
int eob_dopr853_steps(const double *x, double *xCurrent, const double *solOld, const double *h, double *arg,
                      const double *additionalArgs, double *k1, double *k2, double *k3, double *k4, double *k5,
                      double *k6, double *k7, double *k8, double *k9, double *k10, double *ak_term_buffer, int nargs,
                      int numEq, int num_add_args, const void *ctx, const int *hCoeffs_index, cudaStream_t stream);
/* src/dopr853.pyx:139 error -> src/DOPR853.cu:620 */
int eob_dopr853_error(double *err, const double *solOld, double *solNew, const double *h, const double *k1,
                      const double *k2, const double *k3, const double *k6, const double *k7, const double *k8,
                      const double *k9, const double *k10, int numEq, int nargs, cudaStream_t stream);
/* src/dopr853.pyx:187 controllerSuccess -> src/DOPR853.cu:764 (bool arrays as bytes) */
int eob_dopr853_controller(unsigned char *flagSuccess, const double *err, double *errOld,
                           unsigned char *previousReject, double *h, const double *x, int numEq, int nargs,
                           cudaStream_t stream);

/* src/tdinterp.pyx:21 interpolate_TD_wrap -> src/interpolate.cu:269; c1/c2/c3 overwrite
 * upper_diag/diag/lower_diag as in the reference */
int eob_interpolate_td(const double *t_arr, const double *propArrays, double *B, double *upper_diag, double *diag,
                       double *lower_diag, const int *lengths, int numBinAll, int nsubs, cudaStream_t stream);

/* src/tdinterp.pyx:60 TDInterp_wrap2 -> src/interpolate.cu:441-549 (TD2): for binary b and sample
 * i < lengths[b], t = dataTime[i], j = inds[max_length * b + i], x = t - ts[b * old_length + j];
 * series s of binary b at propArrays/c1/c2/c3[b * (2K + 1) * old_length + s * old_lengths[b] + j]
 * (s < K: Re h_k, K..2K-1: Im h_k, 2K: orbital phase); templateChannels[b * data_length + i]
 * (complex, interleaved) = sum_k (Re + i Im) exp(-i m_k phi).  K <= 20.  Knot indices are
 * clamped into the binary's rows. */
int eob_tdinterp2(double *templateChannels, const double *dataTime, const double *ts, const double *propArrays,
                  const double *c1, const double *c2, const double *c3, int old_length, const int *old_lengths,
                  int data_length, int numBinAll, int numModes, const int *ls, const int *ms, const int *inds,
                  const int *lengths, int max_length, cudaStream_t stream);
/* src/tdinterp.pyx:40 TDInterp_wrap -> src/interpolate.cu:323-438 (TD): per-binary arrays given
 * as HOST arrays of device addresses (templateChannels_ptrs, tsAll, propArraysAll, c1All, c2All,
 * c3All, inds_ptrs) and HOST metadata (old_lengths, inds_start, ind_lengths), as the reference's
 * host loop reads them; ls, ms and dataTime on the device.  Binary b writes
 * templateChannels_b[data_length + i] for i < ind_lengths[b] from dataTime[inds_start[b] + i]. */
int eob_tdinterp(const long long *templateChannels_ptrs, const double *dataTime, const long long *tsAll,
                 const long long *propArraysAll, const long long *c1All, const long long *c2All,
                 const long long *c3All, const int *old_lengths, int data_length, int numBinAll, int numModes,
                 const int *ls, const int *ms, const long long *inds_ptrs, const int *inds_start,
                 const int *ind_lengths, cudaStream_t stream);
/* src/tdinterp.pyx:78 all_in_one_likelihood -> src/interpolate.cu:553-627: for frequency block
 * q of 1024 bins, binary b and channel c, temp_sum[(q * num_bin_all + b) * nchannels + c]
 * (complex, imaginary part 0) = sum_i |d_ci - (F+_cb h+_bi + Fx_cb hx_bi) exp(-2 pi i df i tau_cb)|^2
 * / psd_ci, with data[c * data_length + i], psd[c * data_length + i], hp_fd/hc_fd[b * data_length
 * + i] (complex), Fplus/Fcross/time_shift[c * num_bin_all + b].  The caller's lnL is
 * -2 df sum over blocks and channels (eob/seobnrv4phm.py:806-809). */
int eob_all_in_one_likelihood(double *temp_sum, const double *hp_fd, const double *hc_fd, const double *data,
                              const double *psd, const double *Fplus, const double *Fcross, const double *time_shift,
                              double df, int num_bin_all, int nchannels, int data_length, cudaStream_t stream);

/* ---------------------------------------------------------------------------
 * Frequency-domain likelihood (BBHWaveformTD.get_ll, eob/seobnrv4phm.py:772-823)
 */

/* Detector response, eob/seobnrv4phm.py:597-634 (get_detector_information):
 * per binary b (ra, dec, psi [rad], geocent_time [GPS s]) and detector c
 * (detector_tensors[c][3][3], vertices[c][3] in m, Earth-fixed), the antenna
 * patterns Fplus/Fcross[c * B + b] and the delay from the geocenter
 * time_shift[c * B + b] [s].  The Greenwich mean sidereal time (the
 * reference calls lal through bilby) is the IAU 1982 expression of the GPS
 * time with GPS - UTC leap seconds to 2017 and UT1 = UTC.  Device arrays. */
int eob_detector_response(const double *ra, const double *dec, const double *psi, const double *geocent_time,
                          const double *detector_tensors, const double *vertices, int B, int nch, double *Fplus,
                          double *Fcross, double *time_shift, cudaStream_t stream);
/* The likelihood of eob/seobnrv4phm.py:736-744 + 778-817 from H[b][k] (complex,
 * interleaved), the complex FFT over N (even) samples of each binary's summed
 * strain h_+ + i h_x: the two real FFTs of the reference are recovered as
 * h~_+(f) = (H(f) + conj H(N-f)) / 2 and h~_x(f) = (H(f) - conj H(N-f)) / 2i for
 * the N/2 + 1 bins f = k df, set to zero below start_ind (bilby_start_ind);
 * lnl[b] = -1/2 4 df sum_c sum_f |d_c(f) - (F+ h~_+ + Fx h~_x) e^{-2 pi i f tau}|^2
 * / psd_c(f) with data[c][N/2 + 1] (complex), psd[c][N/2 + 1], Fplus, Fcross,
 * time_shift[c * B + b] (the all_in_one_likelihood partials,
 * src/interpolate.cu:551-627, summed).  nch <= 8.  scratch: device memory of
 * eob_fd_lnl_scratch_bytes(B, N) bytes (block partials and 1/psd). */
size_t eob_fd_lnl_scratch_bytes(int B, int N);
int eob_fd_lnl_from_fft(const double *H, int N, int start_ind, const double *data, const double *psd,
                        const double *Fplus, const double *Fcross, const double *time_shift, double df, int B, int nch,
                        void *scratch, size_t scratch_bytes, double *lnl, cudaStream_t stream);

/* ---------------------------------------------------------------------------
 * Measurement and test hooks.  Not part of the waveform path and without a
 * counterpart in the reference: they exist so that the benchmark can measure
 * its roofline denominator on the device it runs on and the tests can check
 * the hot path's arithmetic and its bounded waits.
 */

/* FP64 issue-rate probe: blocks x threads lanes each run iters x 8 independent
 * DFMA chains; out[blocks * threads] receives the chain sums.  Timing it gives
 * the device's FP64 peak used as the integrator's roofline. */
int eob_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t stream);
/* Accuracy probe of the hot path's math: for each of the n device doubles x,
 * out[10 i + 0..9] = the hot path's reciprocal, the device division 1/x, the
 * hot path's x^(-1/3), the device rcbrt, the hot path's log, the device log,
 * the hot path's 1/sqrt(x), the step controller's x^(-1/8), the m factors'
 * e^(-y) - 1 and the device expm1(-y) at y = min(x, 600); out: device, 10 n
 * doubles. */
int eob_math_probe(const double *x, int n, double *out, cudaStream_t stream);
/* The integrator's multi-warp group barrier with its wait limited to limit_ns
 * (1e3..2e9; the integrator itself uses 2 s).  Blocks of 256 threads hold
 * groups of group_warps (2 or 4) warps that pass `rounds` barriers (at most
 * 4096), exchanging values through shared memory; in every group g < 32 with
 * bit g of skip_mask set, warp skip_warp of the group leaves at round
 * skip_round without arriving, so the group's other warps see their wait run
 * out.  out: device int[blocks * 8 * 4], per warp (ok, barriers passed, values
 * read back wrong, microseconds spent in the wait that ran out). */
int eob_sync_expiry_hook(int group_warps, int rounds, unsigned skip_mask, int skip_round, int skip_warp,
                         long long limit_ns, int *out, int blocks, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif
