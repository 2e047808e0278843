// extern "C" entry points of libeobgb300.so: the fused waveform + likelihood
// path over a caller-provided workspace.  Declarations and reference
// citations: include/eobgb300.h.
#include <cstring>
#include "eob_device.cuh"

using namespace eob;

extern "C" {

void eob_options_default(eob_options *o)
{
    o->rtol = 1e-12;
    o->atol = 1e-12;
    o->h_init = 0.01;
    o->step_back = 10.0;
    o->fine_step = 0.05;
    o->ic_mode = 0;
    o->precision = 0;
    o->block = 0;
    o->grid = 0;
    o->max_tries = 0;
    o->lanes_per_binary = 0;
    o->spline_tile = 0;
    o->head_quads = -1;
    o->imr = 0;
}

size_t eob_workspace_bytes(int max_batch, int max_steps, int max_modes, int max_samples)
{
    if (max_batch < 1 || max_steps < 4 || max_modes < 1 || max_modes > kMaxModes || max_samples < 1) return 0;
    return ws_layout(max_batch, max_steps, max_modes, max_samples).total;
}

size_t eob_workspace_bytes_imr(int max_batch, int max_steps, int max_modes, int max_samples)
{
    if (max_batch < 1 || max_steps < 4 || max_modes < 1 || max_modes > kMaxModes || max_samples < 1) return 0;
    return ws_layout(max_batch, max_steps, max_modes, max_samples, 1).total;
}

// the workspace's layout: with the merger-ringdown section when it is large enough for one
static bool dims_ok(size_t workspace_bytes, int max_batch, int max_steps, int max_modes, int max_samples, WsLayout *L)
{
    if (!(max_batch >= 1 && max_steps >= 4 && max_modes >= 1 && max_modes <= kMaxModes && max_samples >= 1))
        return false;
    *L = ws_layout(max_batch, max_steps, max_modes, max_samples, 1);
    if (workspace_bytes >= L->total) return true;
    *L = ws_layout(max_batch, max_steps, max_modes, max_samples, 0);
    return workspace_bytes >= L->total;
}

static bool modes_ok(const int *ells, const int *mms, int K, int max_modes)
{
    if (!ells || !mms || K < 1 || K > max_modes) return false;
    for (int j = 0; j < K; ++j)
        if (ells[j] < 2 || ells[j] > kLMax || mms[j] < 1 || mms[j] > ells[j]) return false;
    return true;
}

int eob_prepare_stages(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                       int max_samples, const double *params, const int *order, int B, const int *ells, const int *mms,
                       int K, double dt, const eob_options *opt, int stages, cudaStream_t stream)
{
    WsLayout L;
    if (!workspace || !params || !dims_ok(workspace_bytes, max_batch, max_steps, max_modes, max_samples, &L))
        return EOB_E_ARG;
    if (B < 1 || B > max_batch || !(dt > 0.0) || !modes_ok(ells, mms, K, max_modes)) return EOB_E_ARG;
    RunArgs a;
    std::memset(&a, 0, sizeof(a));
    a.params = params;
    a.order = order;
    a.B = B;
    a.K = K;
    for (int j = 0; j < K; ++j) { a.ells[j] = ells[j]; a.mms[j] = mms[j]; }
    a.dt = dt;
    if (opt) a.opt = *opt; else eob_options_default(&a.opt);
    if (a.opt.imr && !L.imr) return EOB_E_ARG;  // the workspace has no merger-ringdown section
    const Ws w = ws_views(workspace, L);
    cudaError_t e = cudaSuccess;
    if (stages & 1) e = launch_setup(w, a, stream);
    if (e == cudaSuccess && (stages & 2)) e = launch_integrate(w, a, stream);
    if (e == cudaSuccess && (stages & 4)) e = launch_prepare_post(w, a, stream);
    if (e == cudaSuccess && (stages & 4)) e = launch_imr(w, a, stream);
    return e == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

int eob_prepare(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes, int max_samples,
                const double *params, const int *order, int B, const int *ells, const int *mms, int K, double dt,
                const eob_options *opt, int *status, cudaStream_t stream)
{
    (void)status;
    return eob_prepare_stages(workspace, workspace_bytes, max_batch, max_steps, max_modes, max_samples, params, order,
                              B, ells, mms, K, dt, opt, 7, stream);
}

static int synth(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes, int max_samples,
                 int B, const int *mms, int K, double dt, const double *data, int N, double amp, double *lnl,
                 int mode, double *out, int *status, const eob_options *opt, cudaStream_t stream)
{
    WsLayout L;
    if (!workspace || !dims_ok(workspace_bytes, max_batch, max_steps, max_modes, max_samples, &L)) return EOB_E_ARG;
    if (B < 1 || B > max_batch || N < 1 || N > max_samples || !(dt > 0.0) || !mms || K < 1 || K > max_modes)
        return EOB_E_ARG;
    RunArgs a;
    std::memset(&a, 0, sizeof(a));
    a.B = B;
    a.K = K;
    for (int j = 0; j < K; ++j) a.mms[j] = mms[j];
    a.dt = dt;
    a.data = data;
    a.N = N;
    a.amp = amp;
    a.lnl = lnl;
    a.status_out = status;
    if (opt) a.opt = *opt; else eob_options_default(&a.opt);
    const Ws w = ws_views(workspace, L);
    const cudaError_t e = launch_synth(w, a, mode, out, stream);
    return e == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

int eob_synth_lnl(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                  int max_samples, int B, const int *mms, int K, double dt, const double *data, int N, double amp,
                  const eob_options *opt, double *lnl, int *status, cudaStream_t stream)
{
    if (!data || !lnl) return EOB_E_ARG;
    return synth(workspace, workspace_bytes, max_batch, max_steps, max_modes, max_samples, B, mms, K, dt, data, N, amp,
                 lnl, 0, nullptr, status, opt, stream);
}

int eob_synth_strain(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                     int max_samples, int B, const int *mms, int K, double dt, int N, int per_mode, double *out,
                     int *status, cudaStream_t stream)
{
    if (!out) return EOB_E_ARG;
    return synth(workspace, workspace_bytes, max_batch, max_steps, max_modes, max_samples, B, mms, K, dt, nullptr, N,
                 1.0, nullptr, per_mode ? 2 : 1, out, status, nullptr, stream);
}

int eob_waveform_lnl(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                     int max_samples, const double *params, const int *order, int B, const int *ells,
                     const int *mms, int K, double dt, const double *data, int N, double amp,
                     const eob_options *opt, double *lnl, int *status, cudaStream_t stream)
{
    if (!data || !lnl || N < 1 || N > max_samples) return EOB_E_ARG;
    int rc = eob_prepare(workspace, workspace_bytes, max_batch, max_steps, max_modes, max_samples, params, order, B,
                         ells, mms, K, dt, opt, nullptr, stream);
    if (rc != EOB_OK) return rc;
    return eob_synth_lnl(workspace, workspace_bytes, max_batch, max_steps, max_modes, max_samples, B, mms, K, dt, data,
                         N, amp, opt, lnl, status, stream);
}

int eob_waveform_strain(void *workspace, size_t workspace_bytes, int max_batch, int max_steps, int max_modes,
                        int max_samples, const double *params, const int *order, int B, const int *ells,
                        const int *mms, int K, double dt, int N, const eob_options *opt, double *strain, int *status,
                        cudaStream_t stream)
{
    if (!strain || N < 1 || N > max_samples) return EOB_E_ARG;
    int rc = eob_prepare(workspace, workspace_bytes, max_batch, max_steps, max_modes, max_samples, params, order, B,
                         ells, mms, K, dt, opt, nullptr, stream);
    if (rc != EOB_OK) return rc;
    return synth(workspace, workspace_bytes, max_batch, max_steps, max_modes, max_samples, B, mms, K, dt, nullptr, N,
                 1.0, nullptr, 1, strain, status, opt, stream);
}

int eob_workspace_counters(void *workspace, int max_batch, int max_steps, int max_modes, int max_samples,
                           unsigned long long *out8, cudaStream_t stream)
{
    if (!workspace || !out8) return EOB_E_ARG;
    const WsLayout L = ws_layout(max_batch, max_steps, max_modes, max_samples);
    const Ws w = ws_views(workspace, L);
    cudaError_t e = cudaMemcpyAsync(out8, w.queue, sizeof(unsigned long long) * 8, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}

int eob_workspace_views(void *workspace, int max_batch, int max_steps, int max_modes, int max_samples,
                        eob_views *out)
{
    if (!workspace || !out) return EOB_E_ARG;
    const WsLayout L = ws_layout(max_batch, max_steps, max_modes, max_samples);
    if (L.total == 0) return EOB_E_ARG;
    const Ws w = ws_views(workspace, L);
    out->bins = w.bins;
    out->traj = w.traj;
    out->nsteps = w.nsteps;
    out->status = w.status;
    out->npts = w.npts;
    out->row_off = w.row_off;
    out->tin = w.tin;
    out->spline_y = w.ys;
    out->spline_c1 = w.cA;
    out->spline_c2 = w.cB;
    out->spline_c3 = w.cC;
    out->row_capacity = max_steps;
    out->rows_capacity = (long long)max_batch * (long long)max_steps;
    out->nsubs = L.nsubs;
    out->rhs = w.rhs;
    return EOB_OK;
}

}  // extern "C"
