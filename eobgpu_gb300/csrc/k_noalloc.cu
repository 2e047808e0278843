// Fused waveform + likelihood for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc or any allocating
// routine: code running inside another framework's memory pool or a
// restricted plugin host, or processes that must not touch the allocator
// while other work is in flight.  For them this file provides one entry point
// whose scratch space (the workspace of eob_waveform_lnl) is a file-scope
// __device__ array of fixed size, created when the library's device code is
// loaded.  Every GPU that loads the library holds this array until the
// process exits.
#include "eob_device.cuh"

namespace {

constexpr int kNaBatch = 16;      // binaries per call
constexpr int kNaSteps = 4096;    // trajectory rows per binary
constexpr int kNaModes = 1;       // modes per call
constexpr int kNaSamples = 8192;  // samples of the data
constexpr size_t kNaBytes = eob::ws_layout(kNaBatch, kNaSteps, kNaModes, kNaSamples).total;

// The scratch of every call.  Host code must not use this name as a device
// address (on the host it is a stand-in); the address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

}  // namespace

extern "C" size_t eob_noalloc_scratch_bytes(void) { return kNaBytes; }

extern "C" int eob_waveform_lnl_noalloc(const double *params, int B, const int *ells, const int *mms, int K, double dt,
                                        const double *data, int N, double amp, const eob_options *opt, double *lnl,
                                        int *status, cudaStream_t stream)
{
    if (B < 1 || B > kNaBatch || K < 1 || K > kNaModes || N < 1 || N > kNaSamples) return EOB_E_ARG;
    // The array's device address on the current device, looked up on every
    // call: it is not a stream operation and costs far less than the launch,
    // and a cached value would go stale if the context were reset (the
    // module is then loaded again, possibly elsewhere).  The first lookup on a
    // device loads the library's device code there, so that first call should
    // come before any stream capture.
    void *scratch = nullptr;
    if (cudaGetSymbolAddress(&scratch, g_noalloc_scratch) != cudaSuccess || !scratch) return EOB_E_CUDA;
    // trajectory capacity is bounded by kNaSteps rows per binary
    eob_options o;
    if (opt) o = *opt; else eob_options_default(&o);
    return eob_waveform_lnl(scratch, kNaBytes, kNaBatch, kNaSteps, kNaModes, kNaSamples, params, nullptr, B, ells,
                            mms, K, dt, data, N, amp, &o, lnl, status, stream);
}
