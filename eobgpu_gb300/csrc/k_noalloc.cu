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

constexpr int kMaxDevices = 64;
void *g_noalloc_addr[kMaxDevices] = {nullptr};

}  // namespace

extern "C" size_t eob_noalloc_scratch_bytes(void) { return kNaBytes; }

extern "C" int eob_waveform_lnl_noalloc(const double *params, int B, const int *ells, const int *mms, int K, double dt,
                                        const double *data, int N, double amp, const eob_options *opt, double *lnl,
                                        int *status, cudaStream_t stream)
{
    if (B < 1 || B > kNaBatch || K < 1 || K > kNaModes || N < 1 || N > kNaSamples) return EOB_E_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return EOB_E_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return EOB_E_ARG;
    if (!g_noalloc_addr[dev]) {
        // first call on this device: the device address of the scratch array
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return EOB_E_CUDA;
        g_noalloc_addr[dev] = p;
    }
    // trajectory capacity is bounded by kNaSteps rows per binary
    eob_options o;
    if (opt) o = *opt; else eob_options_default(&o);
    return eob_waveform_lnl(g_noalloc_addr[dev], kNaBytes, kNaBatch, kNaSteps, kNaModes, kNaSamples, params, nullptr,
                            B, ells, mms, K, dt, data, N, amp, &o, lnl, status, stream);
}
