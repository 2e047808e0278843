// FP64 issue-rate probe used by the benchmark to measure the denominator of
// the integrator's roofline on the device it runs on.
#include "eob_device.cuh"

namespace {
__global__ void k_fp64_probe(double *out, int iters)
{
    double a0 = threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const double x = 1.0000001, y = 1e-9;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, x, y); a1 = fma(a1, x, y); a2 = fma(a2, x, y); a3 = fma(a3, x, y);
        a4 = fma(a4, x, y); a5 = fma(a5, x, y); a6 = fma(a6, x, y); a7 = fma(a7, x, y);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}
}  // namespace

extern "C" int eob_fp64_probe(double *out, int blocks, int threads, int iters, cudaStream_t stream)
{
    if (!out || blocks < 1 || threads < 1 || threads > 1024 || iters < 1) return EOB_E_ARG;
    k_fp64_probe<<<blocks, threads, 0, stream>>>(out, iters);
    return cudaGetLastError() == cudaSuccess ? EOB_OK : EOB_E_CUDA;
}
