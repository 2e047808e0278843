/* Force-included header that lets the reference's CUDA sources
 * (src/EOB.cu, src/DOPR853.cu, lines 1-308 of src/interpolate.cu) compile as
 * plain host C++ with g++.  It supplies the handful of CUDA runtime names
 * those files use outside their __CUDACC__ branches.
 *
 * Test infrastructure only: the resulting library (oracle/_ref/) is the
 * reference's own CPU path, used to pin the oracle and to generate the golden
 * fixtures.  Nothing in the product links it.
 */
#ifndef EOBGB300_REF_SHIM_H
#define EOBGB300_REF_SHIM_H
#include <math.h>
#include <stdlib.h>
#include <cmath>

#define CUDART_INF (__builtin_inf())
#define CUDART_NAN (__builtin_nan(""))
#define __noinline__

static inline double sinpi(double x) { return sin(M_PI * x); }
static inline double cospi(double x) { return cos(M_PI * x); }

typedef int cudaError_t;
/* zero-filled so that fields the reference leaves unset (equal-mass branch of
 * its coefficient routine) read as 0 rather than as garbage */
static inline int cudaMalloc(void *p, size_t n) { *(void **)p = calloc(1, n); return 0; }
static inline int cudaFree(void *p) { free(p); return 0; }
static inline int cudaGetLastError() { return 0; }
static inline int cudaDeviceSynchronize() { return 0; }
#define gpuErrchk(x) (void)(x)

#endif
