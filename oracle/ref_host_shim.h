/* Host-compilation shim for the reference's embedded CUDA source.
 *
 * Test infrastructure only. The reference keeps its whole photon-transport
 * device code in one string, `CUDA_SRC` (CLARITAS/CLARITAS.py:1119-5212),
 * JIT-compiled by CuPy NVRTC (CLARITAS/CLARITAS.py:6000). oracle/ref_extract.py
 * writes that string, unmodified, to oracle/_ref/claritas_cuda_src.inc (never
 * committed). This header supplies the few CUDA-only names that source uses so
 * g++ can build it as ordinary host C++:
 *   - `__device__` / `__global__` qualifiers become empty;
 *   - thread/block indices become thread-local variables the driver sets per ray;
 *   - atomics become GCC __atomic builtins (correct under OpenMP);
 *   - bit-casts go through memcpy; rsqrtf is 1/sqrtf; erfinv comes from
 *     oracle_math.h.
 * Every other math call (sinf, logf, erfc, cbrt, ...) resolves to glibc libm,
 * so results are the reference's own arithmetic evaluated on the host.
 */
#ifndef CLARITAS_REF_HOST_SHIM_H
#define CLARITAS_REF_HOST_SHIM_H

#include <math.h>
#include <cmath>
#include <cstring>
#include <cstdint>
#include "oracle_math.h"

#define __device__
#define __global__
#define __host__
#define __forceinline__ inline

struct ref_dim3 { unsigned int x, y, z; };
extern thread_local ref_dim3 threadIdx;
extern thread_local ref_dim3 blockIdx;
extern thread_local ref_dim3 blockDim;

static inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
static inline double erfinv(double y) { return oracle_erfinv(y); }

static inline double __longlong_as_double(long long v) { double d; std::memcpy(&d, &v, sizeof d); return d; }
static inline float __int_as_float(int v) { float f; std::memcpy(&f, &v, sizeof f); return f; }
static inline unsigned int __float_as_uint(float f) { unsigned int u; std::memcpy(&u, &f, sizeof u); return u; }

static inline int atomicAdd(int* p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
static inline unsigned int atomicAdd(unsigned int* p, unsigned int v) { return __atomic_fetch_add(p, v, __ATOMIC_RELAXED); }
static inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v) {
    return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
}
static inline float atomicAdd(float* p, float v) {
    float old;
    __atomic_load(p, &old, __ATOMIC_RELAXED);
    float desired;
    do { desired = old + v; } while (!__atomic_compare_exchange(p, &old, &desired, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
    return old;
}
static inline double atomicAdd(double* p, double v) {
    double old;
    __atomic_load(p, &old, __ATOMIC_RELAXED);
    double desired;
    do { desired = old + v; } while (!__atomic_compare_exchange(p, &old, &desired, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
    return old;
}
static inline int atomicExch(int* p, int v) { return __atomic_exchange_n(p, v, __ATOMIC_RELAXED); }

using std::isfinite;
using std::isnan;
using std::isinf;

#endif
