// Scratch of the allocation-free Mie/phase entry point (clr_mie_phase_noalloc).
//
// The Mie coefficient kernel needs an a_n/b_n buffer of CLR_MIE_MAX_ORDER complex pairs per bin and
// the phase pdf kernel an [n][n_theta] buffer. Here they are file-scope __device__ arrays sized for
// CLR_NOALLOC_MAX_BINS bins and CLR_NOALLOC_MAX_THETA angles (about 3 MB per device, part of the
// module image), so the entry point never calls an allocator. Their addresses are resolved with
// cudaGetSymbolAddress once per device, with that device current, and cached.
#include <mutex>
#include "kernels.h"

namespace clr {
namespace {

__device__ __align__(256) double na_ab[CLR_NOALLOC_MAX_BINS * CLR_MIE_MAX_ORDER * 4];
__device__ __align__(256) double na_pdf[CLR_NOALLOC_MAX_BINS * CLR_NOALLOC_MAX_THETA];
__device__ __align__(256) float na_cdf_f[CLR_NOALLOC_MAX_BINS * CLR_NOALLOC_MAX_THETA];
__device__ __align__(256) float na_theta_f[CLR_NOALLOC_MAX_THETA];
__device__ __align__(256) double na_side[4 * CLR_NOALLOC_MAX_BINS];  // x, qabs, qback, albedo
__device__ __align__(256) int na_nstop[CLR_NOALLOC_MAX_BINS];
__device__ __align__(256) int na_err[1];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
bool g_ready[kMaxDevices] = {};
NoallocScratch g_scratch[kMaxDevices];

template <class T>
cudaError_t symbol(T& sym, void** out) {
    return cudaGetSymbolAddress(out, sym);
}

}  // namespace

cudaError_t noalloc_scratch(int device, NoallocScratch* out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ready[device]) {
        int prev = 0;
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return e;
        if ((e = cudaSetDevice(device)) != cudaSuccess) return e;
        NoallocScratch s;
        void* p = nullptr;
        if ((e = symbol(na_ab, &p)) == cudaSuccess) s.ab = static_cast<double*>(p);
        if (e == cudaSuccess && (e = symbol(na_pdf, &p)) == cudaSuccess) s.pdf = static_cast<double*>(p);
        if (e == cudaSuccess && (e = symbol(na_cdf_f, &p)) == cudaSuccess) s.cdf_f = static_cast<float*>(p);
        if (e == cudaSuccess && (e = symbol(na_theta_f, &p)) == cudaSuccess) s.theta_f = static_cast<float*>(p);
        if (e == cudaSuccess && (e = symbol(na_side, &p)) == cudaSuccess) {
            double* side = static_cast<double*>(p);
            s.x = side;
            s.qabs = side + CLR_NOALLOC_MAX_BINS;
            s.qback = side + 2 * CLR_NOALLOC_MAX_BINS;
            s.albedo = side + 3 * CLR_NOALLOC_MAX_BINS;
        }
        if (e == cudaSuccess && (e = symbol(na_nstop, &p)) == cudaSuccess) s.nstop = static_cast<int*>(p);
        if (e == cudaSuccess && (e = symbol(na_err, &p)) == cudaSuccess) s.err = static_cast<int*>(p);
        const cudaError_t e2 = cudaSetDevice(prev);
        if (e != cudaSuccess) return e;
        if (e2 != cudaSuccess) return e2;
        g_scratch[device] = s;
        g_ready[device] = true;
    }
    *out = g_scratch[device];
    return cudaSuccess;
}

}  // namespace clr
