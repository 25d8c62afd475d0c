// Surrogate network of the detector signals, trained and evaluated on the GPU (no reference
// counterpart: the reference answers every scenario query with a full Monte Carlo run).
//
// Network: 6 -> 256 -> 256 -> 256 -> 256 -> 3, SiLU after each hidden layer, BF16 weights and
// activations, FP32 accumulation, FP32 master weights with Adam. The three 256x256 layers run on the
// 5th-generation tensor cores: one GEMM kernel computes C[M][256] = A[M][K] . B[256][K]^T with both
// operands K-major BF16, staged through shared memory in the canonical no-swizzle core-matrix layout
// and multiplied by tcgen05.mma (M=128, N=256, K=16 per instruction) into a TMEM accumulator, which
// the epilogue reads back with tcgen05.ld. The same kernel serves the forward layers (bias + SiLU
// epilogue), the backward-data products (SiLU-derivative epilogue) and the weight gradients (split-K
// over the batch, FP32 atomics). The thin first (6 -> 256) and last (256 -> 3) layers, the loss, the
// bias gradients and the Adam update are CUDA-core kernels.
#include <cstdint>
#include <cstring>
#include <cmath>
#include <random>
#include <string>
#include <vector>
#include <algorithm>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include "claritas_gb.h"

namespace mlpk {

typedef __nv_bfloat16 bf16;

constexpr int kIn = CLR_MLP_INPUTS, kHid = CLR_MLP_WIDTH, kOut = CLR_MLP_OUTPUTS;
// flat parameter layout: W1 [256][6], b1, W2 [256][256], b2, W3, b3, W4, b4, W5 [3][256], b5
constexpr long long kOffW1 = 0, kOffB1 = kOffW1 + kHid * kIn;
constexpr long long kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid;
constexpr long long kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kHid;
constexpr long long kOffW4 = kOffB3 + kHid, kOffB4 = kOffW4 + kHid * kHid;
constexpr long long kOffW5 = kOffB4 + kHid, kOffB5 = kOffW5 + kOut * kHid;
constexpr long long kParams = kOffB5 + kOut;
static_assert(kParams == CLR_MLP_PARAMS, "parameter count");
// offsets of layer l's weights and biases (l = 1..5)
__host__ __device__ constexpr long long off_w(int l) {
    return l == 1 ? kOffW1 : l == 2 ? kOffW2 : l == 3 ? kOffW3 : l == 4 ? kOffW4 : kOffW5;
}
__host__ __device__ constexpr long long off_b(int l) {
    return l == 1 ? kOffB1 : l == 2 ? kOffB2 : l == 3 ? kOffB3 : l == 4 ? kOffB4 : kOffB5;
}

// ---------------- tcgen05 / mbarrier primitives (inline PTX) ----------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Waits for the phase with the given parity to complete, for at most `limit_ns`. On time-out it
// records error code `code` and returns false (the caller cleans up and leaves).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int* err, int code,
                                          unsigned long long limit_ns = 2000000000ull) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > limit_ns) {
            if (err) atomicCAS(err, 0, code);
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
// D[tmem] (+)= A[smem desc] . B[smem desc]^T, kind::f16 (BF16 inputs per the instruction descriptor)
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on `bar` once every tcgen05 operation this thread issued before has completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// 32 lanes x 32 consecutive 32-bit columns: thread t of the warp receives lane (base lane + t)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of tcgen05 (no swizzle, K-major): start address, leading-dimension
// byte offset (between the two 8x16-byte core matrices along K of one instruction), stride-dimension
// byte offset (between 8-row groups), descriptor version 1 at bits 46-47, layout type 0 (no swizzle).
__host__ __device__ constexpr uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
constexpr int kM = 128, kN = 256, kKC = 64;  // rows per tile, output width, K per shared-memory stage
// Instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                            ((uint32_t)(kM >> 4) << 24);

constexpr int kGemmThreads = 128;               // one warpgroup: warp w reads TMEM lanes 32w..32w+31
constexpr int kStageA = kM * kKC * 2;           // 16 KB
constexpr int kStageB = kN * kKC * 2;           // 32 KB
constexpr int kGemmSmem = 2 * (kStageA + kStageB) + 64;  // two stages, barriers, TMEM address

enum Epi : int { EPI_STORE_F32 = 0, EPI_FWD = 1, EPI_BWD = 2, EPI_ATOMIC_F32 = 3, EPI_INFER = 4 };

struct GemmArgs {
    const bf16* A;           // [M][lda], K contiguous
    long long lda;
    const bf16* B;           // [256][ldb], K contiguous
    long long ldb;
    int M, K, k_split;       // K and k_split multiples of 64; CTA y takes K columns [y*k_split, +k_split)
    const float* bias;       // [256] (EPI_FWD, EPI_INFER)
    const float* zin;        // [M][256] saved pre-activations (EPI_BWD)
    float* out_f32;          // [M][ldo]: result (STORE, ATOMIC) or pre-activation z (FWD)
    long long ldo;
    bf16* out_bf16;          // [M][256]: silu(z) (FWD, INFER) or dz (BWD)
    bf16* out_bf16_t;        // [256][ldt]: transposed copy (FWD, BWD)
    long long ldt;
    int* err;
};

// One K chunk (64 columns) of `rows` rows into the core-matrix layout: element (r, k) at
// (r / 8) * 1024 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2 bytes. Rows at or past `valid` read as zero.
__device__ __forceinline__ void load_chunk(unsigned char* dst, const bf16* src, long long ld, int row0, int rows,
                                           int valid, int k0) {
    for (int q = threadIdx.x; q < rows * 8; q += kGemmThreads) {
        const int r = q >> 3, kc = q & 7;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (row0 + r < valid) v = *reinterpret_cast<const uint4*>(src + (long long)(row0 + r) * ld + k0 + kc * 8);
        *reinterpret_cast<uint4*>(dst + (r >> 3) * 1024 + kc * 128 + (r & 7) * 16) = v;
    }
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
    const float s = 1.0f / (1.0f + expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

template <int EPI>
__global__ void __launch_bounds__(kGemmThreads, 1) umma_gemm_kernel(GemmArgs g) {
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* const stA0 = sm;
    unsigned char* const stB0 = sm + 2 * kStageA;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 2 * (kStageA + kStageB));  // [2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kM;
    const int kb = blockIdx.y * g.k_split;
    const int ke = min(g.K, kb + g.k_split);
    const int nc = ke > kb ? (ke - kb) / kKC : 0;
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot, 256);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;
    int issued = 0;  // chunks whose MMAs were issued
    for (int c = 0; c < nc; ++c) {
        const int s = c & 1;
        // the MMAs of chunk c-2 read this stage: wait for their commit
        if (c >= 2) ok = mbar_wait(&bar[s], ((c - 2) >> 1) & 1, g.err, 1);
        if (!__syncthreads_and(ok)) { ok = false; break; }
        load_chunk(stA0 + s * kStageA, g.A, g.lda, m0, kM, g.M, kb + c * kKC);
        load_chunk(stB0 + s * kStageB, g.B, g.ldb, 0, kN, kN, kb + c * kKC);
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_u32(stA0 + s * kStageA), b0 = smem_u32(stB0 + s * kStageB);
#pragma unroll
            for (int kk = 0; kk < kKC / 16; ++kk)
                mma_bf16(tmem, smem_desc(a0 + kk * 256, 128, 1024), smem_desc(b0 + kk * 256, 128, 1024), kIdesc,
                         (c > 0 || kk > 0) ? 1u : 0u);
            mma_commit(&bar[s]);
        }
        issued = c + 1;
    }
    if (issued > 0) {
        // the last commit covers every MMA issued before it; after a time-out wait once more (bounded)
        // so no MMA still writes the accumulator when it is released
        const bool done = mbar_wait(&bar[(issued - 1) & 1], ((issued - 1) >> 1) & 1, g.err, 2);
        ok = ok && done;
    }
    ok = __syncthreads_and(ok);
    tc_fence_after();
    if (ok && issued > 0) {
        const int m = m0 + 32 * warp + lane;
        const bool row_ok = m < g.M;
        float v[32];
        for (int j0 = 0; j0 < kN; j0 += 32) {
            tmem_ld32(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)j0, v);
            if (!row_ok) continue;
            if constexpr (EPI == EPI_STORE_F32) {
                float4* o = reinterpret_cast<float4*>(g.out_f32 + (long long)m * g.ldo + j0);
#pragma unroll
                for (int i = 0; i < 8; ++i) o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
            } else if constexpr (EPI == EPI_ATOMIC_F32) {
                float* o = g.out_f32 + (long long)m * g.ldo + j0;
#pragma unroll
                for (int i = 0; i < 32; ++i) atomicAdd(o + i, v[i]);
            } else if constexpr (EPI == EPI_FWD || EPI == EPI_INFER) {
                __align__(16) bf16 hb[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float z = v[i] + g.bias[j0 + i];
                    v[i] = z;
                    hb[i] = __float2bfloat16(silu_f(z));
                }
                uint4* ho = reinterpret_cast<uint4*>(g.out_bf16 + (long long)m * kN + j0);
#pragma unroll
                for (int i = 0; i < 4; ++i) ho[i] = reinterpret_cast<const uint4*>(hb)[i];
                if constexpr (EPI == EPI_FWD) {
                    float4* zo = reinterpret_cast<float4*>(g.out_f32 + (long long)m * kN + j0);
#pragma unroll
                    for (int i = 0; i < 8; ++i) zo[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
#pragma unroll
                    for (int i = 0; i < 32; ++i) g.out_bf16_t[(long long)(j0 + i) * g.ldt + m] = hb[i];
                }
            } else {  // EPI_BWD: dz = dh * silu'(z)
                const float4* zi = reinterpret_cast<const float4*>(g.zin + (long long)m * kN + j0);
                __align__(16) bf16 db[32];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float4 z = zi[i];
                    db[4 * i + 0] = __float2bfloat16(v[4 * i + 0] * dsilu_f(z.x));
                    db[4 * i + 1] = __float2bfloat16(v[4 * i + 1] * dsilu_f(z.y));
                    db[4 * i + 2] = __float2bfloat16(v[4 * i + 2] * dsilu_f(z.z));
                    db[4 * i + 3] = __float2bfloat16(v[4 * i + 3] * dsilu_f(z.w));
                }
                uint4* dout = reinterpret_cast<uint4*>(g.out_bf16 + (long long)m * kN + j0);
#pragma unroll
                for (int i = 0; i < 4; ++i) dout[i] = reinterpret_cast<const uint4*>(db)[i];
#pragma unroll
                for (int i = 0; i < 32; ++i) g.out_bf16_t[(long long)(j0 + i) * g.ldt + m] = db[i];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 256);
    }
}

// Opt-in shared memory of every GEMM variant on the current device (called before any launch, outside
// stream capture).
static cudaError_t set_gemm_attributes() {
    const void* fns[] = {(const void*)umma_gemm_kernel<EPI_STORE_F32>, (const void*)umma_gemm_kernel<EPI_FWD>,
                         (const void*)umma_gemm_kernel<EPI_BWD>, (const void*)umma_gemm_kernel<EPI_ATOMIC_F32>,
                         (const void*)umma_gemm_kernel<EPI_INFER>};
    for (const void* f : fns) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <int EPI>
static cudaError_t launch_gemm(const GemmArgs& g, int grid_y, cudaStream_t st) {
    dim3 grid((g.M + kM - 1) / kM, grid_y);
    umma_gemm_kernel<EPI><<<grid, kGemmThreads, kGemmSmem, st>>>(g);
    return cudaGetLastError();
}

// ---------------- CUDA-core kernels: thin layers, loss, gradients, optimizer ----------------
__device__ __forceinline__ float bfr(float x) { return __bfloat162float(__float2bfloat16(x)); }

// rows of the batch by index (training) or copied (inference: idx null)
// (w: per-output loss weights of the rows, nullable)
__global__ void gather_kernel(const float* __restrict__ x, const float* __restrict__ t, const float* __restrict__ w,
                              const int32_t* __restrict__ idx, long long row0, int n, float* xb, float* tb,
                              float* wb) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long src = idx ? (long long)idx[row0 + r] : row0 + r;
#pragma unroll
    for (int i = 0; i < kIn; ++i) xb[r * kIn + i] = bfr(x[src * kIn + i]);
    if (t && tb)
#pragma unroll
        for (int i = 0; i < kOut; ++i) tb[r * kOut + i] = t[src * kOut + i];
    if (w && wb)
#pragma unroll
        for (int i = 0; i < kOut; ++i) wb[r * kOut + i] = w[src * kOut + i];
}

// layer 1 (6 -> 256): one thread per (row, unit)
__global__ void layer1_kernel(const float* __restrict__ xb, int n, const bf16* __restrict__ w1,
                              const float* __restrict__ b1, float* z1, bf16* h1, bf16* h1t, long long ldt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * kHid) return;
    const int r = (int)(t / kHid), j = (int)(t % kHid);
    float z = b1[j];
#pragma unroll
    for (int i = 0; i < kIn; ++i) z = fmaf(xb[r * kIn + i], __bfloat162float(w1[j * kIn + i]), z);
    const bf16 h = __float2bfloat16(silu_f(z));
    h1[(long long)r * kHid + j] = h;
    if (z1) z1[(long long)r * kHid + j] = z;
    if (h1t) h1t[(long long)j * ldt + r] = h;
}

// Output layer (256 -> 3), one warp per row; with targets also the loss L = sum w (y - t)^2 / (3 n) (w = 1
// without weights), dy = dL/dy and the gradient through the output layer into the last hidden layer
// (dz4 = (dy . W5) * silu'(z4)).
__global__ void head_kernel(const bf16* __restrict__ h4, const float* __restrict__ z4, int n,
                            const bf16* __restrict__ w5, const float* __restrict__ b5, const float* __restrict__ tb,
                            const float* __restrict__ wb, float* y, float* dy, bf16* dz4, bf16* dz4t, long long ldt,
                            float* loss_sum) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int r = warp;
    float hv[8], acc[kOut] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 8; ++i) hv[i] = __bfloat162float(h4[(long long)r * kHid + lane * 8 + i]);
#pragma unroll
    for (int k = 0; k < kOut; ++k)
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[k] = fmaf(hv[i], __bfloat162float(w5[k * kHid + lane * 8 + i]), acc[k]);
#pragma unroll
    for (int k = 0; k < kOut; ++k)
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    float yv[kOut];
#pragma unroll
    for (int k = 0; k < kOut; ++k) yv[k] = acc[k] + b5[k];
    if (y && lane == 0)
#pragma unroll
        for (int k = 0; k < kOut; ++k) y[r * kOut + k] = yv[k];
    if (!tb) return;
    const float scale = 2.0f / (3.0f * (float)n);
    float d[kOut], l = 0.0f;
#pragma unroll
    for (int k = 0; k < kOut; ++k) {
        const float e = yv[k] - tb[r * kOut + k];
        const float we = wb ? wb[r * kOut + k] * e : e;
        d[k] = scale * we;
        l += we * e;
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < kOut; ++k) dy[r * kOut + k] = d[k];
        atomicAdd(loss_sum, l);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int j = lane * 8 + i;
        float g = 0.0f;
#pragma unroll
        for (int k = 0; k < kOut; ++k) g = fmaf(d[k], __bfloat162float(w5[k * kHid + j]), g);
        const bf16 v = __float2bfloat16(g * dsilu_f(z4[(long long)r * kHid + j]));
        dz4[(long long)r * kHid + j] = v;
        dz4t[(long long)j * ldt + r] = v;
    }
}

// Small gradient reductions over the batch, one thread per output, rows split over blockIdx.y:
//   db_l[j] = sum_r dz_l[r][j] (l = 1..4, from the transposed copies), dW1[j][i] = sum_r dz1[r][j] x[r][i],
//   dW5[k][j] = sum_r dy[r][k] h4[r][j], db5[k] = sum_r dy[r][k].
__global__ void small_grads_kernel(const bf16* const* __restrict__ dzt, long long ldt, const float* __restrict__ xb,
                                   const float* __restrict__ dy, const bf16* __restrict__ h4, int n, int rows_per,
                                   float* grads) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int r0 = blockIdx.y * rows_per, r1 = min(n, r0 + rows_per);
    constexpr int kBias = 4 * kHid, kW1 = kHid * kIn, kW5 = kOut * kHid;
    if (t < kBias) {
        const int l = t / kHid, j = t % kHid;
        const bf16* row = dzt[l] + (long long)j * ldt;
        float s = 0.0f;
        for (int r = r0; r < r1; ++r) s += __bfloat162float(row[r]);
        atomicAdd(grads + off_b(l + 1) + j, s);
    } else if (t < kBias + kW1) {
        const int q = t - kBias, j = q / kIn, i = q % kIn;
        const bf16* row = dzt[0] + (long long)j * ldt;
        float s = 0.0f;
        for (int r = r0; r < r1; ++r) s = fmaf(__bfloat162float(row[r]), xb[r * kIn + i], s);
        atomicAdd(grads + kOffW1 + q, s);
    } else if (t < kBias + kW1 + kW5) {
        const int q = t - kBias - kW1, k = q / kHid, j = q % kHid;
        float s = 0.0f;
        for (int r = r0; r < r1; ++r) s = fmaf(dy[r * kOut + k], __bfloat162float(h4[(long long)r * kHid + j]), s);
        atomicAdd(grads + kOffW5 + q, s);
    } else if (t < kBias + kW1 + kW5 + kOut) {
        const int k = t - kBias - kW1 - kW5;
        float s = 0.0f;
        for (int r = r0; r < r1; ++r) s += dy[r * kOut + k];
        atomicAdd(grads + kOffB5 + k, s);
    }
}

// BF16 copies of the weights: w[l] = W_l as [out][in] and wt[l] = W_l^T as [in][out] (l = 2..4), plus
// W1 and W5 as [out][in]. One thread per parameter.
struct PackArgs {
    bf16* w[6];
    bf16* wt[6];
    bf16* wp[6];  // l = 2..4: the shared-memory image of W_l as a B operand (256 x 256 core-matrix layout)
};
// element (r, k) of a K = 256 operand image in the core-matrix layout (8 x 16-byte core matrices, K-adjacent
// core matrices 128 bytes apart, 8-row groups 4096 bytes apart), in BF16 elements
__host__ __device__ __forceinline__ int img_idx(int r, int k) {
    return ((r >> 3) * 4096 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2) >> 1;
}
__device__ __forceinline__ void pack_one(const PackArgs& pa, long long p, float v) {
    const bf16 b = __float2bfloat16(v);
    for (int l = 1; l <= 5; ++l) {
        const int nin = (l == 1) ? kIn : kHid;
        const int nout = (l == 5) ? kOut : kHid;
        const long long o = p - off_w(l);
        if (o >= 0 && o < (long long)nin * nout) {
            pa.w[l][o] = b;
            const int out = (int)(o / nin), in = (int)(o % nin);
            if (pa.wt[l]) pa.wt[l][(long long)in * nout + out] = b;
            if (pa.wp[l]) {
                if (l == 1)  // 256 x 16 image (K = 16): 8-row groups 256 bytes apart
                    pa.wp[1][((out >> 3) * 256 + (in >> 3) * 128 + (out & 7) * 16 + (in & 7) * 2) >> 1] = b;
                else
                    pa.wp[l][img_idx(out, in)] = b;  // 256 x 256, or 16 x 256 for W5 (rows 3..15 stay zero)
            }
        }
    }
}
__global__ void pack_kernel(const float* __restrict__ params, PackArgs pa) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < kParams) pack_one(pa, p, params[p]);
}

// Adam (bias-corrected) on every parameter, then the gradient is cleared and the BF16 copies refreshed.
__global__ void adam_kernel(float* params, float* grads, float* m1, float* m2, float lr, float b1, float b2,
                            float eps, float c1, float c2, PackArgs pa) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    const float g = grads[p];
    const float a = b1 * m1[p] + (1.0f - b1) * g;
    const float b = b2 * m2[p] + (1.0f - b2) * g * g;
    m1[p] = a;
    m2[p] = b;
    const float v = params[p] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    params[p] = v;
    grads[p] = 0.0f;
    pack_one(pa, p, v);
}

// ---------------- fused inference: every layer of a 128-row tile on one SM ----------------
// A persistent CTA per SM walks 128-row tiles, with every product on the tensor cores: layer 1 as one
// tcgen05.mma with K padded from 6 to 16, the three 256x256 layers as 16 MMAs each, and the 256 -> 3
// output layer as 16 MMAs with N padded to 16. The small padded weight images (W1, W5) stay in shared
// memory; each 256x256 weight image (128 KB) comes in by one cp.async.bulk copy that starts as soon as
// the previous layer's MMAs have completed, so it overlaps that layer's epilogue. Each epilogue reads the
// accumulator with tcgen05.ld, adds the bias, applies SiLU (one tanh.approx per element) and writes the
// next layer's A image. Activations never leave the SM.
constexpr int kInferThreads = 512;               // warp w reads TMEM lane quarter w % 4, columns 64 (w / 4) ..
constexpr int kABytes = kM * kHid * 2;           // 64 KB: the tile's activations, K = 256
constexpr int kWBytes = kHid * kHid * 2;         // 128 KB: one 256x256 weight image
constexpr int kXBytes = kM * 16 * 2;             // 4 KB: the tile's inputs, K padded to 16
constexpr int kW1Bytes = kHid * 16 * 2;          // 8 KB: W1 image, 256 x 16
constexpr int kW5Bytes = 16 * kHid * 2;          // 8 KB: W5 image, 16 (3 used) x 256
constexpr int kOffSmW = kABytes;
constexpr int kOffSmX = kOffSmW + kWBytes;
constexpr int kOffSmW1 = kOffSmX + kXBytes;
constexpr int kOffSmW5 = kOffSmW1 + kW1Bytes;
constexpr int kOffSmBias = kOffSmW5 + kW5Bytes;              // f32 [4][256]: b1..b4
constexpr int kOffSmB5 = kOffSmBias + 4 * kHid * 4;          // f32 [4]
constexpr int kOffSmBar = kOffSmB5 + 16;                     // 2 mbarriers
constexpr int kOffSmSlot = kOffSmBar + 16;                   // TMEM address
constexpr int kInferSmem = kOffSmSlot + 16;
static_assert(kOffSmBar % 8 == 0 && kInferSmem <= 227 * 1024, "shared-memory plan");
// instruction descriptors: N = 256 (hidden layers) and N = 16 (output layer)
constexpr uint32_t kIdescN16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(16 >> 3) << 17) |
                               ((uint32_t)(kM >> 4) << 24);

struct InferArgs {
    const float* x;      // [n][6]
    float* y;            // [n][3]
    long long n;
    int tiles;
    const bf16* wp[3];   // images of W2, W3, W4 (256 x 256)
    const bf16* w1p;     // image of W1 padded to 256 x 16
    const bf16* w5p;     // image of W5 padded to 16 x 256
    const float* params;
    int* err;
};

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// silu(z) = z/2 (1 + tanh(z/2)): one multi-function-unit operation per element (hardware tanh approximation,
// relative error far below the BF16 rounding that follows)
__device__ __forceinline__ float silu_tanh(float z) {
    const float h = 0.5f * z;
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
    return fmaf(h, t, h);
}
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
    uint32_t r0, r1, r2, r3;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    v[0] = __uint_as_float(r0); v[1] = __uint_as_float(r1); v[2] = __uint_as_float(r2); v[3] = __uint_as_float(r3);
}

__global__ void __launch_bounds__(kInferThreads, 1) mlp_infer_kernel(InferArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    bf16* A = reinterpret_cast<bf16*>(sm);
    bf16* W = reinterpret_cast<bf16*>(sm + kOffSmW);
    unsigned char* X = sm + kOffSmX;
    float* bs = reinterpret_cast<float*>(sm + kOffSmBias);
    float* b5s = reinterpret_cast<float*>(sm + kOffSmB5);
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + kOffSmBar);  // [0] weights arrived, [1] MMAs done
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + kOffSmSlot);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, cgroup = warp >> 2;  // TMEM lane quarter, group of 64 columns
    const int r = quarter * 32 + lane;  // this thread's row of the tile (and TMEM lane)
    {
        const uint4* s1 = reinterpret_cast<const uint4*>(a.w1p);
        const uint4* s5 = reinterpret_cast<const uint4*>(a.w5p);
        uint4* d1 = reinterpret_cast<uint4*>(sm + kOffSmW1);
        uint4* d5 = reinterpret_cast<uint4*>(sm + kOffSmW5);
        for (int i = tid; i < kW1Bytes / 16; i += kInferThreads) d1[i] = s1[i];
        for (int i = tid; i < kW5Bytes / 16; i += kInferThreads) d5[i] = s5[i];
    }
    for (int i = tid; i < 4 * kHid; i += kInferThreads) bs[i] = a.params[off_b(1 + i / kHid) + i % kHid];
    if (tid < kOut) b5s[tid] = a.params[kOffB5 + tid];
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tmem_alloc(tslot, 256);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t tlane = tmem + ((uint32_t)(quarter * 32) << 16);
    const uint32_t sA = smem_u32(A), sW = smem_u32(W), sX = smem_u32(X);
    const uint32_t sW1 = smem_u32(sm + kOffSmW1), sW5 = smem_u32(sm + kOffSmW5);
    unsigned wphase = 0, mphase = 0;
    bool w_pending = false;  // thread 0: a weight copy was issued and not yet waited for
    if (tid == 0 && (int)blockIdx.x < a.tiles) {
        bulk_load(W, a.wp[0], kWBytes, &bar[0]);
        w_pending = true;
    }
    // MMAs of one layer by thread 0, then every thread waits for their completion (bounded)
    auto run_mma = [&](int kind) -> bool {
        bool issued = true;
        if (tid == 0) {
            if (kind == 1) {  // 256x256 layer: needs its weight image
                issued = mbar_wait(&bar[0], wphase & 1u, a.err, 3);
                w_pending = !issued;
            }
            if (issued) {
                tc_fence_after();
                if (kind == 0) {
                    mma_bf16(tmem, smem_desc(sX, 128, 256), smem_desc(sW1, 128, 256), kIdesc, 0u);
                } else {
                    const uint32_t b0 = kind == 1 ? sW : sW5;
                    const uint32_t idesc = kind == 1 ? kIdesc : kIdescN16;
#pragma unroll
                    for (int kk = 0; kk < kHid / 16; ++kk)
                        mma_bf16(tmem, smem_desc(sA + kk * 256, 128, 4096), smem_desc(b0 + kk * 256, 128, 4096),
                                 idesc, kk > 0 ? 1u : 0u);
                }
                mma_commit(&bar[1]);
            }
        }
        if (kind == 1) wphase++;
        if (!__syncthreads_and(issued)) return false;
        const bool done = mbar_wait(&bar[1], mphase & 1u, a.err, 4);
        mphase++;
        return __syncthreads_and(done);
    };
    // bias + SiLU of this thread's 64 columns of the accumulator row into the next A image
    auto hidden_epilogue = [&](const float* bias) {
        tc_fence_after();
#pragma unroll 1
        for (int c = 0; c < 2; ++c) {
            const int j0 = cgroup * 64 + c * 32;
            float v[32];
            tmem_ld32(tlane + (uint32_t)j0, v);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 b0 = *reinterpret_cast<const float4*>(bias + j0 + 8 * q);
                const float4 b1 = *reinterpret_cast<const float4*>(bias + j0 + 8 * q + 4);
                const float* e = v + 8 * q;
                uint4 o;
                o.x = pack_bf16x2(silu_tanh(e[0] + b0.x), silu_tanh(e[1] + b0.y));
                o.y = pack_bf16x2(silu_tanh(e[2] + b0.z), silu_tanh(e[3] + b0.w));
                o.z = pack_bf16x2(silu_tanh(e[4] + b1.x), silu_tanh(e[5] + b1.y));
                o.w = pack_bf16x2(silu_tanh(e[6] + b1.z), silu_tanh(e[7] + b1.w));
                *reinterpret_cast<uint4*>(A + img_idx(r, j0 + 8 * q)) = o;
            }
        }
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
    };
    bool ok = true;
    for (int tile = blockIdx.x; tile < a.tiles && ok; tile += gridDim.x) {
        const long long row = (long long)tile * kM + r;
        const bool valid = row < a.n;
        if (cgroup == 0) {  // the tile's inputs as a 128 x 16 A image (K 6..15 zero)
            float xv[kIn];
#pragma unroll
            for (int i = 0; i < kIn; ++i) xv[i] = valid ? a.x[row * kIn + i] : 0.0f;
            uint4 lo;
            lo.x = pack_bf16x2(xv[0], xv[1]);
            lo.y = pack_bf16x2(xv[2], xv[3]);
            lo.z = pack_bf16x2(xv[4], xv[5]);
            lo.w = 0u;
            *reinterpret_cast<uint4*>(X + (r >> 3) * 256 + (r & 7) * 16) = lo;
            *reinterpret_cast<uint4*>(X + (r >> 3) * 256 + 128 + (r & 7) * 16) = make_uint4(0u, 0u, 0u, 0u);
        }
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        if (!(ok = run_mma(0))) break;
        hidden_epilogue(bs);
        for (int l = 0; l < 3 && ok; ++l) {
            if (!(ok = run_mma(1))) break;
            // the weight buffer is free: bring in the next layer's weights (or the first layer's for the next tile)
            if (tid == 0) {
                if (l < 2) { bulk_load(W, a.wp[l + 1], kWBytes, &bar[0]); w_pending = true; }
                else if (tile + (int)gridDim.x < a.tiles) { bulk_load(W, a.wp[0], kWBytes, &bar[0]); w_pending = true; }
            }
            hidden_epilogue(bs + (l + 1) * kHid);
        }
        if (!ok) break;
        if (!(ok = run_mma(2))) break;
        tc_fence_after();
        float v[4];
        if (cgroup == 0) {
            tmem_ld4(tlane, v);
            if (valid)
#pragma unroll
                for (int k = 0; k < kOut; ++k) a.y[row * kOut + k] = v[k] + b5s[k];
        }
        tc_fence_before();
        __syncthreads();
    }
    // a weight copy still in flight (only after a failed wait) must land before the CTA leaves
    if (tid == 0 && w_pending) (void)mbar_wait(&bar[0], wphase & 1u, a.err, 5);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 256);
    }
}

}  // namespace mlpk

using namespace mlpk;

// ---------------- the network object behind the C ABI ----------------
struct clr_mlp {
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    int cap = 0;  // batch rows of the work buffers (multiple of 128)
    std::string err;
    std::vector<void*> allocs;
    float *params = nullptr, *grads = nullptr, *m1 = nullptr, *m2 = nullptr;
    PackArgs pa{};
    float* z[5] = {};          // [cap][256] pre-activations of hidden layers 1..4
    bf16* h[5] = {};           // [cap][256] activations
    bf16* ht[5] = {};          // [256][cap] transposed activations
    bf16* dz[5] = {};          // [cap][256] gradients at the pre-activations
    bf16* dzt[5] = {};         // [256][cap]
    const bf16** d_dzt = nullptr;  // device array of dzt[1..4]
    float *xb = nullptr, *tb = nullptr, *dy = nullptr, *y = nullptr, *loss = nullptr;
    float* wb = nullptr;          // [cap][3] loss weights of the batch rows
    const float* d_w = nullptr;   // the caller's loss weights (clr_mlp_set_loss_weights), or null
    int* d_err = nullptr;
    long long steps = 0;
    float last_ms = 0.0f;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // one captured training step per batch size
    cudaGraphExec_t step_exec = nullptr;
    int step_n = 0;
    const float* step_x = nullptr;
    const float* step_t = nullptr;
    const int32_t* step_idx = nullptr;
    const float* step_w = nullptr;
    long long* d_row0 = nullptr;  // device copy of the batch's first index position (graph input)
    float* d_lr = nullptr;        // device scalars of the captured Adam step: lr, c1, c2
};

static int mfail(clr_mlp* m, int code, const char* msg) {
    if (m) m->err = msg;
    return code;
}
#define MCU(call)                                                                           \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            if (m) m->err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
            return CLR_ERR_CUDA;                                                            \
        }                                                                                   \
    } while (0)

static cudaError_t malloc_tracked(clr_mlp* m, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) m->allocs.push_back(*p);
    return e;
}

// Forward pass of n rows (n <= cap) already gathered into xb. With `train` the pre-activations and
// transposed activations are kept for the backward pass.
static cudaError_t forward_rows(clr_mlp* m, int n, bool train, cudaStream_t st) {
    const int thr = 256;
    layer1_kernel<<<(int)(((long long)n * kHid + thr - 1) / thr), thr, 0, st>>>(
        m->xb, n, m->pa.w[1], m->params + kOffB1, train ? m->z[1] : nullptr, m->h[1], train ? m->ht[1] : nullptr,
        m->cap);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    for (int l = 2; l <= 4; ++l) {
        GemmArgs g{};
        g.A = m->h[l - 1]; g.lda = kHid; g.B = m->pa.w[l]; g.ldb = kHid;
        g.M = n; g.K = kHid; g.k_split = kHid;
        g.bias = m->params + off_b(l);
        g.out_f32 = m->z[l]; g.ldo = kHid; g.out_bf16 = m->h[l]; g.out_bf16_t = m->ht[l]; g.ldt = m->cap;
        g.err = m->d_err;
        e = train ? launch_gemm<EPI_FWD>(g, 1, st) : launch_gemm<EPI_INFER>(g, 1, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Backward pass of the n rows of the last forward (targets in tb): gradients accumulate into grads.
static cudaError_t backward_rows(clr_mlp* m, int n, cudaStream_t st) {
    head_kernel<<<(n * 32 + 255) / 256, 256, 0, st>>>(m->h[4], m->z[4], n, m->pa.w[5], m->params + kOffB5, m->tb,
                                                      m->d_w ? m->wb : nullptr,
                                                      m->y, m->dy, m->dz[4], m->dzt[4], m->cap, m->loss);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    for (int l = 4; l >= 2; --l) {  // dz_{l-1} = (dz_l . W_l) * silu'(z_{l-1})
        GemmArgs g{};
        g.A = m->dz[l]; g.lda = kHid; g.B = m->pa.wt[l]; g.ldb = kHid;
        g.M = n; g.K = kHid; g.k_split = kHid;
        g.zin = m->z[l - 1]; g.out_bf16 = m->dz[l - 1]; g.out_bf16_t = m->dzt[l - 1]; g.ldt = m->cap;
        g.err = m->d_err;
        if ((e = launch_gemm<EPI_BWD>(g, 1, st)) != cudaSuccess) return e;
    }
    const int ksplit = 512;
    for (int l = 2; l <= 4; ++l) {  // dW_l = dz_l^T . h_{l-1}, split over the batch
        GemmArgs g{};
        g.A = m->dzt[l]; g.lda = m->cap; g.B = m->ht[l - 1]; g.ldb = m->cap;
        g.M = kHid; g.K = n; g.k_split = ksplit;
        g.out_f32 = m->grads + off_w(l); g.ldo = kHid; g.err = m->d_err;
        if ((e = launch_gemm<EPI_ATOMIC_F32>(g, (n + ksplit - 1) / ksplit, st)) != cudaSuccess) return e;
    }
    const int rows_per = 256;
    const int outs = 4 * kHid + kHid * kIn + kOut * kHid + kOut;
    dim3 grid((outs + 255) / 256, (n + rows_per - 1) / rows_per);
    small_grads_kernel<<<grid, 256, 0, st>>>(m->d_dzt, m->cap, m->xb, m->dy, m->h[4], n, rows_per, m->grads);
    return cudaGetLastError();
}

static int check_dev(clr_mlp* m) {
    int herr = 0;
    MCU(cudaMemcpyAsync(&herr, m->d_err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    MCU(cudaStreamSynchronize(m->stream));
    if (herr) {
        MCU(cudaMemsetAsync(m->d_err, 0, sizeof(int), m->stream));
        return mfail(m, CLR_ERR_DEVICE_TIMEOUT, "tensor-core GEMM timed out waiting for its MMAs");
    }
    return CLR_OK;
}

extern "C" {

int clr_mlp_create(clr_mlp** out, int device, int max_batch, uint64_t seed) {
    if (!out || max_batch < 128 || max_batch % 128) return CLR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    clr_mlp* m = new clr_mlp();
    m->device = device;
    m->cap = max_batch;
    MCU(cudaSetDevice(device));
    MCU(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    MCU(set_gemm_attributes());
    MCU(cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem));
    MCU(cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, device));
    MCU(cudaEventCreate(&m->ev0));
    MCU(cudaEventCreate(&m->ev1));
    auto F = [&](float** p, size_t cnt) { return malloc_tracked(m, (void**)p, cnt * sizeof(float)); };
    auto H = [&](bf16** p, size_t cnt) { return malloc_tracked(m, (void**)p, cnt * sizeof(bf16)); };
    MCU(F(&m->params, kParams)); MCU(F(&m->grads, kParams)); MCU(F(&m->m1, kParams)); MCU(F(&m->m2, kParams));
    for (int l = 1; l <= 5; ++l) {
        const int nin = l == 1 ? kIn : kHid, nout = l == 5 ? kOut : kHid;
        MCU(H(&m->pa.w[l], (size_t)nin * nout));
        if (l >= 2 && l <= 4) {
            MCU(H(&m->pa.wt[l], (size_t)nin * nout));
            MCU(H(&m->pa.wp[l], (size_t)nin * nout));
        }
        if (l == 1 || l == 5) {  // padded images: zero padding written once, weights by every pack
            MCU(H(&m->pa.wp[l], (size_t)kHid * 16));
            MCU(cudaMemset(m->pa.wp[l], 0, (size_t)kHid * 16 * sizeof(bf16)));
        }
    }
    const size_t act = (size_t)m->cap * kHid;
    for (int l = 1; l <= 4; ++l) {
        MCU(F(&m->z[l], act)); MCU(H(&m->h[l], act)); MCU(H(&m->ht[l], act));
        MCU(H(&m->dz[l], act)); MCU(H(&m->dzt[l], act));
    }
    MCU(F(&m->xb, (size_t)m->cap * kIn)); MCU(F(&m->tb, (size_t)m->cap * kOut)); MCU(F(&m->wb, (size_t)m->cap * kOut));
    MCU(F(&m->dy, (size_t)m->cap * kOut)); MCU(F(&m->y, (size_t)m->cap * kOut)); MCU(F(&m->loss, 4));
    MCU(malloc_tracked(m, (void**)&m->d_err, sizeof(int)));
    MCU(malloc_tracked(m, (void**)&m->d_dzt, 4 * sizeof(bf16*)));
    MCU(malloc_tracked(m, (void**)&m->d_row0, sizeof(long long)));
    MCU(F(&m->d_lr, 4));
    const bf16* dzt[4] = {m->dzt[1], m->dzt[2], m->dzt[3], m->dzt[4]};
    MCU(cudaMemcpy(m->d_dzt, dzt, sizeof dzt, cudaMemcpyHostToDevice));
    MCU(cudaMemset(m->d_err, 0, sizeof(int)));
    MCU(cudaMemset(m->grads, 0, kParams * sizeof(float)));
    MCU(cudaMemset(m->m1, 0, kParams * sizeof(float)));
    MCU(cudaMemset(m->m2, 0, kParams * sizeof(float)));
    // initial weights and biases uniform in +-1/sqrt(fan_in) from a seeded host generator
    std::vector<float> p(kParams);
    std::mt19937_64 rng(seed);
    for (int l = 1; l <= 5; ++l) {
        const int nin = l == 1 ? kIn : kHid, nout = l == 5 ? kOut : kHid;
        std::uniform_real_distribution<float> U(-1.0f / std::sqrt((float)nin), 1.0f / std::sqrt((float)nin));
        for (long long i = 0; i < (long long)nin * nout; ++i) p[off_w(l) + i] = U(rng);
        for (int i = 0; i < nout; ++i) p[off_b(l) + i] = U(rng);
    }
    MCU(cudaMemcpy(m->params, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice));
    pack_kernel<<<(int)((kParams + 255) / 256), 256, 0, m->stream>>>(m->params, m->pa);
    MCU(cudaGetLastError());
    MCU(cudaStreamSynchronize(m->stream));
    *out = m;
    return CLR_OK;
}

int clr_mlp_destroy(clr_mlp* m) {
    if (!m) return CLR_ERR_INVALID_ARGUMENT;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    if (m->step_exec) cudaGraphExecDestroy(m->step_exec);
    for (void* p : m->allocs) cudaFree(p);
    if (m->ev0) cudaEventDestroy(m->ev0);
    if (m->ev1) cudaEventDestroy(m->ev1);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return CLR_OK;
}

const char* clr_mlp_last_error(const clr_mlp* m) { return m ? m->err.c_str() : "null network"; }

int clr_mlp_set_params(clr_mlp* m, const float* host, int64_t count) {
    if (!m || !host || count != kParams) return mfail(m, CLR_ERR_INVALID_ARGUMENT, "expected CLR_MLP_PARAMS floats");
    MCU(cudaSetDevice(m->device));
    MCU(cudaMemcpyAsync(m->params, host, kParams * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    MCU(cudaMemsetAsync(m->m1, 0, kParams * sizeof(float), m->stream));
    MCU(cudaMemsetAsync(m->m2, 0, kParams * sizeof(float), m->stream));
    pack_kernel<<<(int)((kParams + 255) / 256), 256, 0, m->stream>>>(m->params, m->pa);
    MCU(cudaGetLastError());
    MCU(cudaStreamSynchronize(m->stream));
    m->steps = 0;
    return CLR_OK;
}

int clr_mlp_get_params(clr_mlp* m, float* host, int64_t count) {
    if (!m || !host || count != kParams) return mfail(m, CLR_ERR_INVALID_ARGUMENT, "expected CLR_MLP_PARAMS floats");
    MCU(cudaSetDevice(m->device));
    MCU(cudaMemcpyAsync(host, m->params, kParams * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCU(cudaStreamSynchronize(m->stream));
    return CLR_OK;
}

int clr_mlp_forward(clr_mlp* m, const float* d_x, int64_t n, float* d_y, void* stream) {
    if (!m || !d_x || !d_y || n < 0) return mfail(m, CLR_ERR_INVALID_ARGUMENT, "clr_mlp_forward: bad arguments");
    MCU(cudaSetDevice(m->device));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : m->stream;
    MCU(cudaEventRecord(m->ev0, st));
    if (n > 0) {
        InferArgs a{};
        a.x = d_x; a.y = d_y; a.n = n;
        const long long tiles = (n + kM - 1) / kM;
        if (tiles > (1LL << 30)) return mfail(m, CLR_ERR_INVALID_ARGUMENT, "clr_mlp_forward: too many rows");
        a.tiles = (int)tiles;
        a.wp[0] = m->pa.wp[2]; a.wp[1] = m->pa.wp[3]; a.wp[2] = m->pa.wp[4];
        a.w1p = m->pa.wp[1]; a.w5p = m->pa.wp[5]; a.params = m->params; a.err = m->d_err;
        const int grid = (int)std::min<long long>(tiles, m->num_sms);
        mlp_infer_kernel<<<grid, kInferThreads, kInferSmem, st>>>(a);
        MCU(cudaGetLastError());
    }
    MCU(cudaEventRecord(m->ev1, st));
    MCU(cudaStreamSynchronize(st));
    MCU(cudaEventElapsedTime(&m->last_ms, m->ev0, m->ev1));
    return check_dev(m);
}

int clr_mlp_gradients(clr_mlp* m, const float* d_x, const float* d_t, int64_t n, float* grads_host, float* loss) {
    if (!m || !d_x || !d_t || n < 128 || n > m->cap || n % 128)
        return mfail(m, CLR_ERR_INVALID_ARGUMENT, "clr_mlp_gradients: n must be a multiple of 128 up to max_batch");
    MCU(cudaSetDevice(m->device));
    cudaStream_t st = m->stream;
    MCU(cudaMemsetAsync(m->grads, 0, kParams * sizeof(float), st));
    MCU(cudaMemsetAsync(m->loss, 0, sizeof(float), st));
    gather_kernel<<<((int)n + 255) / 256, 256, 0, st>>>(d_x, d_t, m->d_w, nullptr, 0, (int)n, m->xb, m->tb, m->wb);
    MCU(cudaGetLastError());
    MCU(forward_rows(m, (int)n, true, st));
    MCU(backward_rows(m, (int)n, st));
    float ls = 0.0f;
    MCU(cudaMemcpyAsync(&ls, m->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    if (grads_host) MCU(cudaMemcpyAsync(grads_host, m->grads, kParams * sizeof(float), cudaMemcpyDeviceToHost, st));
    MCU(cudaMemsetAsync(m->grads, 0, kParams * sizeof(float), st));
    int rc = check_dev(m);
    if (rc != CLR_OK) return rc;
    if (loss) *loss = ls / (3.0f * (float)n);
    return CLR_OK;
}

}  // extern "C"

// Gathers batch rows by index, with the batch start read from device memory so the captured step
// serves every batch of an epoch.
__global__ void gather_dev_kernel(const float* __restrict__ x, const float* __restrict__ t,
                                  const float* __restrict__ w, const int32_t* __restrict__ idx,
                                  const long long* __restrict__ row0, int n, float* xb, float* tb, float* wb) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const long long src = (long long)idx[*row0 + r];
#pragma unroll
    for (int i = 0; i < kIn; ++i) xb[r * kIn + i] = bfr(x[src * kIn + i]);
#pragma unroll
    for (int i = 0; i < kOut; ++i) tb[r * kOut + i] = t[src * kOut + i];
    if (w)
#pragma unroll
        for (int i = 0; i < kOut; ++i) wb[r * kOut + i] = w[src * kOut + i];
}

__global__ void adam_dev_kernel(float* params, float* grads, float* m1, float* m2, const float* __restrict__ hp,
                                PackArgs pa) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    const float lr = hp[0], c1 = hp[1], c2 = hp[2];
    const float g = grads[p];
    const float a = 0.9f * m1[p] + 0.1f * g;
    const float b = 0.999f * m2[p] + 0.001f * g * g;
    m1[p] = a;
    m2[p] = b;
    const float v = params[p] - lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
    params[p] = v;
    grads[p] = 0.0f;
    pack_one(pa, p, v);
}

// One training step (gather, forward, backward, Adam) captured as a graph for batch size n.
static int build_step_graph(clr_mlp* m, const float* d_x, const float* d_t, const int32_t* d_idx, int n) {
    if (m->step_exec && m->step_n == n && m->step_x == d_x && m->step_t == d_t && m->step_idx == d_idx &&
        m->step_w == m->d_w)
        return CLR_OK;
    if (m->step_exec) {
        cudaGraphExecDestroy(m->step_exec);
        m->step_exec = nullptr;
    }
    cudaStream_t st = m->stream;
    cudaGraph_t graph;
    MCU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    gather_dev_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_x, d_t, m->d_w, d_idx, m->d_row0, n, m->xb, m->tb, m->wb);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = forward_rows(m, n, true, st);
    if (e == cudaSuccess) e = backward_rows(m, n, st);
    if (e == cudaSuccess) {
        adam_dev_kernel<<<(int)((kParams + 255) / 256), 256, 0, st>>>(m->params, m->grads, m->m1, m->m2, m->d_lr,
                                                                       m->pa);
        e = cudaGetLastError();
    }
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    MCU(e);
    MCU(e2);
    e = cudaGraphInstantiate(&m->step_exec, graph, 0);
    cudaGraphDestroy(graph);
    MCU(e);
    m->step_n = n; m->step_x = d_x; m->step_t = d_t; m->step_idx = d_idx; m->step_w = m->d_w;
    return CLR_OK;
}

extern "C" int clr_mlp_train(clr_mlp* m, const float* d_x, const float* d_t, const int32_t* d_index, int64_t n_index,
                             int batch, float lr, float* mean_loss) {
    if (!m || !d_x || !d_t || !d_index || batch < 128 || batch % 128 || batch > m->cap || n_index < batch)
        return mfail(m, CLR_ERR_INVALID_ARGUMENT,
                     "clr_mlp_train: batch must be a multiple of 128 up to max_batch, and at most n_index");
    MCU(cudaSetDevice(m->device));
    int rc = build_step_graph(m, d_x, d_t, d_index, batch);
    if (rc != CLR_OK) return rc;
    cudaStream_t st = m->stream;
    MCU(cudaMemsetAsync(m->loss, 0, sizeof(float), st));
    const long long steps = n_index / batch;
    MCU(cudaEventRecord(m->ev0, st));
    for (long long s = 0; s < steps; ++s) {
        const long long row0 = s * batch;
        m->steps++;
        const float hp[3] = {lr, 1.0f - std::pow(0.9f, (float)m->steps), 1.0f - std::pow(0.999f, (float)m->steps)};
        // pageable copies are staged by the driver before the call returns, so the host values may change
        MCU(cudaMemcpyAsync(m->d_row0, &row0, sizeof row0, cudaMemcpyHostToDevice, st));
        MCU(cudaMemcpyAsync(m->d_lr, hp, sizeof hp, cudaMemcpyHostToDevice, st));
        MCU(cudaGraphLaunch(m->step_exec, st));
    }
    MCU(cudaEventRecord(m->ev1, st));
    float ls = 0.0f;
    MCU(cudaMemcpyAsync(&ls, m->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    rc = check_dev(m);
    if (rc != CLR_OK) return rc;
    MCU(cudaEventElapsedTime(&m->last_ms, m->ev0, m->ev1));
    if (mean_loss) *mean_loss = steps > 0 ? ls / (3.0f * (float)batch * (float)steps) : 0.0f;
    return CLR_OK;
}

extern "C" int clr_mlp_set_loss_weights(clr_mlp* m, const float* d_w) {
    if (!m) return CLR_ERR_INVALID_ARGUMENT;
    m->d_w = d_w;
    return CLR_OK;
}

extern "C" int clr_mlp_last_ms(const clr_mlp* m, float* ms) {
    if (!m || !ms) return CLR_ERR_INVALID_ARGUMENT;
    *ms = m->last_ms;
    return CLR_OK;
}

// Plain tensor-core product C[M][256] = A[M][K] . B[256][K]^T (BF16 in, FP32 out), the kernel the
// network's layers use, exposed for its own tests and for callers with other 256-wide products.
extern "C" int clr_bf16_gemm_n256(const void* d_a, int64_t lda, const void* d_b, int64_t ldb, int64_t M, int64_t K,
                                  float* d_c, int64_t ldc, void* stream) {
    if (!d_a || !d_b || !d_c || M < 1 || K < 64 || K % 64 || lda % 8 || ldb % 8 || ldc % 4 || lda < K || ldb < K ||
        ldc < 256 || (reinterpret_cast<uintptr_t>(d_a) & 15) || (reinterpret_cast<uintptr_t>(d_b) & 15) ||
        (reinterpret_cast<uintptr_t>(d_c) & 15))
        return CLR_ERR_INVALID_ARGUMENT;
    static int* err = nullptr;  // error word of this entry point (first device it runs on)
    if (!err && cudaMalloc(&err, sizeof(int)) != cudaSuccess) return CLR_ERR_CUDA;
    if (set_gemm_attributes() != cudaSuccess) return CLR_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) return CLR_ERR_CUDA;
    GemmArgs g{};
    g.A = static_cast<const bf16*>(d_a); g.lda = lda; g.B = static_cast<const bf16*>(d_b); g.ldb = ldb;
    g.M = (int)M; g.K = (int)K; g.k_split = (int)K; g.out_f32 = d_c; g.ldo = ldc; g.err = err;
    if (launch_gemm<EPI_STORE_F32>(g, 1, st) != cudaSuccess) return CLR_ERR_CUDA;
    int herr = 0;
    if (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return CLR_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return CLR_ERR_CUDA;
    return herr ? CLR_ERR_DEVICE_TIMEOUT : CLR_OK;
}
