// Random streams for the photon kernel.
//
// Two back-ends share one interface (next() returns a raw 32-bit word):
//  * XorStream reproduces the reference's per-ray xorshift32 streams
//    (CLARITAS/CLARITAS.py:1125-1129; seeding :4612 and :4396-4397) for
//    bit-exact parity runs;
//  * PhiloxStream is a counter-based Philox4x32-10 generator (Salmon et al.,
//    SC'11) keyed by the run seed, with the counter (ray id, scenario, draw
//    index): every photon owns a disjoint, reproducible sequence no matter how
//    rays are partitioned over blocks, launches or GPUs.
// The float/double conversions are the reference's (rnd_uniform :1131-1133,
// beckmann_open_uniform :1908-1912, conditional_uniform :4486-4490), so both
// back-ends feed identical sampling code.
#pragma once
#include <cstdint>

namespace clr {

struct XorStream {
    uint32_t s;
    __device__ __forceinline__ uint32_t next() {
        uint32_t x = s;
        x ^= x << 13; x ^= x >> 17; x ^= x << 5;
        s = x;
        return x;
    }
};

struct PhiloxStream {
    uint32_t k0, k1;      // key
    uint32_t c0, c1, c2;  // counter words fixed per ray: ray id, scenario, stream tag
    uint32_t draw;        // block counter
    uint32_t buf[4];
    int idx;
    __device__ __forceinline__ void init(uint64_t key, uint32_t ray, uint32_t scenario, uint32_t tag) {
        k0 = (uint32_t)key; k1 = (uint32_t)(key >> 32);
        c0 = ray; c1 = scenario; c2 = tag; draw = 0; idx = 4;
    }
    __device__ __forceinline__ void refill() {
        uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = draw, a = k0, b = k1;
#pragma unroll
        for (int r = 0; r < 10; ++r) {
            uint32_t lo0 = 0xD2511F53u * x0, hi0 = __umulhi(0xD2511F53u, x0);
            uint32_t lo1 = 0xCD9E8D57u * x2, hi1 = __umulhi(0xCD9E8D57u, x2);
            uint32_t n0 = hi1 ^ x1 ^ a, n2 = hi0 ^ x3 ^ b;
            x0 = n0; x1 = lo1; x2 = n2; x3 = lo0;
            a += 0x9E3779B9u; b += 0xBB67AE85u;
        }
        buf[0] = x0; buf[1] = x1; buf[2] = x2; buf[3] = x3;
        ++draw;
        idx = 0;
    }
    __device__ __forceinline__ uint32_t next() {
        if (idx >= 4) refill();
        uint32_t v = buf[0];
        buf[0] = buf[1]; buf[1] = buf[2]; buf[2] = buf[3];
        ++idx;
        return v;
    }
};

// True for the counter-based stream: paths that only need the reference's distributions (not its
// draw sequence) may then use cheaper but equivalent samplers.
template <class S> constexpr bool kCounterStream = false;
template <> constexpr bool kCounterStream<PhiloxStream> = true;

template <class S>
__device__ __forceinline__ float uniform(S* s) { return (float)s->next() * 2.3283064e-10f; }

template <class S>
__device__ __forceinline__ double open_uniform(S* s) {
    uint32_t r = s->next();
    return ((double)r + 0.5) * 2.3283064365386962890625e-10;
}

template <class S>
__device__ __forceinline__ double uniform53(S* s) {
    uint32_t a = s->next(), b = s->next();
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * 1.11022302462515654042e-16;
}

}  // namespace clr
