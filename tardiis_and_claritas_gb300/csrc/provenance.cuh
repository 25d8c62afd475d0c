// Particle-event provenance of one photon history and its partitions over the detected rays.
//
// The reference keeps, per ray, the first and last size bin of its particle events (all events, the
// geometric ones, the wave ones), the type and deflection of its first and last event, whether the first
// event turned it back or sent it towards the source side, and whether it returned from the acrylic (or
// the headspace) after a particle event and met a particle afterwards (CLARITAS/CLARITAS.py:4625-4647,
// :4966-4979, :5005-5058); its host partitions the detected rays by them (:8063-8160, :8470-8481). Here
// the state is 16 bytes per photon slot and the partitions are counted on the device when the photon is
// scored. Nothing in it feeds a transport decision or draws a random number.
#pragma once
#include <cstdint>
#include "claritas_gb.h"

namespace clr {
namespace {

// x: first / last particle bin, first / last geometric bin (a byte each, 0xFF none)
// y: first / last wave bin (bytes 0, 1), first type (bits 16-19), last type (20-23), first event backscatter
//    (24), first event into the source hemisphere (25), acrylic return after a particle event (26), particle
//    event after such a return (27)
// z, w: deflection (deg) of the first and last event, -1 before any
constexpr unsigned kProvBack = 1u << 24, kProvHemi = 1u << 25, kProvReturn = 1u << 26, kProvAfter = 1u << 27;

__device__ __forceinline__ uint4 prov_init() {
    return make_uint4(0xFFFFFFFFu, 0x0000FFFFu, __float_as_uint(-1.0f), __float_as_uint(-1.0f));
}

__device__ __forceinline__ unsigned prov_byte(unsigned v, int k) { return (v >> (8 * k)) & 0xFFu; }
__device__ __forceinline__ unsigned prov_set_byte(unsigned v, int k, unsigned b) {
    return (v & ~(0xFFu << (8 * k))) | ((b & 0xFFu) << (8 * k));
}

// The bins, types and return flag of a particle event of bin pidx, type code (1..7), with interaction
// count ic including this event.
__device__ __forceinline__ void prov_mark(uint4& p, int ic, int type, int pidx) {
    const unsigned b = (unsigned)pidx;
    if (prov_byte(p.x, 0) == 0xFFu) p.x = prov_set_byte(p.x, 0, b);
    p.x = prov_set_byte(p.x, 1, b);
    if (type >= 1 && type <= 3) {
        if (prov_byte(p.x, 2) == 0xFFu) p.x = prov_set_byte(p.x, 2, b);
        p.x = prov_set_byte(p.x, 3, b);
    } else if (type >= 4 && type <= 7) {
        if (prov_byte(p.y, 0) == 0xFFu) p.y = prov_set_byte(p.y, 0, b);
        p.y = prov_set_byte(p.y, 1, b);
    }
    if (p.y & kProvReturn) p.y |= kProvAfter;
    p.y = (p.y & ~(0xFu << 20)) | ((unsigned)type << 20);
    if (ic == 1) p.y = (p.y & ~(0xFu << 16)) | ((unsigned)type << 16);
}

// A particle event that the photon survived, with its direction before (vin) and after (v) (:4966-4979).
__device__ __forceinline__ void prov_event(uint4& p, int ic, int type, int pidx, float vinx, float viny, float vinz,
                                           float vx, float vy, float vz) {
    const float dcos = fminf(fmaxf(o_dot(vinx, viny, vinz, vx, vy, vz), -1.0f), 1.0f);
    const float defl = acosf(dcos) * (180.0f / CLR_PI_F);
    prov_mark(p, ic, type, pidx);
    p.w = __float_as_uint(defl);
    if (ic == 1) {
        p.y = (p.y & ~(kProvBack | kProvHemi)) | (dcos < 0.0f ? kProvBack : 0u) | (vy < 0.0f ? kProvHemi : 0u);
        p.z = __float_as_uint(defl);
    }
}

// Back in the water from the acrylic or the headspace (:5009, :5019, :5028, :5049, :5058).
__device__ __forceinline__ void prov_return(uint4& p, int ic) {
    if (ic > 0) p.y |= kProvReturn;
}

// Type of a completed event from the photon's counters before (0) and after it: a coherent or a
// morphology wave event raises wcoh / wmorph (a closure can turn a geometric proposal into either), and
// the particle-surface outcome is an entry reflection, else an internal-reflection path, else a
// transmission (:4517, :4529, :4879, :4934).
__device__ __forceinline__ int prov_type(int dcoh, int dmorph, int dper, int dpir) {
    if (dcoh > 0) return 4;
    const int base = dmorph > 0 ? 5 : 1;
    return base + (dper > 0 ? 0 : (dpir > 0 ? 2 : 1));
}

__device__ __forceinline__ void prov_add(int64_t* c, unsigned long long v = 1ull) {
    atomicAdd(reinterpret_cast<unsigned long long*>(c), v);
}

// The partitions of one detected ray (native detector id ni, mirrored mi; -1 none) (:8063-8160, :8470-8481).
__device__ __forceinline__ void prov_count(clr_path_provenance& T, const uint4& p, int ic, int ni, int mi) {
    const int first_type = (int)((p.y >> 16) & 0xFu), last_type = (int)((p.y >> 20) & 0xFu);
    const float first_defl = __uint_as_float(p.z), last_defl = __uint_as_float(p.w);
    const bool valid = last_type > 0;
    const bool fav = valid && isfinite(first_defl) && first_defl >= 0.0f;
    const bool lav = valid && isfinite(last_defl) && last_defl >= 0.0f;
    const unsigned bins[CLR_PB_COUNT] = {prov_byte(p.x, 0), prov_byte(p.x, 1), prov_byte(p.x, 2), prov_byte(p.x, 3),
                                         prov_byte(p.y, 0), prov_byte(p.y, 1)};
    const int wall = ic == 0 ? CLR_WALL_ZERO_PARTICLE
                             : ((p.y & kProvReturn) ? CLR_WALL_ACRYLIC_RETURN : CLR_WALL_NO_ACRYLIC_RETURN);
    // deflection bin of the H170 histograms: edges 0, 30, ..., 150, 180.0001 deg
    auto angle_bin = [](float a) -> int {
        const double edges[CLR_N_H170_ANGLE_BINS + 1] = {0.0, 30.0, 60.0, 90.0, 120.0, 150.0, 180.0001};
        for (int b = 0; b < CLR_N_H170_ANGLE_BINS; ++b)
            if ((double)a >= edges[b] && (double)a < edges[b + 1]) return b;
        return -1;
    };
    for (int side = 0; side < 2; ++side) {
        const int id = side ? mi : ni;
        if (id < 0 || id >= CLR_N_DETECTORS) continue;
        for (int k = 0; k < CLR_PB_COUNT; ++k)
            if (bins[k] < CLR_MAX_BINS) prov_add(&T.bin_hits[k][side][bins[k]][id]);
        if (first_type > 0) prov_add(&T.first_type_hits[side][first_type][id]);
        if (last_type > 0) prov_add(&T.last_type_hits[side][last_type][id]);
        prov_add(&T.wall_hits[side][wall][id]);
        if (p.y & kProvAfter) prov_add(&T.after_return_hits[side][id]);
        if (valid && (p.y & kProvBack)) prov_add(&T.first_backscatter_hits[side][id]);
        if (valid && (p.y & kProvHemi)) prov_add(&T.first_source_hemisphere_hits[side][id]);
        if (fav) {
            atomicAdd(&T.first_angle_sum[side][id], (double)first_defl);
            prov_add(&T.first_angle_count[side][id]);
        }
        if (lav) {
            atomicAdd(&T.last_angle_sum[side][id], (double)last_defl);
            prov_add(&T.last_angle_count[side][id]);
            atomicAdd(&T.last_type_angle_sum[side][last_type][id], (double)last_defl);
            prov_add(&T.last_type_angle_count[side][last_type][id]);
        }
        if (id == 17) {
            if (lav) {
                const int b = angle_bin(last_defl);
                if (b >= 0) {
                    prov_add(&T.h170_last_angle_hits[side][0][b]);
                    prov_add(&T.h170_last_angle_hits[side][last_type][b]);
                }
            }
            if (fav) {
                const int b = angle_bin(first_defl);
                if (b >= 0) prov_add(&T.h170_first_angle_hits[side][b]);
            }
        }
    }
}

}  // namespace
}  // namespace clr
