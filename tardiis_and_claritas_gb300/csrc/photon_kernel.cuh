// Persistent photon kernel: transport + detector scoring + tallies in one launch.
//
// Replaces the reference's two launches per 250k-ray chunk (trace_kernel then
// score_detectors_kernel, CLARITAS/CLARITAS.py:7638-7847), its 129 per-ray
// output arrays (516 B/ray) and its host-side accumulation (:7849-7862):
//  * every resident warp loops until the global work queue is empty; a lane
//    whose photon finished takes the next ray id of the warp's current chunk
//    (warp-aggregated), so lanes never idle while histories of very different
//    lengths run side by side;
//  * work chunks are contiguous ray ranges of one scenario, so one launch can
//    serve hundreds of scenarios with uneven photon counts (work stealing via
//    one global atomic per chunk);
//  * detector scoring runs in the finishing lane; counts go to a per-warp
//    shared-memory tally (64-bit) that is flushed to the scenario's device
//    tally when the warp changes scenario or exits.
// Per-ray records (the reference's integer outputs) are written only by the
// kRecord instantiation used by the parity tests.
#include <cstdint>
#include <cstring>
#pragma once
#include "photon.cuh"
#include "provenance.cuh"
#include "kernels.h"

namespace clr {
namespace {  // header-only device code: internal linkage in every translation unit

// ---------------- detectors (:4237-4376) ----------------
// Bore direction table (per block, shared memory): sin/cos of (10 j)(pi/180) for j = 0..18.
struct DetTable {
    float s[20], c[20];
};
__device__ __forceinline__ void det_table_init(DetTable* t) {
    if (threadIdx.x < 19) {
        const float th = o_det_theta((int)threadIdx.x);
        t->s[threadIdx.x] = sinf(th);
        t->c[threadIdx.x] = cosf(th);
    }
}

__device__ __forceinline__ int hardware_detector(const DetTable& T, float x, float y, float z, float vx, float vy,
                                                 float vz, int mirror, float ring_in, float throat_out, float ring_out,
                                                 float throat_r, float counterbore_r) {
    if (mirror) { x = -x; vx = -vx; }
    float best_t = CLR_INF_F;
    int best = -1;
    float rth2 = throat_r * throat_r, rcb2 = counterbore_r * counterbore_r;
    for (int j = 0; j < 18; ++j) {
        float ux = T.s[j], uy = T.c[j];
        float den = vx * ux + vy * uy;
        if (den <= 1e-10f) continue;
        float pdot = x * ux + y * uy;
        float t0 = (ring_in - pdot) / den, t1 = (throat_out - pdot) / den, t2 = (ring_out - pdot) / den;
        if (!(t0 > 0.0f && t1 > t0 && t2 > t1)) continue;
        float q0x = x + t0 * vx - ring_in * ux, q0y = y + t0 * vy - ring_in * uy, q0z = z + t0 * vz;
        float q1x = x + t1 * vx - throat_out * ux, q1y = y + t1 * vy - throat_out * uy, q1z = z + t1 * vz;
        float q2x = x + t2 * vx - ring_out * ux, q2y = y + t2 * vy - ring_out * uy, q2z = z + t2 * vz;
        if (q0x * q0x + q0y * q0y + q0z * q0z <= rth2 && q1x * q1x + q1y * q1y + q1z * q1z <= rth2 &&
            q2x * q2x + q2y * q2y + q2z * q2z <= rcb2) {
            if (t0 < best_t) { best_t = t0; best = j; }
        }
    }
    return best;
}
__device__ __forceinline__ float sfh213(float phi_deg) {
    const float HALF_DEG = 10.0f, PW = 3.169925001442312f;
    float a = fabsf(phi_deg);
    if (a >= 90.0f) return 0.0f;
    float u = a / HALF_DEG;
    return 1.0f / (1.0f + powf(u, PW));
}
__device__ __forceinline__ float incidence_deg(const DetTable& T, float vx, float vy, int id, int mirror) {
    if (id < 0 || id >= 18) return -1.0f;
    if (mirror) vx = -vx;
    float ux = T.s[id], uy = T.c[id];
    float c = vx * ux + vy * uy;
    c = fminf(fmaxf(c, -1.0f), 1.0f);
    return acosf(c) * (180.0f / CLR_PI_F);
}
__device__ __forceinline__ int throat_opening(const DetTable& T, float x, float y, float z, float vx, float vy,
                                              float vz, float ring_in, float throat_r) {
    float best_t = CLR_INF_F;
    int best = -1;
    float r2 = throat_r * throat_r;
    for (int j = 0; j < 19; ++j) {
        float ux = T.s[j], uy = T.c[j];
        float den = vx * ux + vy * uy;
        if (den <= 1.0e-10f) continue;
        float pdot = x * ux + y * uy;
        float t = (ring_in - pdot) / den;
        if (t <= 0.0f) continue;
        float qx = x + t * vx - ring_in * ux, qy = y + t * vy - ring_in * uy, qz = z + t * vz;
        if (qx * qx + qy * qy + qz * qz <= r2 && t < best_t) { best_t = t; best = j; }
    }
    return best;
}
__device__ __forceinline__ float cylinder_hit(float x, float y, float vx, float vy, float R) {
    float a = vx * vx + vy * vy;
    if (a < 1e-18f) return CLR_INF_F;
    float b = x * vx + y * vy;
    float c = x * x + y * y - R * R;
    float d = b * b - a * c;
    if (d < 0.0f) return CLR_INF_F;
    float sd = sqrtf(fmaxf(d, 0.0f));
    float t1 = (-b - sd) / a, t2 = (-b + sd) / a;
    float t = CLR_INF_F;
    if (t1 > CLR_EPS_F) t = t1;
    if (t2 > CLR_EPS_F && t2 < t) t = t2;
    return t;
}
template <class S>
__device__ __noinline__ int ring_face_path(S* s, const DetTable* T, float x, float y, float z, float vx, float vy,
                                           float vz, int mirror, const clr_scene_params* P, int* bore_bounces,
                                           int* face_reflections) {
    if (mirror) { x = -x; vx = -vx; }
    *bore_bounces = 0;
    *face_reflections = 0;
    if (P->ring_face_model == 0) return -1;
    if (throat_opening(*T, x, y, z, vx, vy, vz, P->ring_in, P->throat_r) >= 0) return -1;
    for (int b = 0; b < P->max_ring_face_bounces; ++b) {
        float tr = cylinder_hit(x, y, vx, vy, P->ring_in);
        if (tr >= CLR_INF_F * 0.5f) return -1;
        x += tr * vx; y += tr * vy; z += tr * vz;
        float nx, ny;
        o_radial_normal(x, y, &nx, &ny);
        float ci = fminf(fmaxf(vx * nx + vy * ny, 0.0f), 1.0f);
        int tir = 0;
        float R = o_fresnel(ci, P->n_air, P->ring_face_n, &tir);
        if (uniform(s) >= R) return -1;
        float a, c, d;
        o_reflect(vx, vy, vz, -nx, -ny, 0.0f, &a, &c, &d);
        vx = a; vy = c; vz = d;
        (*face_reflections)++;
        x -= CLR_EPS_F * nx; y -= CLR_EPS_F * ny;
        float ta = cylinder_hit(x, y, vx, vy, P->rout);
        if (ta >= CLR_INF_F * 0.5f) return -1;
        x += ta * vx; y += ta * vy; z += ta * vz;
        o_radial_normal(x, y, &nx, &ny);
        ci = fminf(fmaxf(-o_dot(vx, vy, vz, nx, ny, 0.0f), 0.0f), 1.0f);
        R = o_fresnel(ci, P->n_air, P->n_acrylic, &tir);
        if (uniform(s) >= R) return -1;
        o_reflect(vx, vy, vz, nx, ny, 0.0f, &a, &c, &d);
        vx = a; vy = c; vz = d;
        x += CLR_EPS_F * nx; y += CLR_EPS_F * ny;
        int db = 0, det;
        if (P->detector_bore_model == 0)
            det = hardware_detector(*T, x, y, z, vx, vy, vz, 0, P->ring_in, P->throat_out, P->ring_out, P->throat_r,
                                    P->counterbore_r);
        else
            det = o_detector_collimator_path(s, x, y, z, vx, vy, vz, 0, P->ring_in, P->throat_out, P->ring_out,
                                             P->throat_r, P->counterbore_r, P->detector_bore_model, P->n_air, P->bore_n,
                                             P->max_bore_bounces, &db, T->s, T->c);
        if (det >= 0) { *bore_bounces = db; return det; }
        if (throat_opening(*T, x, y, z, vx, vy, vz, P->ring_in, P->throat_r) >= 0) return -1;
    }
    return -1;
}

// Sink addressing: counters after hw live at status[0]; map the flat CLR_OFF_* space onto the struct.
struct TallySink {
    unsigned long long* hw;    // 10*18
    double* sums;              // 8*18
    unsigned long long* tail;  // status..ic_lo
    __device__ __forceinline__ void add_u(int idx, unsigned long long v) const {
        if (idx < 10 * CLR_N_DETECTORS) atomicAdd(hw + idx, v);
        else atomicAdd(tail + (idx - CLR_OFF_STATUS), v);
    }
    __device__ __forceinline__ void add_d(int idx, double v) const { atomicAdd(sums + idx, v); }
};

template <class T>
__device__ __forceinline__ TallySink tally_sink(T* t) {
    TallySink s;
    s.hw = &t->hw[0][0];
    s.sums = &t->sums[0][0];
    s.tail = &t->status[0];
    return s;
}
__device__ __forceinline__ TallySink tally_sink_dev(DevTally* t) { return tally_sink(&t->c); }

// Sum `v` over the lanes of `grp` and let the group's leader add it (one atomic per group, not per lane).
__device__ __forceinline__ void group_add(const TallySink& sink, unsigned grp, bool leader, int idx, int v) {
    const unsigned sum = __reduce_add_sync(grp, (unsigned)v);
    if (leader && sum) sink.add_u(idx, (unsigned long long)sum);
}
// Count lanes of `grp` with `pred` and let the leader add the count.
__device__ __forceinline__ void group_count(const TallySink& sink, unsigned grp, bool leader, int idx, bool pred) {
    const unsigned n = __popc(__ballot_sync(grp, pred));
    if (leader && n) sink.add_u(idx, (unsigned long long)n);
}
// Histogram update: lanes with equal keys are merged before one atomic per distinct key.
__device__ __forceinline__ void group_hist(const TallySink& sink, unsigned grp, int base, int key, bool active) {
    const unsigned part = __ballot_sync(grp, active);
    if (active) {
        const unsigned same = __match_any_sync(part, key);
        if ((int)(threadIdx.x & 31) == __ffs(same) - 1) sink.add_u(base + key, (unsigned long long)__popc(same));
    }
}

// The reference's event-history masks of one ray (_event_history_masks, CLARITAS/CLARITAS.py:5265-5321) as
// bits in CLR_PM_* order.
__device__ __forceinline__ unsigned path_mask_bits(const Ray& r) {
    const int ic = r.ic, g = r.gic, w = r.wic, coh = r.wcoh, mor = r.wmorph;
    const int per = r.pc.entry_reflections, pir = r.pc.internal_reflections, pabs = r.pc.absorptions;
    const bool single = ic == 1, multiple = ic >= 2, surface = g > 0 || mor > 0;
    unsigned m = 0u;
    auto set = [&](int k, bool v) { m |= (v ? 1u : 0u) << k; };
    set(CLR_PM_ANY_PARTICLE, ic > 0);
    set(CLR_PM_ANY_GEOMETRIC, g > 0);
    set(CLR_PM_ANY_WAVE, w > 0);
    set(CLR_PM_ANY_COHERENT_WAVE, coh > 0);
    set(CLR_PM_ANY_MORPHOLOGY_WAVE, mor > 0);
    set(CLR_PM_ANY_ENTRY_REFLECTION, per > 0);
    set(CLR_PM_ANY_INTERNAL_REFLECTION, pir > 0);
    set(CLR_PM_BALLISTIC, ic == 0);
    set(CLR_PM_SINGLE, single);
    set(CLR_PM_SINGLE_ENTRY_REFLECTION, single && per > 0);
    set(CLR_PM_MULTIPLE, multiple);
    set(CLR_PM_ORDER_2, ic == 2);
    set(CLR_PM_ORDER_3, ic == 3);
    set(CLR_PM_ORDER_4PLUS, ic >= 4);
    set(CLR_PM_EXACTLY_ONE_GEOMETRIC, single && g == 1 && w == 0);
    set(CLR_PM_EXACTLY_ONE_WAVE, single && g == 0 && w == 1);
    set(CLR_PM_SINGLE_COHERENT_ESCAPE, single && coh == 1);
    set(CLR_PM_SINGLE_ENTRY_REFLECTION_ESCAPE, single && per > 0);
    set(CLR_PM_SINGLE_INTERNAL_REFLECTION_ESCAPE, single && pir > 0);
    set(CLR_PM_SINGLE_TRANSMISSION_ESCAPE, single && surface && per == 0 && pir == 0 && pabs == 0);
    set(CLR_PM_MIXED_GEOMETRIC_WAVE, multiple && g > 0 && w > 0);
    set(CLR_PM_GEOMETRIC_ONLY_MULTIPLE, multiple && g > 0 && w == 0);
    set(CLR_PM_WAVE_ONLY_MULTIPLE, multiple && g == 0 && w > 0);
    set(CLR_PM_MULTIPLE_ENTRY_REFLECTION, multiple && per > 0);
    set(CLR_PM_MULTIPLE_INTERNAL_REFLECTION, multiple && pir > 0);
    return m;
}

// The event-history masks and acrylic-reflection order of a detected ray (native id ni, mirrored mi), and its
// provenance partitions when they are counted. One out-of-line copy shared by the kernels that score.
__device__ __noinline__ void path_partitions_more(PathDiag& pd, clr_path_provenance* pt, const Ray& r,
                                                  const uint4* prov, int ni, int mi) {
    const unsigned masks = path_mask_bits(r);
    const int acr = r.cir + r.cor + r.bir + r.bor, ai = acr < 4 ? acr : 4;
    for (int side = 0; side < 2; ++side) {
        const int id = side ? mi : ni;
        if (id < 0) continue;
        atomicAdd(&pd.acrylic_order[side][ai][id], 1ull);
        for (unsigned m = masks; m; m &= m - 1u) atomicAdd(&pd.masks[side][__ffs(m) - 1][id], 1ull);
    }
    if (pt) prov_count(*pt, prov ? *prov : prov_init(), r.ic, ni, mi);
}

// Score finished histories and add them to the scenario tallies (:4390-4436, tallies :7849-7862,
// per-ray statistics :8483-8508 and :8665-8735). Called by every lane whose photon finished in this
// iteration; lanes are grouped by scenario so the frequent counters are reduced across the group first.
template <class Mode>
__device__ __forceinline__ void finish_ray(const DevScene& D, const DetTable& T, const Ray& r, uint32_t gid,
                                           int sid, int home, WarpTally* wt, DevTally* tallies,
                                           clr_ray_record* rec, const uint4* prov = nullptr) {
    const clr_scene_params& P = D.P;
    const int lane = threadIdx.x & 31;
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, sid);
    const bool leader = lane == __ffs(grp) - 1;
    const TallySink sink = (sid == home) ? tally_sink(wt) : tally_sink_dev(tallies + sid);
    int ni = -1, mi = -1, nb = 0, mb = 0, nfb = 0, mfb = 0;
    const int st = r.st;
    if (st == 1 && isfinite(r.x) && isfinite(r.y) && isfinite(r.z) && isfinite(r.vx) && isfinite(r.vy) &&
        isfinite(r.vz)) {
        const float x = r.x, y = r.y, z = r.z, vx = r.vx, vy = r.vy, vz = r.vz;
        if (P.detector_bore_model == 0 && P.ring_face_model == 0) {
            ni = hardware_detector(T, x, y, z, vx, vy, vz, 0, P.ring_in, P.throat_out, P.ring_out, P.throat_r,
                                   P.counterbore_r);
            mi = hardware_detector(T, x, y, z, vx, vy, vz, 1, P.ring_in, P.throat_out, P.ring_out, P.throat_r,
                                   P.counterbore_r);
        } else {
            typename Mode::Stream sN, sM;
            Mode::detector_streams(D, gid, &sN, &sM);
            if (P.detector_bore_model == 0) {
                ni = hardware_detector(T, x, y, z, vx, vy, vz, 0, P.ring_in, P.throat_out, P.ring_out, P.throat_r,
                                       P.counterbore_r);
                mi = hardware_detector(T, x, y, z, vx, vy, vz, 1, P.ring_in, P.throat_out, P.ring_out, P.throat_r,
                                       P.counterbore_r);
            } else {
                ni = o_detector_collimator_path(&sN, x, y, z, vx, vy, vz, 0, P.ring_in, P.throat_out, P.ring_out,
                                                P.throat_r, P.counterbore_r, P.detector_bore_model, P.n_air, P.bore_n,
                                                P.max_bore_bounces, &nb, T.s, T.c);
                mi = o_detector_collimator_path(&sM, x, y, z, vx, vy, vz, 1, P.ring_in, P.throat_out, P.ring_out,
                                                P.throat_r, P.counterbore_r, P.detector_bore_model, P.n_air, P.bore_n,
                                                P.max_bore_bounces, &mb, T.s, T.c);
            }
            if (ni < 0 && P.ring_face_model != 0) ni = ring_face_path(&sN, &T, x, y, z, vx, vy, vz, 0, &P, &nb, &nfb);
            if (mi < 0 && P.ring_face_model != 0) mi = ring_face_path(&sM, &T, x, y, z, vx, vy, vz, 1, &P, &mb, &mfb);
        }
        // detector hits are rare and spread over 18 channels: per-lane atomics
        const double w = (double)r.w;
        if (ni >= 0) {
            sink.add_u(CLR_OFF_HW(0, ni), 1ull);
            sink.add_u(CLR_OFF_HW((nb > 0 || nfb > 0) ? 4 : 2, ni), 1ull);
            if (nfb > 0) sink.add_u(CLR_OFF_HW(6, ni), 1ull);
            float phi = incidence_deg(T, vx, vy, ni, 0);
            if (phi >= 0.0f && isfinite(phi)) {
                float resp = (P.photodiode_model == 0) ? 1.0f : sfh213(phi);
                sink.add_d(0 * CLR_N_DETECTORS + ni, (double)resp * w);
                sink.add_d(2 * CLR_N_DETECTORS + ni, (double)phi);
            }
            sink.add_d(4 * CLR_N_DETECTORS + ni, w);
            sink.add_d(6 * CLR_N_DETECTORS + ni, w * w);
        }
        if (mi >= 0) {
            sink.add_u(CLR_OFF_HW(1, mi), 1ull);
            sink.add_u(CLR_OFF_HW((mb > 0 || mfb > 0) ? 5 : 3, mi), 1ull);
            if (mfb > 0) sink.add_u(CLR_OFF_HW(7, mi), 1ull);
            float phi = incidence_deg(T, vx, vy, mi, 1);
            if (phi >= 0.0f && isfinite(phi)) {
                float resp = (P.photodiode_model == 0) ? 1.0f : sfh213(phi);
                sink.add_d(1 * CLR_N_DETECTORS + mi, (double)resp * w);
                sink.add_d(3 * CLR_N_DETECTORS + mi, (double)phi);
            }
            sink.add_d(5 * CLR_N_DETECTORS + mi, w);
            sink.add_d(7 * CLR_N_DETECTORS + mi, w * w);
        }
        // particle-path partitions of the detected ray (one set per detector id it reaches); the less frequent
        // ones (event-history masks, acrylic order, provenance) are counted out of line, so that the scoring
        // code every finishing photon runs through stays as small as it was without them
        {
            PathDiag& pd = tallies[sid].pd;
            const int oi = r.ic < 5 ? r.ic : 5, gi = r.gic < 5 ? r.gic : 5;
            const int pv[CLR_N_PATH_SUMS] = {r.ic, r.gic, r.wic, r.wcoh, r.wmorph, r.pc.entry_reflections,
                                            r.pc.internal_reflections};
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int id = side ? mi : ni;
                if (id < 0) continue;
                atomicAdd(&pd.order[side][oi][id], 1ull);
                atomicAdd(&pd.geom_order[side][gi][id], 1ull);
#pragma unroll
                for (int k = 0; k < CLR_N_PATH_SUMS; ++k)
                    if (pv[k] > 0) atomicAdd(&pd.sums[k][side][id], (unsigned long long)pv[k]);
            }
            if (ni >= 0 || mi >= 0) path_partitions_more(pd, D.prov, r, prov, ni, mi);
        }
        // legacy angular windows (:4429-4434)
        for (int mirror = 0; mirror < 2; ++mirror) {
            float xx = mirror ? -x : x;
            float ang = atan2f(xx, y) * (180.0f / CLR_PI_F);
            if (ang < 0.0f) ang += 360.0f;
            if (ang < 0.0f || ang > 180.0f) continue;
            for (int j = 0; j < 18; ++j) {
                float deg = 10.0f * j;
                if (r.ic <= 0 && deg >= 90.0f) continue;
                if (fabsf(ang - deg) <= P.legacy_accept_deg) sink.add_u(CLR_OFF_HW(mirror ? 9 : 8, j), 1ull);
            }
        }
    }
    // frequent counters: reduced over the scenario group, one atomic per group
    group_hist(sink, grp, CLR_OFF_STATUS, (st >= 0 && st < CLR_N_STATUS) ? st : 0, st >= 0 && st < CLR_N_STATUS);
    group_hist(sink, grp, CLR_OFF_FAIL, r.pf, r.pf >= 0 && r.pf < CLR_N_FAILURE_CODES);
    const int ev[22] = {r.ic, r.gic, r.wic, r.wcoh, r.wmorph, r.pc.reflections, r.pc.entry_reflections,
                        r.pc.internal_reflections, r.pc.absorptions, r.cir, r.cor, r.ctir, r.tr, r.ttir, r.bir,
                        r.bor, r.btir, r.sbi, r.sbr, r.entered, r.steps, r.nulls};
    const bool any_ev = __any_sync(grp, r.ic | r.cir | r.cor | r.ctir | r.tr | r.bir | r.bor | r.sbi | r.entered |
                                            r.steps | r.nulls | r.pc.reflections | r.pc.absorptions);
    if (any_ev) {
#pragma unroll
        for (int k = 0; k < 22; ++k) group_add(sink, grp, leader, CLR_OFF_EV + k, ev[k]);
    }
    if (leader) sink.add_u(CLR_OFF_DONE, (unsigned long long)__popc(grp));
    if (r.pf != 0) sink.add_u(CLR_OFF_SUB + CLR_SUBCODE_INDEX(r.pfs), 1ull);
    group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_SOURCE_ACCEPTED, st != 3);
    group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_SOURCE_DIRECT, st != 3 && r.sbr == 0);
    group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_SOURCE_REFLECTED, st != 3 && r.sbr != 0);
    group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_VALID_AIR, st == 1 && isfinite(r.x) && isfinite(r.vx));
    group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_TRAPPED, st == 8);
    const bool ent = r.entered != 0;
    if (__any_sync(grp, ent)) {
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_ENTERED, ent);
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_BALLISTIC, ent && r.ic == 0);
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_ENTRY_REFLECTED, ent && r.pc.entry_reflections > 0);
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_INTERNAL_REFLECTED, ent && r.pc.internal_reflections > 0);
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_ABSORBED, ent && r.pc.absorptions > 0);
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_CELL_TIR, ent && r.ctir > 0);
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_TOP_TIR, ent && r.ttir > 0);
        group_count(sink, grp, leader, CLR_OFF_RF + CLR_RF_BOTTOM_TIR, ent && r.btir > 0);
        const int es[16] = {r.ic, r.gic, r.wic, r.wcoh, r.wmorph, r.pc.reflections, r.cir, r.cor, r.tr, r.bir, r.bor,
                            r.ctir, r.ttir, r.btir, r.pc.entry_reflections, r.pc.internal_reflections};
#pragma unroll
        for (int k = 0; k < 16; ++k) group_add(sink, grp, leader, CLR_OFF_ES + k, ent ? es[k] : 0);
        const int ic = r.ic < 0 ? 0 : r.ic;
        group_hist(sink, grp, CLR_OFF_ICLO, ic < 64 ? ic : 0, ent && ic < 64);
        if (ent && ic >= 64) atomicAdd(tallies[sid].ic_hi + (ic < CLR_IC_HIST - 1 ? ic : CLR_IC_HIST - 1), 1ull);
    }
    if (rec) {
        clr_ray_record o;
        o.status = st;
        o.interaction_count = r.ic; o.geometric = r.gic; o.wave = r.wic; o.coherent = r.wcoh; o.morphology = r.wmorph;
        o.particle_reflections = r.pc.reflections; o.entry_reflections = r.pc.entry_reflections;
        o.internal_reflections = r.pc.internal_reflections; o.absorptions = r.pc.absorptions;
        o.cell_inner_reflections = r.cir; o.cell_outer_reflections = r.cor; o.cell_tir = r.ctir;
        o.top_reflections = r.tr; o.top_tir = r.ttir; o.bottom_inner_reflections = r.bir;
        o.bottom_outer_reflections = r.bor; o.bottom_tir = r.btir;
        o.source_bore_interactions = r.sbi; o.source_bore_reflections = r.sbr; o.entered_water = r.entered;
        o.failure_code = r.pf; o.failure_subcode = r.pfs;
        o.native_id = ni; o.mirror_id = mi; o.native_bounces = nb; o.mirror_bounces = mb;
        const float nanf_ = __int_as_float(0x7fc00000);
        o.air_x = st == 1 ? r.x : nanf_; o.air_y = st == 1 ? r.y : nanf_; o.air_z = st == 1 ? r.z : nanf_;
        o.air_vx = st == 1 ? r.vx : nanf_; o.air_vy = st == 1 ? r.vy : nanf_; o.air_vz = st == 1 ? r.vz : nanf_;
        o.water_path = r.wp; o.acrylic_path = r.ap;
        *rec = o;
    }
}

// ---------------- random-stream modes ----------------
struct XorMode {
    using Stream = XorStream;
    struct Lane {
        XorStream st, opt, src;
        __device__ __forceinline__ XorStream* transport() { return &st; }
        __device__ __forceinline__ XorStream* optics() { return &opt; }
        __device__ __forceinline__ XorStream* source() { return &src; }
    };
    // per-ray seeding of the three transport streams (:4612)
    __device__ __forceinline__ static void seed(const DevScene& D, uint32_t gid, Lane& L) {
        L.st.s = D.seed0 + gid * 74729u + 13u;
        L.opt.s = D.seed1 + gid * 104729u + 29u;
        L.src.s = D.seed2 + gid * 130363u + 43u;
    }
    // detector streams (:4396-4397)
    __device__ __forceinline__ static void detector_streams(const DevScene& D, uint32_t gid, XorStream* n, XorStream* m) {
        n->s = D.det_seed + gid * 2246822519u + 3266489917u;
        m->s = D.det_seed + gid * 3266489917u + 668265263u;
    }
};
struct PhiloxMode {
    using Stream = PhiloxStream;
    struct Lane {
        PhiloxStream p;
        __device__ __forceinline__ PhiloxStream* transport() { return &p; }
        __device__ __forceinline__ PhiloxStream* optics() { return &p; }
        __device__ __forceinline__ PhiloxStream* source() { return &p; }
    };
    __device__ __forceinline__ static void seed(const DevScene& D, uint32_t gid, Lane& L) {
        L.p.init(D.philox_key, gid, D.scenario_id, 0u);
    }
    __device__ __forceinline__ static void detector_streams(const DevScene& D, uint32_t gid, PhiloxStream* n,
                                                            PhiloxStream* m) {
        n->init(D.philox_key, gid, D.scenario_id, 1u);
        m->init(D.philox_key, gid, D.scenario_id, 2u);
    }
};

__device__ __forceinline__ void flush_warp_tally(WarpTally* t, DevTally* dst, int lane) {
    unsigned long long* su = &t->hw[0][0];
    unsigned long long* du = &dst->c.hw[0][0];
    for (int i = lane; i < 10 * CLR_N_DETECTORS; i += 32) {
        unsigned long long v = su[i];
        if (v) { atomicAdd(du + i, v); su[i] = 0ull; }
    }
    double* sd = &t->sums[0][0];
    double* dd = &dst->c.sums[0][0];
    for (int i = lane; i < 8 * CLR_N_DETECTORS; i += 32) {
        double v = sd[i];
        if (v != 0.0) { atomicAdd(dd + i, v); sd[i] = 0.0; }
    }
    unsigned long long* su2 = &t->status[0];
    unsigned long long* du2 = &dst->c.status[0];
    for (int i = lane; i < CLR_TALLY_TAIL; i += 32) {
        unsigned long long v = su2[i];
        if (v) { atomicAdd(du2 + i, v); su2[i] = 0ull; }
    }
    __syncwarp();
}

// lanes that must wait in ENTRY/WATER before the warp stops drawing new photons
constexpr int kDeepThreshold = 24;

template <class Mode, bool kRecord, bool kWeighted>
__global__ void __launch_bounds__(CLR_TRACE_THREADS) photon_kernel(const DevScene* __restrict__ scenes,
                                                                   const long long* __restrict__ chunk_begin,
                                                                   int n_scen, long long n_chunks, int chunk_rays,
                                                                   unsigned long long* __restrict__ work,
                                                                   DevTally* __restrict__ tallies,
                                                                   clr_ray_record* __restrict__ records) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpTally* wt = reinterpret_cast<WarpTally*>(smem_raw) + (threadIdx.x >> 5);
    __shared__ DetTable det;
    det_table_init(&det);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    {
        unsigned long long* p = reinterpret_cast<unsigned long long*>(wt);
        for (int i = lane; i < (int)(sizeof(WarpTally) / 8); i += 32) p[i] = 0ull;
        __syncwarp();
    }
    int home = -1;
    long long cur_pos = 0, cur_end = 0;  // ray range of the warp's current chunk (within scenario cur_sid)
    int cur_sid = 0;
    bool exhausted = false;
    bool have = false;
    int sid = 0;
    uint32_t gid = 0;
    long long rid = 0;
    Ray r;
    typename Mode::Lane L;
    ray_reset(r);
    const unsigned FULL = 0xffffffffu;
    const unsigned lt_mask = (1u << lane) - 1u;
    unsigned long long sched_it[3] = {0, 0, 0}, sched_lanes[3] = {0, 0, 0}, sched_cyc[4] = {0, 0, 0, 0};
    while (true) {
        // refill idle lanes from the warp's chunk, fetching new chunks as needed
        unsigned need = __ballot_sync(FULL, !have);
        while (need && !exhausted) {
            if (cur_pos >= cur_end) {
                long long c = 0;
                if (lane == 0) c = (long long)atomicAdd(work, 1ull);
                c = __shfl_sync(FULL, c, 0);
                if (c >= n_chunks) { exhausted = true; break; }
                int lo = 0, hi = n_scen - 1;
                while (lo < hi) {  // last scenario whose first chunk is <= c
                    int mid = (lo + hi + 1) >> 1;
                    if (chunk_begin[mid] <= c) lo = mid; else hi = mid - 1;
                }
                cur_sid = lo;
                cur_pos = (c - chunk_begin[lo]) * (long long)chunk_rays;
                long long nr = scenes[lo].n_rays;
                cur_end = cur_pos + chunk_rays < nr ? cur_pos + chunk_rays : nr;
                if (cur_sid != home) {
                    if (home >= 0) flush_warp_tally(wt, tallies + home, lane);
                    home = cur_sid;
                }
                continue;
            }
            const long long avail = cur_end - cur_pos;
            const int rank = __popc(need & lt_mask);
            const bool mine = ((need >> lane) & 1u) && rank < avail;
            if (mine) {
                sid = cur_sid;
                rid = cur_pos + rank;
                const DevScene& D = scenes[sid];
                gid = D.ray_offset + (uint32_t)rid;
                Mode::seed(D, gid, L);
                ray_reset(r);
                have = true;
            }
            const int taken = __popc(need) < avail ? __popc(need) : (int)avail;
            cur_pos += taken;
            need = __ballot_sync(FULL, !have);
        }
        // Phase-coherent scheduling: the warp runs one phase per iteration so the FP64-heavy phases
        // execute with many lanes converged. SOURCE keeps refilling lanes until most lanes wait in a
        // deeper phase (or the work queue is empty); then the deeper phase with the most lanes runs.
        const unsigned m_src = __ballot_sync(FULL, have && r.phase == PHASE_SOURCE);
        const unsigned m_ent = __ballot_sync(FULL, have && r.phase == PHASE_ENTRY);
        const unsigned m_wat = __ballot_sync(FULL, have && r.phase == PHASE_WATER);
        if (!(m_src | m_ent | m_wat)) break;
        const int n_src = __popc(m_src), n_ent = __popc(m_ent), n_wat = __popc(m_wat);
        int pick;
        if (n_src && !exhausted && n_ent + n_wat < kDeepThreshold) pick = PHASE_SOURCE;
        else if (n_ent >= n_wat && n_ent >= n_src) pick = PHASE_ENTRY;
        else if (n_wat >= n_src) pick = PHASE_WATER;
        else pick = PHASE_SOURCE;
        const long long t0 = clock64();
        if (lane == 0) { sched_it[pick]++; sched_lanes[pick] += (unsigned)__popc(pick == PHASE_SOURCE ? m_src : (pick == PHASE_ENTRY ? m_ent : m_wat)); }
        if (have && r.phase == pick) {
            const DevScene& D = scenes[sid];
            bool done;
            if (pick == PHASE_SOURCE) done = source_segment(D, r, L.source());
            else if (pick == PHASE_ENTRY) done = entry_segment(D, r, L.transport());
            else done = water_step<typename Mode::Stream, kWeighted>(D, r, L.transport(), L.optics(),
                                                                      (sid == home) ? &wt->cstats[0] : &tallies[sid].c.cstats[0],
                                                                      gid);
            if (done) {
                const long long tf = clock64();
                finish_ray<Mode>(D, det, r, gid, sid, home, wt, tallies, kRecord ? records + rid : nullptr);
                have = false;
                if (lane == __ffs(__activemask()) - 1) sched_cyc[3] += (unsigned long long)(clock64() - tf);
            }
        }
        __syncwarp();
        if (lane == 0) sched_cyc[pick] += (unsigned long long)(clock64() - t0);
    }
    if (lane == 0) {
        for (int k = 0; k < 3; ++k) {
            atomicAdd(&tallies[0].sched[k], sched_it[k]);
            atomicAdd(&tallies[0].sched[4 + k], sched_lanes[k]);
            atomicAdd(&tallies[0].sched[8 + k], sched_cyc[k]);
        }
        atomicAdd(&tallies[0].sched[11], sched_cyc[3]);
    }
    __syncwarp();
    if (home >= 0) flush_warp_tally(wt, tallies + home, lane);
}

template <class Mode, bool kRecord, bool kWeighted>
cudaError_t launch_t(const LaunchArgs& a) {
    auto k = photon_kernel<Mode, kRecord, kWeighted>;
    const int smem = (CLR_TRACE_THREADS / 32) * (int)sizeof(WarpTally);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k<<<a.grid, CLR_TRACE_THREADS, smem, a.stream>>>(a.scenes, a.chunk_begin, a.n_scen, a.n_chunks, a.chunk_rays,
                                                    a.work, a.tallies, a.records);
    return cudaGetLastError();
}

template <class Mode, bool kRecord, bool kWeighted>
int occupancy_t() {
    int blocks = 0;
    const int smem = (CLR_TRACE_THREADS / 32) * (int)sizeof(WarpTally);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, photon_kernel<Mode, kRecord, kWeighted>, CLR_TRACE_THREADS,
                                                  smem);
    return blocks;
}

}  // namespace
}  // namespace clr
