// Wavefront photon engine: one short kernel per stage of a history, photons parked in HBM between stages.
//
// The persistent photon kernel (photon_kernel.cuh) runs a whole history per lane. Its code is large and
// its lanes diverge at every event, so on GB300 it is bound by instruction fetch and divergence, not by
// any pipe. Here every photon lives in a slot of a resident pool (Ray state, random stream, ids), and
// each stage of a history is its own kernel that processes a queue of slots:
//
//   GEN    free slots: draw photons, run the source segment; photons rejected by the collimator are
//          scored at once (most photons), accepted ones go to ENTRY
//   ENTRY  air gap, outer wall, acrylic, headspace               -> FLIGHT or FIN
//   FLIGHT water flights with the cheap outcomes inline (null collisions, coherent Mie scattering,
//          Fresnel reflections at the surface and the wall)     -> an event queue, FIN, or FLIGHT
//   COND, GEOM, MORPH   particle events (conditional closure, geometric sphere, spheroid); a long
//          closure runs in bounded pieces through the COND queue
//   TOP, BOTTOM, SIDE   transmission into the headspace, the bottom disc, the acrylic wall
//                                                                -> FLIGHT, FIN or ACRYL
//   ACRYL  the next bounded piece of a long traversal of the acrylic solid
//   FIN    detector scoring and tallies; the slot returns to the free queue
//
// A pass is one CUDA graph: a begin kernel, then the eleven stage kernels as independent branches, so
// the latency-bound stages (long FP64 chains in the acrylic, rare events) overlap with the
// throughput-bound ones instead of idling the GPU behind them. Queues are ring buffers of slot ids
// with monotonically increasing 32-bit head/tail counters; the ring holds twice the pool, so a window
// being consumed and the pushes that land behind it never collide (wrap-around is exact because the
// ring size is a power of two). The begin kernel retires the previous pass's windows and snapshots
// every queue: during the pass each stage consumes [head, snap) of its queue while all pushes land at
// or after the tail, so no slot is handled twice in a pass and no stage reads an entry still being
// written. Pushes are aggregated per warp and queue. Rare stages skip passes until a batch is queued.
//
// Within each stage the device functions, arithmetic and per-ray draw order are the persistent
// kernel's (they are the same functions), so per-ray results in the xorshift parity mode are
// identical to the reference's whichever engine runs.
#pragma once
#include <algorithm>
#include <cstddef>
#include "photon_kernel.cuh"

namespace clr {
namespace {

enum : int { WQ_FREE = 0, WQ_ENTRY, WQ_FLIGHT, WQ_COND, WQ_GEOM, WQ_MORPH, WQ_TOP, WQ_BOTTOM, WQ_SIDE, WQ_ACRYL,
             WQ_FIN };
static_assert(WQ_FIN + 1 == CLR_WQ_COUNT, "queue count");
static_assert(CLR_WQ_COUNT == CLR_N_STAGES, "one engine setting per stage queue");

constexpr int kWaveThreads = 256;
// Engine settings (WaveLaunch, from clr_engine_config; defaults CLR_ENGINE_DEFAULT_*, chosen per GPU and
// scene by the tuner): flight_steps water flights per FLIGHT visit before the photon is re-queued (bounds
// lane imbalance in a warp); tail_photons, the photons in flight at or below which, once every photon is
// drawn, the passes stop and one tail kernel runs each remaining photon to its end in a single thread (the
// longest histories, thousands of flights in optically dense scenes, then cost one step each instead of a
// pass each); rare_batch, the queue length at which a rare stage runs (below); acr_budget, the bounces per
// piece of an acrylic traversal; pass_batch and stage_blocks on the host side.
constexpr int kTailThreads = 128;
// Rare stages (few photons per pass, long serial work per photon) run only when their queue holds
// rare_batch photons, after kMaxSkips passes, or while the pool drains.
constexpr unsigned kMaxSkips = 8;
__host__ __device__ constexpr bool stage_is_rare(int q) {
    return q == WQ_MORPH || q == WQ_TOP || q == WQ_BOTTOM;
}
// minimum resident blocks per SM (register budget) per stage
__host__ __device__ constexpr int stage_min_blocks(int q) { return q == WQ_COND ? 1 : 2; }
// acrylic bounces per visit of SIDE, BOTTOM and ACRYL while photons are drawn (acr_budget; a traversal can
// take 16384), all of them once every photon has been drawn
static_assert(CLR_ENGINE_DEFAULT_ACR_BUDGET % (2 * kTrapWindow) == 0 &&
                  CLR_ENGINE_ACR_BUDGET_STEP % (2 * kTrapWindow) == 0,
              "traversal pieces start where no trapped-orbit window spans them");
// closure trials per visit: a few inline in GEOM (most closures end in one or two), more per COND visit
// (a closure can take 16384 trials, e.g. when no sampled sphere fits)
constexpr int kCondInline = 8;
constexpr int kCondBudget = 512;
// trials per COND visit when a whole warp runs them (counter-based stream): 32 warp steps
constexpr int kCondWarpBudget = 1024;

template <class Mode>
struct WavePool {
    Ray* ray;
    typename Mode::Lane* lane;
    SlotMeta* meta;
};

template <class Mode>
__device__ __forceinline__ WavePool<Mode> wave_pool(const WaveLaunch& w) {
    WavePool<Mode> p;
    p.ray = reinterpret_cast<Ray*>(w.ray);
    p.lane = reinterpret_cast<typename Mode::Lane*>(w.lane);
    p.meta = w.meta;
    return p;
}

// ring of queue q (2 * cap entries)
__device__ __forceinline__ uint32_t* wave_ring(const WaveLaunch& w, int q) { return w.qbuf + (size_t)q * 2u * w.cap; }
__device__ __forceinline__ unsigned wave_mask(const WaveLaunch& w) { return 2u * w.cap - 1u; }

// Warp-aggregated push of `slot` to queue `q` (q < 0: no push). Called by all 32 lanes.
__device__ __forceinline__ void wave_push(const WaveLaunch& w, int q, uint32_t slot) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned grp = __match_any_sync(FULL, q);
    const int leader = __ffs(grp) - 1;
    unsigned base = 0;
    if (lane == leader && q >= 0) base = atomicAdd(&w.ctl->tail[q], (unsigned)__popc(grp));
    base = __shfl_sync(FULL, base, leader);
    if (q >= 0) {
        const unsigned pos = base + (unsigned)__popc(grp & ((1u << lane) - 1u));
        wave_ring(w, q)[pos & wave_mask(w)] = slot;
    }
}

// Begin of a pass (one thread): retire the windows of the previous pass, decide which stages run, take
// the windows of this pass, and publish whether any photon is still in flight or undrawn.
__global__ void wave_begin_kernel(WaveLaunch w) {
    if (threadIdx.x | blockIdx.x) return;
    WaveCtl* c = w.ctl;
    const bool drawing = c->next_photon < c->total_photons;
    unsigned pending = 0;
    for (int q = 0; q < CLR_WQ_COUNT; ++q) {
        c->head[q] = c->snap[q];
        const unsigned n = c->tail[q] - c->head[q];
        if (q != WQ_FREE) pending |= n;
        bool run = n > 0;
        if (q == WQ_FREE) run = run && drawing;
        else if (stage_is_rare(q) && n < w.rare_batch && c->skips[q] < kMaxSkips && drawing) run = false;
        c->snap[q] = run ? c->tail[q] : c->head[q];
        c->skips[q] = run ? 0u : c->skips[q] + (n > 0 ? 1u : 0u);
        c->claim[q] = 0u;
    }
    c->live = (pending != 0u || drawing) ? 1u : 0u;
    c->passes++;
    // photons still in flight after this pass at the most (every queue but FREE), once all are drawn
    unsigned in_flight = 0;
    for (int q = 1; q < CLR_WQ_COUNT; ++q) in_flight += c->tail[q] - c->head[q];
    c->tail_ready = (!drawing && in_flight <= w.tail_photons) ? 1u : 0u;
    c->in_flight = in_flight;
}

// Per-block conditional-closure statistics for scenario 0 (others go straight to the device tally).
// The last warp of the block to finish flushes them, so warps leave without waiting at a barrier.
struct BlockStats {
    unsigned long long cs[CLR_N_CONDITIONAL_STATS];
    unsigned warps_done;
};
__device__ __forceinline__ void block_stats_init(BlockStats* b) {
    if (threadIdx.x < CLR_N_CONDITIONAL_STATS) b->cs[threadIdx.x] = 0ull;
    if (threadIdx.x == 0) b->warps_done = 0u;
    __syncthreads();
}
__device__ __forceinline__ void warp_done(BlockStats* b, DevTally* t, int q, unsigned long long items) {
    const int lane = threadIdx.x & 31;
    const unsigned long long sum = __reduce_add_sync(0xffffffffu, (unsigned)items);
    if (lane == 0 && sum) atomicAdd(&t[0].sched[q], sum);
    __threadfence_block();
    unsigned done = 0;
    if (lane == 0) done = atomicAdd(&b->warps_done, 1u);
    done = __shfl_sync(0xffffffffu, done, 0);
    if (done == (blockDim.x >> 5) - 1) {
        __threadfence_block();
        if (lane < CLR_N_CONDITIONAL_STATS) {
            const unsigned long long v = atomicAdd(&b->cs[lane], 0ull);
            if (v) atomicAdd(&t[0].c.cstats[lane], v);
        }
    }
}

// Next chunk of 32 entries of this pass's window for the calling warp (all lanes call). Warps claim
// chunks dynamically, so a warp that drew short histories takes more chunks than one that drew long ones.
__device__ __forceinline__ unsigned wave_claim(const WaveLaunch& w, int q) {
    unsigned b = 0;
    if ((threadIdx.x & 31) == 0) b = atomicAdd(&w.ctl->claim[q], 32u);
    return __shfl_sync(0xffffffffu, b, 0);
}

// This pass's window of queue q, iterated in warp-uniform chunks of 32 entries.
struct WaveWindow {
    unsigned head, n;
};
__device__ __forceinline__ WaveWindow wave_window(const WaveLaunch& w, int q) {
    WaveWindow win;
    win.head = w.ctl->head[q];
    win.n = w.ctl->snap[q] - win.head;
    return win;
}

__device__ __forceinline__ bool wave_drawing(const WaveLaunch& w) {
    return *(volatile unsigned long long*)&w.ctl->next_photon < w.ctl->total_photons;
}

__device__ __forceinline__ void photon_of(const WaveLaunch& w, unsigned long long p, int* sid, long long* rid) {
    int lo = 0, hi = w.n_scen - 1;
    while (lo < hi) {  // last scenario whose first photon is <= p
        const int mid = (lo + hi + 1) >> 1;
        if ((unsigned long long)w.ray_begin[mid] <= p) lo = mid; else hi = mid - 1;
    }
    *sid = lo;
    *rid = (long long)(p - (unsigned long long)w.ray_begin[lo]);
}

__device__ __forceinline__ void warp_tally_zero(WarpTally* wt, int lane) {
    unsigned long long* p = reinterpret_cast<unsigned long long*>(wt);
    for (int i = lane; i < (int)(sizeof(WarpTally) / 8); i += 32) p[i] = 0ull;
}

// ---------------- GEN: fill free slots with photons that pass the source collimator ----------------
template <class Mode>
__global__ void __launch_bounds__(kWaveThreads) wave_gen_kernel(WaveLaunch w) {
    const WaveWindow win = wave_window(w, WQ_FREE);
    if (win.n == 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpTally* wt = reinterpret_cast<WarpTally*>(smem_raw) + (threadIdx.x >> 5);
    __shared__ DetTable det;
    det_table_init(&det);
    const int lane = threadIdx.x & 31;
    warp_tally_zero(wt, lane);
    __syncthreads();
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    const uint32_t* ring = wave_ring(w, WQ_FREE);
    const unsigned FULL = 0xffffffffu;
    bool out = !wave_drawing(w);
    unsigned long long drawn = 0;
    int home = -1;  // scenario whose counts this warp keeps in shared memory (that of its first photon)
    // A photon rejected at the collimator (most of them) changes only its end-status, failure-code-0 and
    // done counters and the source-bore counters: without per-ray records those are counted in registers
    // and added once per warp instead of running the whole scoring routine per photon.
    const bool count_rejects = !w.records && !w.prov_rec;
    unsigned rej = 0, rej_sbi = 0, rej_sbr = 0;
    for (unsigned base = wave_claim(w, WQ_FREE); base < win.n && !__all_sync(FULL, out); base = wave_claim(w, WQ_FREE)) {
        const unsigned i = base + lane;
        const bool valid = i < win.n;
        const uint32_t slot = valid ? ring[(win.head + i) & wave_mask(w)] : 0u;
        bool filled = false;
        while (true) {
            const unsigned need = __ballot_sync(FULL, valid && !filled && !out);
            if (!need) break;
            unsigned long long b0 = 0;
            if (lane == __ffs(need) - 1) b0 = atomicAdd(&w.ctl->next_photon, (unsigned long long)__popc(need));
            b0 = __shfl_sync(FULL, b0, __ffs(need) - 1);
            if (home < 0 && b0 < w.ctl->total_photons) {
                int hs;
                long long hr;
                photon_of(w, b0, &hs, &hr);
                home = hs;
            }
            if ((need >> lane) & 1u) {
                const unsigned long long p = b0 + (unsigned long long)__popc(need & ((1u << lane) - 1u));
                if (p >= w.ctl->total_photons) {
                    out = true;
                } else {
                    int sid;
                    long long rid;
                    photon_of(w, p, &sid, &rid);
                    const DevScene& D = w.scenes[sid];
                    const uint32_t gid = D.ray_offset + (uint32_t)rid;
                    typename Mode::Lane L;
                    Mode::seed(D, gid, L);
                    Ray r;
                    ray_reset(r);
                    drawn++;
                    if (source_segment(D, r, L.source())) {
                        if (count_rejects && sid == home) {
                            rej++;
                            rej_sbi += (unsigned)r.sbi;
                            rej_sbr += (unsigned)r.sbr;
                        } else {
                            finish_ray<Mode>(D, det, r, gid, sid, home, wt, w.tallies,
                                             w.records ? w.records + rid : nullptr);
                            if (w.prov_rec) w.prov_rec[rid] = prov_init();
                        }
                    } else {
                        pool.ray[slot] = r;
                        pool.lane[slot] = L;
                        if (w.prov) w.prov[slot] = prov_init();
                        SlotMeta m;
                        m.gid = gid; m.sid = sid; m.rid = rid; m.pidx = -1;
                        m.acr_caller = 0; m.acr_it = 0; m.acr_stuck = 0; m.acr_last = -1;
                        m.cond_kind = 0; m.cond_started = 0; m.cond_trial = 0; m.cond_target = 0;
                        m.pad[0] = m.pad[1] = 0;
                        pool.meta[slot] = m;
                        filled = true;
                    }
                }
            }
        }
        // slots left unfilled once every photon is drawn are not needed again
        wave_push(w, filled ? WQ_ENTRY : -1, slot);
    }
    const unsigned long long sum = __reduce_add_sync(FULL, (unsigned)drawn);
    if (lane == 0 && sum) atomicAdd(&w.tallies[0].sched[WQ_FREE], sum);
    const unsigned n_rej = __reduce_add_sync(FULL, rej);
    const unsigned n_sbi = __reduce_add_sync(FULL, rej_sbi), n_sbr = __reduce_add_sync(FULL, rej_sbr);
    if (lane == 0 && n_rej) {  // rejected photons end with status 3 and failure code 0 (r.pf is 0)
        atomicAdd(&wt->status[3], (unsigned long long)n_rej);
        atomicAdd(&wt->failure[0], (unsigned long long)n_rej);
        atomicAdd(&wt->n_done, (unsigned long long)n_rej);
        if (n_sbi) atomicAdd(&wt->events[CLR_EV_SOURCE_BORE_INTERACTIONS], (unsigned long long)n_sbi);
        if (n_sbr) atomicAdd(&wt->events[CLR_EV_SOURCE_BORE_REFLECTIONS], (unsigned long long)n_sbr);
    }
    __syncwarp();
    if (home >= 0) flush_warp_tally(wt, w.tallies + home, lane);
}

// ---------------- generic stage kernel (ENTRY, FLIGHT and the event handlers) ----------------
// kLight: the water flights carry the diagnostic hooks, light history and particle-event provenance (a
// separate FLIGHT kernel, used only when a diagnostic is on, keeps them out of the production kernel).
// pv: the photon's provenance state, or null when provenance is not counted.
template <class Mode, int Q, bool kLight = true>
__device__ __forceinline__ int wave_stage_body(const WaveLaunch& w, const DevScene& D, Ray& r,
                                               typename Mode::Lane& L, SlotMeta& m,
                                               unsigned long long* cstats, uint4* pv) {
    if constexpr (Q == WQ_ENTRY) {
        return entry_segment(D, r, L.transport()) ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_FLIGHT) {
        for (int k = 0; k < w.flight_steps; ++k) {
            int pidx = -1;
            const float vinx = r.vx, viny = r.vy, vinz = r.vz;
            const int coh0 = r.wcoh;
            const int e = water_flight<typename Mode::Stream, kLight>(D, r, L.transport(), L.optics(), cstats, &pidx,
                                                                       m.gid);
            if constexpr (kLight) {  // a coherent wave event completes inside the flight
                if (pv && e == WE_NONE && r.wcoh != coh0)
                    prov_event(*pv, r.ic, 4, pidx, vinx, viny, vinz, r.vx, r.vy, r.vz);
            }
            if (e == WE_NONE) continue;
            m.pidx = pidx;
            switch (e) {
                case WE_ENDED: return WQ_FIN;
                case WE_COND:
                    m.cond_kind = CK_FLIGHT; m.cond_started = 0; m.cond_trial = 0; m.cond_target = 0;
                    return WQ_COND;
                case WE_GEOM: return WQ_GEOM;
                case WE_MORPH: return WQ_MORPH;
                case WE_TOP: return WQ_TOP;
                case WE_BOTTOM: return WQ_BOTTOM;
                default: return WQ_SIDE;
            }
        }
        return WQ_FLIGHT;
    } else if constexpr (Q == WQ_COND || Q == WQ_GEOM) {
        // counters and direction before the event: a closure changes them only when it completes
        const int ic0 = r.ic, coh0 = r.wcoh, mor0 = r.wmorph;
        const int per0 = r.pc.entry_reflections, pir0 = r.pc.internal_reflections;
        const float vinx = r.vx, viny = r.vy, vinz = r.vz;
        auto survived = [&]() {  // the event completed with the photon in the water (not a null proposal)
            if (pv && r.ic == ic0)
                prov_event(*pv, r.ic, prov_type(r.wcoh - coh0, r.wmorph - mor0, r.pc.entry_reflections - per0,
                                                r.pc.internal_reflections - pir0),
                           m.pidx, vinx, viny, vinz, r.vx, r.vy, r.vz);
        };
        CondState cs;
        int v;
        if constexpr (Q == WQ_GEOM) {
            v = water_geom_visit(D, r, L.optics(), cstats, m.pidx);
            if (v != 3) {
                if (v == 0) survived();
                return v ? WQ_FIN : WQ_FLIGHT;
            }
            m.cond_kind = CK_GEOM;
            cs = cond_start();
            v = closure_visit(D, r, L.optics(), cstats, m.pidx, CK_GEOM, &cs, kCondInline);
        } else {
            cs.started = m.cond_started; cs.trial = m.cond_trial; cs.target = m.cond_target;
            v = closure_visit(D, r, L.optics(), cstats, m.pidx, m.cond_kind, &cs, kCondBudget);
        }
        if (v == 2) {
            m.cond_started = cs.started; m.cond_trial = cs.trial; m.cond_target = cs.target;
            return WQ_COND;
        }
        if (v == 0) survived();
        // an absorbing encounter of the closure ends the history; the reference keeps its bin and type
        // (not a deflection) (:4836-4848)
        if (v == 1 && pv && r.st == 5 && r.ic == ic0)
            prov_mark(*pv, r.ic, prov_type(r.wcoh - coh0, r.wmorph - mor0, r.pc.entry_reflections - per0,
                                           r.pc.internal_reflections - pir0), m.pidx);
        return v ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_MORPH) {
        const int per0 = r.pc.entry_reflections, pir0 = r.pc.internal_reflections;
        const float vinx = r.vx, viny = r.vy, vinz = r.vz;
        const bool ended = water_morph(D, r, L.optics(), cstats, m.pidx);
        if (pv && !ended)
            prov_event(*pv, r.ic, prov_type(0, 1, r.pc.entry_reflections - per0, r.pc.internal_reflections - pir0),
                       m.pidx, vinx, viny, vinz, r.vx, r.vy, r.vz);
        return ended ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_TOP) {
        const bool ended = water_top(D, r, L.transport());
        if (pv && !ended) prov_return(*pv, r.ic);  // back from the headspace
        return ended ? WQ_FIN : WQ_FLIGHT;
    } else {
        // SIDE, BOTTOM and ACRYL: a bounded piece of the acrylic traversal
        const int budget = wave_drawing(w) ? w.acr_budget : 0;
        o_acr_state as;
        int caller, v;
        if constexpr (Q == WQ_BOTTOM) {
            caller = ACR_BOTTOM;
            v = water_bottom_visit(D, r, L.transport(), &as, budget);
        } else if constexpr (Q == WQ_SIDE) {
            caller = ACR_SIDE;
            as = o_acr_start();
            v = acrylic_visit(D, r, L.transport(), ACR_SIDE, &as, budget);
        } else {
            caller = m.acr_caller;
            as.it = m.acr_it; as.stuck = m.acr_stuck; as.last_surf = m.acr_last;
            v = acrylic_visit(D, r, L.transport(), caller, &as, budget);
        }
        if (v == 2) {
            m.acr_caller = caller; m.acr_it = as.it; m.acr_stuck = as.stuck; m.acr_last = as.last_surf;
            return WQ_ACRYL;
        }
        if (pv && v == 0) prov_return(*pv, r.ic);  // back from the acrylic (or the headspace beyond it)
        return v ? WQ_FIN : WQ_FLIGHT;
    }
}

template <class Mode, int Q, bool kLight = false>
__global__ void __launch_bounds__(kWaveThreads, stage_min_blocks(Q)) wave_stage_kernel(WaveLaunch w) {
    const WaveWindow win = wave_window(w, Q);
    if (win.n == 0) return;
    __shared__ BlockStats bs;
    block_stats_init(&bs);
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    const uint32_t* ring = wave_ring(w, Q);
    const int lane = threadIdx.x & 31;
    unsigned long long done = 0;
    for (unsigned base = wave_claim(w, Q); base < win.n; base = wave_claim(w, Q)) {
        const unsigned i = base + lane;
        const bool valid = i < win.n;
        const uint32_t slot = valid ? ring[(win.head + i) & wave_mask(w)] : 0u;
        int dest = -1;
        if (valid) {
            Ray r = pool.ray[slot];
            typename Mode::Lane L = pool.lane[slot];
            SlotMeta m = pool.meta[slot];
            const DevScene& D = w.scenes[m.sid];
            unsigned long long* cstats = (m.sid == 0) ? bs.cs : w.tallies[m.sid].c.cstats;
            // only the diagnostic variants carry the provenance (ENTRY never changes it)
            constexpr bool kProv = Q != WQ_ENTRY && kLight;
            uint4 pvv;
            uint4* pv = nullptr;
            if (kProv && w.prov) { pvv = w.prov[slot]; pv = &pvv; }
            dest = wave_stage_body<Mode, Q, kLight>(w, D, r, L, m, cstats, pv);
            if (kProv && pv) w.prov[slot] = pvv;
            pool.ray[slot] = r;
            pool.lane[slot] = L;
            if (Q == WQ_FLIGHT || dest == WQ_ACRYL || dest == WQ_COND) pool.meta[slot] = m;
            done++;
        }
        wave_push(w, dest, slot);
    }
    warp_done(&bs, w.tallies, Q, done);
}

// COND stage of the counter-based stream without diagnostics: the photons of a warp's chunk are taken one
// at a time and each one's closure trials run 32 at a time across the warp (closure_visit_warp), so a
// closure of thousands of trials costs tens of warp steps instead of thousands of serial steps.
template <class Mode>
__global__ void __launch_bounds__(kWaveThreads, 1) wave_cond_warp_kernel(WaveLaunch w) {
    const WaveWindow win = wave_window(w, WQ_COND);
    if (win.n == 0) return;
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    const uint32_t* ring = wave_ring(w, WQ_COND);
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    unsigned long long done = 0;
    for (unsigned base = wave_claim(w, WQ_COND); base < win.n; base = wave_claim(w, WQ_COND)) {
        const unsigned i = base + lane;
        const bool valid = i < win.n;
        const uint32_t my_slot = valid ? ring[(win.head + i) & wave_mask(w)] : 0u;
        int my_dest = -1;
        for (unsigned todo = __ballot_sync(FULL, valid); todo; todo &= todo - 1u) {
            const int owner = __ffs(todo) - 1;
            const uint32_t slot = __shfl_sync(FULL, my_slot, owner);
            Ray r = pool.ray[slot];
            typename Mode::Lane L = pool.lane[slot];
            SlotMeta m = pool.meta[slot];
            const DevScene& D = w.scenes[m.sid];
            CondState cs;
            cs.started = m.cond_started; cs.trial = m.cond_trial; cs.target = m.cond_target;
            const int v = closure_visit_warp(D, r, L.optics(), w.tallies[m.sid].c.cstats, m.pidx, m.cond_kind, &cs,
                                             kCondWarpBudget);
            if (lane == owner) {
                if (v == 2) { m.cond_started = cs.started; m.cond_trial = cs.trial; m.cond_target = cs.target; }
                pool.ray[slot] = r;
                pool.lane[slot] = L;
                pool.meta[slot] = m;
                my_dest = v == 2 ? WQ_COND : (v ? WQ_FIN : WQ_FLIGHT);
                done++;
            }
            __syncwarp();
        }
        wave_push(w, my_dest, my_slot);
    }
    const unsigned long long sum = __reduce_add_sync(FULL, (unsigned)done);
    if (lane == 0 && sum) atomicAdd(&w.tallies[0].sched[WQ_COND], sum);
}

// The event-handler stage kernel: its provenance-counting variant when provenance is on.
template <class Mode, int Q>
const void* stage_fn(const void* prov) {
    return prov ? (const void*)wave_stage_kernel<Mode, Q, true> : (const void*)wave_stage_kernel<Mode, Q, false>;
}

// The COND stage kernel: warp-cooperative closures on the counter-based stream without diagnostics, else
// the per-lane stage kernel.
template <class Mode>
const void* cond_fn(const WaveLaunch& w) {
    if constexpr (kCounterStream<typename Mode::Stream>) {
        if (!w.prov && !w.light) return (const void*)wave_cond_warp_kernel<Mode>;
    }
    return stage_fn<Mode, WQ_COND>(w.prov);
}

// ---------------- FIN: detector scoring and tallies; the slot becomes free ----------------
template <class Mode, bool kRecord>
__global__ void __launch_bounds__(kWaveThreads) wave_fin_kernel(WaveLaunch w) {
    const WaveWindow win = wave_window(w, WQ_FIN);
    if (win.n == 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpTally* wt = reinterpret_cast<WarpTally*>(smem_raw) + (threadIdx.x >> 5);
    __shared__ DetTable det;
    det_table_init(&det);
    const int lane = threadIdx.x & 31;
    warp_tally_zero(wt, lane);
    __syncthreads();
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    const uint32_t* ring = wave_ring(w, WQ_FIN);
    unsigned long long done = 0;
    int home = -1;  // scenario whose counts this warp keeps in shared memory (that of its first photon)
    for (unsigned base = wave_claim(w, WQ_FIN); base < win.n; base = wave_claim(w, WQ_FIN)) {
        const unsigned i = base + lane;
        const bool valid = i < win.n;
        const uint32_t slot = valid ? ring[(win.head + i) & wave_mask(w)] : 0u;
        SlotMeta m;
        m.sid = 0;
        if (valid) m = pool.meta[slot];
        if (home < 0) home = __shfl_sync(0xffffffffu, m.sid, 0);  // lane 0 is valid in every claimed chunk
        if (valid) {
            const Ray r = pool.ray[slot];
            const DevScene& D = w.scenes[m.sid];
            finish_ray<Mode>(D, det, r, m.gid, m.sid, home, wt, w.tallies, kRecord ? w.records + m.rid : nullptr,
                             w.prov ? w.prov + slot : nullptr);
            if (kRecord && w.prov_rec) w.prov_rec[m.rid] = w.prov ? w.prov[slot] : prov_init();
            done++;
        }
        wave_push(w, valid ? WQ_FREE : -1, slot);
    }
    const unsigned long long sum = __reduce_add_sync(0xffffffffu, (unsigned)done);
    if (lane == 0 && sum) atomicAdd(&w.tallies[0].sched[WQ_FIN], sum);
    if (home >= 0) flush_warp_tally(wt, w.tallies + home, lane);
}

// ---------------- TAIL: the last photons, each run to its end by one thread ----------------
// kDiag: the stage bodies with the diagnostic hooks (light history, provenance); the production tail
// carries none of them.
template <class Mode, bool kDiag>
__device__ __forceinline__ int tail_visit(const WaveLaunch& w, int q, const DevScene& D, Ray& r,
                                          typename Mode::Lane& L, SlotMeta& m, unsigned long long* cstats,
                                          uint4* pv) {
    switch (q) {
        case WQ_ENTRY: return wave_stage_body<Mode, WQ_ENTRY, kDiag>(w, D, r, L, m, cstats, pv);
        case WQ_FLIGHT: return wave_stage_body<Mode, WQ_FLIGHT, kDiag>(w, D, r, L, m, cstats, pv);
        case WQ_COND: return wave_stage_body<Mode, WQ_COND, kDiag>(w, D, r, L, m, cstats, pv);
        case WQ_GEOM: return wave_stage_body<Mode, WQ_GEOM, kDiag>(w, D, r, L, m, cstats, pv);
        case WQ_MORPH: return wave_stage_body<Mode, WQ_MORPH, kDiag>(w, D, r, L, m, cstats, pv);
        case WQ_TOP: return wave_stage_body<Mode, WQ_TOP, kDiag>(w, D, r, L, m, cstats, pv);
        case WQ_BOTTOM: return wave_stage_body<Mode, WQ_BOTTOM, kDiag>(w, D, r, L, m, cstats, pv);
        case WQ_SIDE: return wave_stage_body<Mode, WQ_SIDE, kDiag>(w, D, r, L, m, cstats, pv);
        default: return wave_stage_body<Mode, WQ_ACRYL, kDiag>(w, D, r, L, m, cstats, pv);
    }
}

// Runs after the last pass, when every photon is drawn: the photons still queued (entries [snap, tail)
// of every queue but FREE) are taken one per thread and carried through the same stage bodies, in the
// same order, as the passes would carry them, then scored. Per-ray results are those of the passes.
template <class Mode, bool kRecord, bool kDiag>
__global__ void __launch_bounds__(kTailThreads) wave_tail_kernel(WaveLaunch w) {
    __shared__ DetTable det;
    det_table_init(&det);
    __syncthreads();
    const WaveCtl* c = w.ctl;
    unsigned first[CLR_WQ_COUNT + 1];
    first[0] = first[1] = 0;
    for (int q = 1; q < CLR_WQ_COUNT; ++q) first[q + 1] = first[q] + (c->tail[q] - c->snap[q]);
    const unsigned total = first[CLR_WQ_COUNT];
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    unsigned long long visits[CLR_WQ_COUNT] = {};
    for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        int q = 1;
        while (idx >= first[q + 1]) ++q;
        const uint32_t slot = wave_ring(w, q)[(c->snap[q] + (idx - first[q])) & wave_mask(w)];
        Ray r = pool.ray[slot];
        typename Mode::Lane L = pool.lane[slot];
        SlotMeta m = pool.meta[slot];
        const DevScene& D = w.scenes[m.sid];
        unsigned long long* cstats = w.tallies[m.sid].c.cstats;
        uint4 pvv = prov_init();
        uint4* pv = nullptr;
        if constexpr (kDiag) {
            if (w.prov) { pvv = w.prov[slot]; pv = &pvv; }
        }
        while (q != WQ_FIN) {
            ++visits[q];
            q = tail_visit<Mode, kDiag>(w, q, D, r, L, m, cstats, pv);
        }
        ++visits[WQ_FIN];
        finish_ray<Mode>(D, det, r, m.gid, m.sid, -1, nullptr, w.tallies, kRecord ? w.records + m.rid : nullptr, pv);
        if constexpr (kDiag) {
            if (kRecord && w.prov_rec) w.prov_rec[m.rid] = pvv;
        }
    }
    for (int q = 1; q < CLR_WQ_COUNT; ++q)
        if (visits[q]) atomicAdd(&w.tallies[0].sched[q], visits[q]);
}

__global__ void wave_init_kernel(WaveLaunch w) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.cap) wave_ring(w, WQ_FREE)[i] = i;
    if (i == 0) {
        WaveCtl* c = w.ctl;
        for (int k = 0; k < CLR_WQ_COUNT; ++k) {
            c->head[k] = 0u; c->tail[k] = 0u; c->snap[k] = 0u; c->finished[k] = 0u; c->skips[k] = 0u;
            c->claim[k] = 0u;
        }
        c->tail[WQ_FREE] = w.cap;
        c->next_photon = 0ull;
        c->total_photons = w.total;
        c->live = w.total > 0 ? 1u : 0u;
        c->passes = 0u;
        c->tail_ready = 0u;
        c->in_flight = 0u;
    }
}

// ---------------- host driver ----------------
// One pass as a graph: the begin kernel, then every stage kernel depending only on it.
template <class Mode, bool kRecord>
struct WavePass {
    static constexpr int kSmemTally = (kWaveThreads / 32) * (int)sizeof(WarpTally);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    ~WavePass() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }

    static cudaError_t grid_of(const void* kernel, int smem, int num_sms, int per_sm_cap, dim3* g) {
        int occ = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, kWaveThreads, smem);
        if (e != cudaSuccess) return e;
        if (occ < 1) occ = 1;
        if (per_sm_cap > 0 && occ > per_sm_cap) occ = per_sm_cap;
        *g = dim3((unsigned)(num_sms * occ));
        return cudaSuccess;
    }

    cudaError_t build(const WaveLaunch& w, int num_sms) {
        cudaError_t e;
        if ((e = cudaFuncSetAttribute(wave_gen_kernel<Mode>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kSmemTally)) != cudaSuccess)
            return e;
        if ((e = cudaFuncSetAttribute(wave_fin_kernel<Mode, kRecord>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      kSmemTally)) != cudaSuccess)
            return e;
        if ((e = cudaGraphCreate(&graph, 0)) != cudaSuccess) return e;
        void* args[] = {const_cast<WaveLaunch*>(&w)};
        cudaKernelNodeParams p = {};
        p.kernelParams = args;
        p.func = (void*)wave_begin_kernel;
        p.gridDim = dim3(1);
        p.blockDim = dim3(32);
        p.sharedMemBytes = 0;
        cudaGraphNode_t begin;
        if ((e = cudaGraphAddKernelNode(&begin, graph, nullptr, 0, &p)) != cudaSuccess) return e;
        struct StageK {
            const void* fn;
            int smem;
            int per_sm_cap;
        };
        // rare stages get one block per SM: their windows are small and their warps long-lived
        const StageK ks[CLR_WQ_COUNT] = {
            {(const void*)wave_gen_kernel<Mode>, kSmemTally, 0},
            {(const void*)wave_stage_kernel<Mode, WQ_ENTRY>, 0, 0},
            {(w.light || w.prov) ? (const void*)wave_stage_kernel<Mode, WQ_FLIGHT, true>
                     : (const void*)wave_stage_kernel<Mode, WQ_FLIGHT, false>, 0, 0},
            {cond_fn<Mode>(w), 0, 1},
            {stage_fn<Mode, WQ_GEOM>(w.prov), 0, 0},
            {stage_fn<Mode, WQ_MORPH>(w.prov), 0, 1},
            {stage_fn<Mode, WQ_TOP>(w.prov), 0, 1},
            {stage_fn<Mode, WQ_BOTTOM>(w.prov), 0, 1},
            {stage_fn<Mode, WQ_SIDE>(w.prov), 0, 0},
            {stage_fn<Mode, WQ_ACRYL>(w.prov), 0, 1},
            {(const void*)wave_fin_kernel<Mode, kRecord>, kSmemTally, 0},
        };
        p.blockDim = dim3(kWaveThreads);
        for (int q = 0; q < CLR_WQ_COUNT; ++q) {
            dim3 g;
            const int cap = w.stage_blocks[q] > 0 ? w.stage_blocks[q] : ks[q].per_sm_cap;
            if ((e = grid_of(ks[q].fn, ks[q].smem, num_sms, cap, &g)) != cudaSuccess) return e;
            p.func = const_cast<void*>(ks[q].fn);
            p.gridDim = g;
            p.sharedMemBytes = (unsigned)ks[q].smem;
            cudaGraphNode_t node;
            if ((e = cudaGraphAddKernelNode(&node, graph, &begin, 1, &p)) != cudaSuccess) return e;
        }
        return cudaGraphInstantiate(&exec, graph, 0);
    }
};

// Runs passes until the pool drains. Every `batch` passes the host reads the live flag; the next batch
// is already queued when it does, so the GPU does not idle on the read. Passes after the pool drained
// find empty windows and return at once.
template <class Mode, bool kRecord>
cudaError_t wave_run_t(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes, WaveRunInfo* info) {
    info->passes = 0;
    info->tail = 0;
    info->tail_photons = 0;
    WavePass<Mode, kRecord> P;
    cudaError_t e = P.build(w, num_sms);
    if (e != cudaSuccess) return e;
    wave_init_kernel<<<(w.cap + 255) / 256, 256, 0, st>>>(w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int batch = w.pass_batch > 0 ? w.pass_batch : CLR_ENGINE_DEFAULT_PASS_BATCH;
    long long launched = 0;
    volatile unsigned* live = w.host_live;  // [live, tail_ready, in_flight] of the pass before the read
    static_assert(offsetof(WaveCtl, tail_ready) == offsetof(WaveCtl, live) + sizeof(unsigned) &&
                      offsetof(WaveCtl, in_flight) == offsetof(WaveCtl, live) + 2 * sizeof(unsigned),
                  "flag words are read together");
    for (int k = 0; k < batch; ++k)
        if ((e = cudaGraphLaunch(P.exec, st)) != cudaSuccess) return e;
    launched += batch;
    while (true) {
        if ((e = cudaMemcpyAsync((void*)w.host_live, &w.ctl->live, 3 * sizeof(unsigned), cudaMemcpyDeviceToHost,
                                 st)) != cudaSuccess)
            return e;
        if ((e = cudaEventRecord(w.flag_event, st)) != cudaSuccess) return e;
        for (int k = 0; k < batch; ++k)
            if ((e = cudaGraphLaunch(P.exec, st)) != cudaSuccess) return e;
        launched += batch;
        if ((e = cudaEventSynchronize(w.flag_event)) != cudaSuccess) return e;
        if (live[0] == 0u) break;
        if (live[1] != 0u) {
            // at most live[2] photons remain after the passes already queued: finish them in one launch
            const unsigned n = live[2];
            const int blocks = (int)std::max(1u, std::min(n, 65536u * kTailThreads) / kTailThreads + 1);
            if (w.tail_begin && (e = cudaEventRecord(w.tail_begin, st)) != cudaSuccess) return e;
            if (w.light || w.prov) wave_tail_kernel<Mode, kRecord, true><<<blocks, kTailThreads, 0, st>>>(w);
            else wave_tail_kernel<Mode, kRecord, false><<<blocks, kTailThreads, 0, st>>>(w);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            if (w.tail_end && (e = cudaEventRecord(w.tail_end, st)) != cudaSuccess) return e;
            info->tail = 1;
            info->tail_photons = n;
            launched += 1;
            break;
        }
        if (launched > max_passes) {
            cudaStreamSynchronize(st);
            return cudaErrorLaunchTimeout;
        }
    }
    // wait for the passes queued after the flag read before the graph is destroyed
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    info->passes = (int)launched - info->tail;
    return cudaSuccess;
}

}  // namespace
}  // namespace clr
