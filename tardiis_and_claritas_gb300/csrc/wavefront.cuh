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
//   COND, GEOM, MORPH   particle events (conditional closure, geometric sphere, spheroid)
//   TOP, BOTTOM, SIDE   transmission into the headspace, the bottom disc, the acrylic wall
//                                                                -> FLIGHT or FIN
//   FIN    detector scoring and tallies; the slot returns to the free queue
//
// One pass launches the ten stage kernels in that order. Queues are ring buffers of slot ids with
// monotonically increasing 32-bit head/tail counters (capacity a power of two, so wrap-around is
// exact). A stage consumes the window [head, snap) of its queue, where snap is the tail that the
// previous stage kernel's last block recorded after all of its pushes, so a stage never consumes
// slots pushed while it runs (FLIGHT may push to itself). Pushes are aggregated per warp and queue.
// The last block of FIN sets a live flag that the host reads every few passes.
//
// Within each stage the device functions, arithmetic and per-ray draw order are the persistent
// kernel's (they are the same functions), so per-ray results in the xorshift parity mode are
// identical to the reference's whichever engine runs.
#pragma once
#include "photon_kernel.cuh"

namespace clr {
namespace {

enum : int { WQ_FREE = 0, WQ_ENTRY, WQ_FLIGHT, WQ_COND, WQ_GEOM, WQ_MORPH, WQ_TOP, WQ_BOTTOM, WQ_SIDE, WQ_FIN };
static_assert(WQ_FIN + 1 == CLR_WQ_COUNT, "queue count");

constexpr int kWaveThreads = 256;
// water flights per FLIGHT visit before the photon is re-queued (bounds lane imbalance in a warp)
constexpr int kFlightSteps = 8;

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
        w.qbuf[(size_t)q * w.cap + (pos & (w.cap - 1u))] = slot;
    }
}

// End of a stage kernel: the last block to finish retires the consumed window and records the
// snapshot of the next stage's queue; the last block of FIN also computes the live flag.
__device__ __forceinline__ void wave_commit(const WaveLaunch& w, int q) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned done = atomicAdd(&w.ctl->finished[q], 1u);
        if (done == gridDim.x - 1) {
            __threadfence();
            WaveCtl* c = w.ctl;
            c->head[q] = c->snap[q];
            const int nq = (q + 1) % CLR_WQ_COUNT;
            c->snap[nq] = atomicAdd(&c->tail[nq], 0u);
            c->finished[q] = 0u;
            if (q == WQ_FIN) {
                unsigned pending = 0;
                for (int k = 1; k < CLR_WQ_COUNT; ++k) pending |= atomicAdd(&c->tail[k], 0u) - c->head[k];
                const unsigned long long np = atomicAdd(&c->next_photon, 0ull);
                c->live = (pending != 0u || np < c->total_photons) ? 1u : 0u;
                c->passes++;
            }
            __threadfence();
        }
    }
}

// Per-block conditional-closure statistics for scenario 0 (others go straight to the device tally).
struct BlockStats {
    unsigned long long cs[CLR_N_CONDITIONAL_STATS];
    unsigned long long items;
};
__device__ __forceinline__ void block_stats_init(BlockStats* b) {
    if (threadIdx.x < CLR_N_CONDITIONAL_STATS) b->cs[threadIdx.x] = 0ull;
    if (threadIdx.x == 0) b->items = 0ull;
    __syncthreads();
}
__device__ __forceinline__ void block_stats_flush(BlockStats* b, DevTally* t, int q) {
    __syncthreads();
    if (threadIdx.x < CLR_N_CONDITIONAL_STATS && b->cs[threadIdx.x])
        atomicAdd(&t[0].c.cstats[threadIdx.x], b->cs[threadIdx.x]);
    if (threadIdx.x == 0 && b->items) atomicAdd(&t[0].sched[q], b->items);
}

// Window of the stage's queue, iterated in warp-uniform chunks of 32 entries.
struct WaveWindow {
    unsigned head, n;
};
__device__ __forceinline__ WaveWindow wave_window(const WaveLaunch& w, int q) {
    WaveWindow win;
    win.head = *(volatile unsigned*)&w.ctl->head[q];
    win.n = *(volatile unsigned*)&w.ctl->snap[q] - win.head;
    return win;
}

template <class Mode>
__device__ __forceinline__ void photon_of(const WaveLaunch& w, unsigned long long p, int* sid, long long* rid) {
    int lo = 0, hi = w.n_scen - 1;
    while (lo < hi) {  // last scenario whose first photon is <= p
        const int mid = (lo + hi + 1) >> 1;
        if ((unsigned long long)w.ray_begin[mid] <= p) lo = mid; else hi = mid - 1;
    }
    *sid = lo;
    *rid = (long long)(p - (unsigned long long)w.ray_begin[lo]);
}

// ---------------- GEN: fill free slots with photons that pass the source collimator ----------------
template <class Mode>
__global__ void __launch_bounds__(kWaveThreads) wave_gen_kernel(WaveLaunch w) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpTally* wt = reinterpret_cast<WarpTally*>(smem_raw) + (threadIdx.x >> 5);
    __shared__ DetTable det;
    __shared__ unsigned long long items;
    det_table_init(&det);
    const int lane = threadIdx.x & 31;
    {
        unsigned long long* p = reinterpret_cast<unsigned long long*>(wt);
        for (int i = lane; i < (int)(sizeof(WarpTally) / 8); i += 32) p[i] = 0ull;
    }
    if (threadIdx.x == 0) items = 0ull;
    __syncthreads();
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    const WaveWindow win = wave_window(w, WQ_FREE);
    const unsigned FULL = 0xffffffffu;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
    bool out = *(volatile unsigned long long*)&w.ctl->next_photon >= w.ctl->total_photons;
    unsigned long long drawn = 0;
    for (unsigned base = warp * 32u; base < win.n && !__all_sync(FULL, out); base += n_warps * 32u) {
        const unsigned i = base + lane;
        const bool valid = i < win.n;
        const uint32_t slot = valid ? w.qbuf[(size_t)WQ_FREE * w.cap + ((win.head + i) & (w.cap - 1u))] : 0u;
        bool filled = false;
        while (true) {
            const unsigned need = __ballot_sync(FULL, valid && !filled && !out);
            if (!need) break;
            unsigned long long b0 = 0;
            if (lane == __ffs(need) - 1) b0 = atomicAdd(&w.ctl->next_photon, (unsigned long long)__popc(need));
            b0 = __shfl_sync(FULL, b0, __ffs(need) - 1);
            if ((need >> lane) & 1u) {
                const unsigned long long p = b0 + (unsigned long long)__popc(need & ((1u << lane) - 1u));
                if (p >= w.ctl->total_photons) {
                    out = true;
                } else {
                    int sid;
                    long long rid;
                    photon_of<Mode>(w, p, &sid, &rid);
                    const DevScene& D = w.scenes[sid];
                    const uint32_t gid = D.ray_offset + (uint32_t)rid;
                    typename Mode::Lane L;
                    Mode::seed(D, gid, L);
                    Ray r;
                    ray_reset(r);
                    drawn++;
                    if (source_segment(D, r, L.source())) {
                        finish_ray<Mode>(D, det, r, gid, sid, 0, wt, w.tallies, w.records ? w.records + rid : nullptr);
                    } else {
                        pool.ray[slot] = r;
                        pool.lane[slot] = L;
                        SlotMeta m;
                        m.gid = gid; m.sid = sid; m.rid = rid; m.pidx = -1; m.pad = 0;
                        pool.meta[slot] = m;
                        filled = true;
                    }
                }
            }
        }
        wave_push(w, filled ? WQ_ENTRY : -1, slot);
    }
    atomicAdd(&items, drawn);
    __syncthreads();
    flush_warp_tally(wt, w.tallies, lane);
    if (threadIdx.x == 0 && items) atomicAdd(&w.tallies[0].sched[WQ_FREE], items);
    wave_commit(w, WQ_FREE);
}

// ---------------- generic stage kernel (ENTRY, FLIGHT and the event handlers) ----------------
template <class Mode, int Q>
__device__ __forceinline__ int wave_stage_body(const WaveLaunch& w, const DevScene& D, Ray& r,
                                               typename Mode::Lane& L, SlotMeta& m,
                                               unsigned long long* cstats) {
    if constexpr (Q == WQ_ENTRY) {
        return entry_segment(D, r, L.transport()) ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_FLIGHT) {
        for (int k = 0; k < kFlightSteps; ++k) {
            int pidx = -1;
            const int e = water_flight(D, r, L.transport(), L.optics(), cstats, &pidx);
            if (e == WE_NONE) continue;
            m.pidx = pidx;
            switch (e) {
                case WE_ENDED: return WQ_FIN;
                case WE_COND: return WQ_COND;
                case WE_GEOM: return WQ_GEOM;
                case WE_MORPH: return WQ_MORPH;
                case WE_TOP: return WQ_TOP;
                case WE_BOTTOM: return WQ_BOTTOM;
                default: return WQ_SIDE;
            }
        }
        return WQ_FLIGHT;
    } else if constexpr (Q == WQ_COND) {
        return water_cond(D, r, L.optics(), cstats, m.pidx) ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_GEOM) {
        return water_geom(D, r, L.optics(), cstats, m.pidx) ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_MORPH) {
        return water_morph(D, r, L.optics(), cstats, m.pidx) ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_TOP) {
        return water_top(D, r, L.transport()) ? WQ_FIN : WQ_FLIGHT;
    } else if constexpr (Q == WQ_BOTTOM) {
        return water_bottom(D, r, L.transport()) ? WQ_FIN : WQ_FLIGHT;
    } else {
        return water_side(D, r, L.transport()) ? WQ_FIN : WQ_FLIGHT;
    }
}

template <class Mode, int Q>
__global__ void __launch_bounds__(kWaveThreads) wave_stage_kernel(WaveLaunch w) {
    __shared__ BlockStats bs;
    block_stats_init(&bs);
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    const WaveWindow win = wave_window(w, Q);
    const int lane = threadIdx.x & 31;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long done = 0;
    for (unsigned base = warp * 32u; base < win.n; base += n_warps * 32u) {
        const unsigned i = base + lane;
        const bool valid = i < win.n;
        const uint32_t slot = valid ? w.qbuf[(size_t)Q * w.cap + ((win.head + i) & (w.cap - 1u))] : 0u;
        int dest = -1;
        if (valid) {
            Ray r = pool.ray[slot];
            typename Mode::Lane L = pool.lane[slot];
            SlotMeta m = pool.meta[slot];
            const DevScene& D = w.scenes[m.sid];
            unsigned long long* cstats = (m.sid == 0) ? bs.cs : w.tallies[m.sid].c.cstats;
            dest = wave_stage_body<Mode, Q>(w, D, r, L, m, cstats);
            pool.ray[slot] = r;
            pool.lane[slot] = L;
            if (Q == WQ_FLIGHT) pool.meta[slot].pidx = m.pidx;
            done++;
        }
        wave_push(w, dest, slot);
    }
    atomicAdd(&bs.items, done);
    block_stats_flush(&bs, w.tallies, Q);
    wave_commit(w, Q);
}

// ---------------- FIN: detector scoring and tallies; the slot becomes free ----------------
template <class Mode, bool kRecord>
__global__ void __launch_bounds__(kWaveThreads) wave_fin_kernel(WaveLaunch w) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpTally* wt = reinterpret_cast<WarpTally*>(smem_raw) + (threadIdx.x >> 5);
    __shared__ DetTable det;
    __shared__ unsigned long long items;
    det_table_init(&det);
    const int lane = threadIdx.x & 31;
    {
        unsigned long long* p = reinterpret_cast<unsigned long long*>(wt);
        for (int i = lane; i < (int)(sizeof(WarpTally) / 8); i += 32) p[i] = 0ull;
    }
    if (threadIdx.x == 0) items = 0ull;
    __syncthreads();
    const WavePool<Mode> pool = wave_pool<Mode>(w);
    const WaveWindow win = wave_window(w, WQ_FIN);
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
    unsigned long long done = 0;
    for (unsigned base = warp * 32u; base < win.n; base += n_warps * 32u) {
        const unsigned i = base + lane;
        const bool valid = i < win.n;
        const uint32_t slot = valid ? w.qbuf[(size_t)WQ_FIN * w.cap + ((win.head + i) & (w.cap - 1u))] : 0u;
        if (valid) {
            const Ray r = pool.ray[slot];
            const SlotMeta m = pool.meta[slot];
            const DevScene& D = w.scenes[m.sid];
            finish_ray<Mode>(D, det, r, m.gid, m.sid, 0, wt, w.tallies, kRecord ? w.records + m.rid : nullptr);
            done++;
        }
        wave_push(w, valid ? WQ_FREE : -1, slot);
    }
    atomicAdd(&items, done);
    __syncthreads();
    flush_warp_tally(wt, w.tallies, lane);
    if (threadIdx.x == 0 && items) atomicAdd(&w.tallies[0].sched[WQ_FIN], items);
    wave_commit(w, WQ_FIN);
}

__global__ void wave_init_kernel(WaveLaunch w) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < w.cap) w.qbuf[(size_t)WQ_FREE * w.cap + i] = i;
    if (i == 0) {
        WaveCtl* c = w.ctl;
        for (int k = 0; k < CLR_WQ_COUNT; ++k) { c->head[k] = 0u; c->tail[k] = 0u; c->snap[k] = 0u; c->finished[k] = 0u; }
        c->tail[WQ_FREE] = w.cap;
        c->snap[WQ_FREE] = w.cap;
        c->next_photon = 0ull;
        c->total_photons = w.total;
        c->live = w.total > 0 ? 1u : 0u;
        c->passes = 0u;
    }
}

// ---------------- host driver ----------------
template <class Mode, bool kRecord>
struct WaveKernels {
    static constexpr int kSmemTally = (kWaveThreads / 32) * (int)sizeof(WarpTally);
    int grid[CLR_WQ_COUNT] = {0};

    cudaError_t setup(int num_sms) {
        cudaError_t e;
        e = cudaFuncSetAttribute(wave_gen_kernel<Mode>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTally);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(wave_fin_kernel<Mode, kRecord>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kSmemTally);
        if (e != cudaSuccess) return e;
        int occ[CLR_WQ_COUNT] = {0};
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_FREE], wave_gen_kernel<Mode>, kWaveThreads, kSmemTally);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_ENTRY], wave_stage_kernel<Mode, WQ_ENTRY>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_FLIGHT], wave_stage_kernel<Mode, WQ_FLIGHT>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_COND], wave_stage_kernel<Mode, WQ_COND>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_GEOM], wave_stage_kernel<Mode, WQ_GEOM>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_MORPH], wave_stage_kernel<Mode, WQ_MORPH>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_TOP], wave_stage_kernel<Mode, WQ_TOP>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_BOTTOM], wave_stage_kernel<Mode, WQ_BOTTOM>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_SIDE], wave_stage_kernel<Mode, WQ_SIDE>, kWaveThreads, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[WQ_FIN], wave_fin_kernel<Mode, kRecord>, kWaveThreads, kSmemTally);
        for (int k = 0; k < CLR_WQ_COUNT; ++k) grid[k] = num_sms * (occ[k] > 0 ? occ[k] : 1);
        return cudaGetLastError();
    }

    void pass(const WaveLaunch& w, cudaStream_t st) const {
        wave_gen_kernel<Mode><<<grid[WQ_FREE], kWaveThreads, kSmemTally, st>>>(w);
        wave_stage_kernel<Mode, WQ_ENTRY><<<grid[WQ_ENTRY], kWaveThreads, 0, st>>>(w);
        wave_stage_kernel<Mode, WQ_FLIGHT><<<grid[WQ_FLIGHT], kWaveThreads, 0, st>>>(w);
        wave_stage_kernel<Mode, WQ_COND><<<grid[WQ_COND], kWaveThreads, 0, st>>>(w);
        wave_stage_kernel<Mode, WQ_GEOM><<<grid[WQ_GEOM], kWaveThreads, 0, st>>>(w);
        wave_stage_kernel<Mode, WQ_MORPH><<<grid[WQ_MORPH], kWaveThreads, 0, st>>>(w);
        wave_stage_kernel<Mode, WQ_TOP><<<grid[WQ_TOP], kWaveThreads, 0, st>>>(w);
        wave_stage_kernel<Mode, WQ_BOTTOM><<<grid[WQ_BOTTOM], kWaveThreads, 0, st>>>(w);
        wave_stage_kernel<Mode, WQ_SIDE><<<grid[WQ_SIDE], kWaveThreads, 0, st>>>(w);
        wave_fin_kernel<Mode, kRecord><<<grid[WQ_FIN], kWaveThreads, kSmemTally, st>>>(w);
    }
};

// Runs passes until the pool drains. Every `batch` passes the host reads the live flag; the next batch
// is already queued when it does, so the GPU does not idle on the read. Passes after the pool drained
// find empty windows and return at once.
template <class Mode, bool kRecord>
cudaError_t wave_run_t(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes, int* passes_out) {
    WaveKernels<Mode, kRecord> K;
    cudaError_t e = K.setup(num_sms);
    if (e != cudaSuccess) return e;
    wave_init_kernel<<<(w.cap + 255) / 256, 256, 0, st>>>(w);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int batch = 8;
    long long launched = 0;
    volatile unsigned* live = w.host_live;
    for (int k = 0; k < batch; ++k) K.pass(w, st);
    launched += batch;
    while (true) {
        if ((e = cudaMemcpyAsync((void*)w.host_live, &w.ctl->live, sizeof(unsigned), cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess)
            return e;
        if ((e = cudaEventRecord(w.flag_event, st)) != cudaSuccess) return e;
        for (int k = 0; k < batch; ++k) K.pass(w, st);
        launched += batch;
        if ((e = cudaEventSynchronize(w.flag_event)) != cudaSuccess) return e;
        if (*live == 0u) break;
        if (launched > max_passes) return cudaErrorLaunchTimeout;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (passes_out) *passes_out = (int)launched;
    return cudaSuccess;
}

}  // namespace
}  // namespace clr
