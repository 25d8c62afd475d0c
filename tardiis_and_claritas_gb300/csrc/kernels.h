// Internal launch interface between the C ABI (clr_api.cu) and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "device_scene.cuh"

#define CLR_TRACE_THREADS 256

namespace clr {

struct LaunchArgs {
    const DevScene* scenes;
    const long long* chunk_begin;  // [n_scen + 1] first work chunk of each scenario
    int n_scen;
    long long n_chunks;
    int chunk_rays;
    unsigned long long* work;      // global chunk counter (zeroed before launch)
    DevTally* tallies;             // [n_scen]
    clr_ray_record* records;       // nullable; single-scenario parity runs only
    int grid;
    cudaStream_t stream;
    int rng_mode;
    bool weighted;
};

cudaError_t launch_xor(const LaunchArgs& a);
cudaError_t launch_philox(const LaunchArgs& a);
int occupancy_xor(bool records);
int occupancy_philox(bool records);
inline cudaError_t launch_photon_kernel(const LaunchArgs& a) {
    return a.rng_mode == CLR_RNG_PHILOX ? launch_philox(a) : launch_xor(a);
}
inline int photon_kernel_occupancy(int rng_mode, bool records, bool /*weighted*/) {
    return rng_mode == CLR_RNG_PHILOX ? occupancy_philox(records) : occupancy_xor(records);
}

// ---------------- wavefront engine (wavefront.cuh) ----------------
#define CLR_WQ_COUNT 11  // stage queues: free, entry, flight, cond, geom, morph, top, bottom, side, acrylic, fin

struct SlotMeta {
    uint32_t gid;   // global ray id (ray_offset + rid): the random-stream key
    int32_t sid;    // scenario
    long long rid;  // ray index within the scenario
    int32_t pidx;   // size bin of a pending particle event
    int32_t acr_caller;                       // pending acrylic traversal: which handler started it
    int32_t acr_it, acr_stuck, acr_last;      // and its loop state
    int32_t cond_kind;                        // pending conditional closure: which event it completes
    int32_t cond_started, cond_trial, cond_target;  // and its loop state
    int32_t pad[2];
};

struct WaveCtl {
    unsigned long long next_photon, total_photons;
    unsigned head[CLR_WQ_COUNT], tail[CLR_WQ_COUNT], snap[CLR_WQ_COUNT], finished[CLR_WQ_COUNT], skips[CLR_WQ_COUNT];
    unsigned claim[CLR_WQ_COUNT];  // next unclaimed entry of this pass's window (chunks of 32)
    unsigned live;        // a photon is undrawn or in flight (read by the host)
    unsigned tail_ready;  // every photon is drawn and few remain in flight: the tail kernel may finish them
    unsigned in_flight;   // photons in flight at the last pass's begin
    unsigned passes;
};

struct WaveLaunch {
    const DevScene* scenes;
    int n_scen;
    const long long* ray_begin;    // [n_scen + 1] first photon of each scenario in the run's photon order
    unsigned long long total;
    DevTally* tallies;
    clr_ray_record* records;       // nullable
    void* ray;                     // [cap] Ray
    void* lane;                    // [cap] random-stream state
    SlotMeta* meta;                // [cap]
    uint32_t* qbuf;                // [CLR_WQ_COUNT][2 * cap] queue rings
    WaveCtl* ctl;
    unsigned cap;                  // slots, a power of two
    unsigned* host_live;           // pinned host words: live, tail ready, photons in flight
    cudaEvent_t flag_event;
    cudaEvent_t tail_begin, tail_end;  // timing events recorded around the tail kernel
    // engine settings (clr_engine_config, defaults filled in): water flights per FLIGHT visit, photons in
    // flight at which the tail kernel takes over, queue length at which a rare stage runs, and per stage a
    // cap on resident blocks per SM (0: occupancy)
    int flight_steps;
    unsigned tail_photons, rare_batch;
    int stage_blocks[CLR_WQ_COUNT];
    int pass_batch;
    int acr_budget;  // bounces per acrylic-traversal piece while photons are still drawn
    bool light;                    // light-history diagnostics on: the FLIGHT stage with its hooks
    uint4* prov;                   // [cap] particle-event provenance per slot; null unless counted
    uint4* prov_rec;               // [n_rays] provenance of every ray, with per-ray records; nullable
};

// What one engine execution did: pass graphs launched, and whether (with how many photons) the tail kernel ran.
struct WaveRunInfo {
    int passes;
    int tail;
    unsigned tail_photons;
};
cudaError_t wave_run_xor(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes, WaveRunInfo* info);
cudaError_t wave_run_philox(const WaveLaunch& w, int num_sms, cudaStream_t st, long long max_passes,
                            WaveRunInfo* info);
size_t wave_ray_bytes();
size_t wave_lane_bytes(int rng_mode);

// Calibration kernels (calibrate.cu): FP32 FFMA (which=0) or FP64 DFMA (which=1) throughput loops.
// Sets *ops to the number of operations the launch performs (an FMA counts 2).
cudaError_t launch_calibration(int which, int num_sms, cudaStream_t stream, double* ops);

// Device buffers of one scenario's particle physics (all FP64 unless named _f).
struct ParticleBuffers {
    int n = 0, nt = 0, n_radial = 0, grid_nr = 2, grid_nz = 2;
    double grid_zmax = 0.0;
    double *d = nullptr, *w = nullptr, *nidx = nullptr, *kidx = nullptr;
    int* nstop = nullptr;
    double *x = nullptr, *qext = nullptr, *qsca = nullptr, *qabs = nullptr, *qback = nullptr, *g = nullptr,
           *albedo = nullptr;
    double* ab = nullptr;  // Mie a_n, b_n scratch: [n][CLR_MIE_MAX_ORDER][4] (a.re, a.im, b.re, b.im)
    double *theta = nullptr, *pdf = nullptr, *phase_cdf = nullptr;
    float *theta_f = nullptr, *phase_cdf_f = nullptr;
    int* phase_guide = nullptr;  // [n][kPhaseGuide + 1]
    double *radius = nullptr, *nden = nullptr, *mug = nullptr, *mus = nullptr, *mue = nullptr, *muw = nullptr,
           *muev = nullptr, *gcdf = nullptr, *wcdf = nullptr, *pcdf = nullptr, *muscal = nullptr;
    float *gcdf_f = nullptr, *wcdf_f = nullptr, *pn_f = nullptr, *pk_f = nullptr, *prad_f = nullptr;
    double *moment_a = nullptr, *moment_b = nullptr;
    uint8_t* moment_mode = nullptr;
    int any_moment = 0;
    double *trace_geom = nullptr, *trace_wave = nullptr;
    double *sedA = nullptr, *sedB = nullptr, *sed_norm = nullptr, *sed_max = nullptr, *sed_radial_log = nullptr,
           *sed_wr = nullptr, *sed_major = nullptr, *sed_grid = nullptr, *grid_max = nullptr;
    double* sed_terms = nullptr;  // [n][n_quad] quadrature terms of the sediment normalisation
    double* sed_ws = nullptr;     // [n] settling velocity
    // sediment model 3 without a supplied grid: the meridional solver's coefficient planes [n][5][nr*nz],
    // residuals [2][n] + the final largest residual, grid-barrier words and iteration count (null otherwise)
    double* merid_coef = nullptr;
    double* merid_residual = nullptr;
    unsigned* merid_bar = nullptr;
    int* merid_stats = nullptr;
    int solver_iterations = 0;
    double solver_max_residual = 0.0;
    int* err = nullptr;
    // node tables of the (r, z) field for the counter-based stream (sediment model 3, non-negative grid)
    int node_tables = 0;
    float2* node_mu = nullptr;     // [nr*nz]
    int2* node_alias = nullptr;    // [2][nr*nz][n]
    float* node_major = nullptr;   // [1]
    float node_major_host = 0.0f;
    double muscal_host[8] = {0}, sed_major_host[4] = {0};  // host copies of muscal and sed_major
};

// Buffers of enqueue_mie_phase (every one supplied by the caller).
struct MiePhaseBuffers {
    double* ab;       // [n][CLR_MIE_MAX_ORDER][4] a_n, b_n scratch
    int* nstop;       // [n]
    double *x, *qext, *qsca, *qabs, *qback, *g, *albedo;  // [n]
    double* theta;    // [nt]
    float* theta_f;   // [nt]
    double* pdf;      // [n][nt] scratch
    double* cdf;      // [n][nt]
    float* cdf_f;     // [n][nt]
    int* guide = nullptr;  // [n][kPhaseGuide + 1] search guide of cdf_f, or null (not built)
    int* err;         // error word, cleared by the call
};
cudaError_t enqueue_mie_phase(const double* d, const double* nr, const double* k, int n, double n_medium,
                              double wavelength, int nt, const MiePhaseBuffers& b, cudaStream_t stream);
// The same for a launch whose a_n/b_n rows are `order_cap` orders apart (mie_order_bound of its bins),
// placeholder tables instead of the phase tables when `hybrid` is false, and no reset of the error word;
// `fast_pdf` selects the FMA, two-angle phase pdf (CLR_TABLES_FAST) over the reference's order of operations.
cudaError_t enqueue_mie_tables(const double* d, const double* nr, const double* k, int n, double n_medium,
                               double wavelength, int nt, bool hybrid, int order_cap, const MiePhaseBuffers& b,
                               cudaStream_t stream, bool fast_pdf = false);
// Orders the Mie kernel needs for these bins (host arithmetic, with slack), at most CLR_MIE_MAX_ORDER.
int mie_order_bound(const double* d, const double* nr, const double* k, int n, double n_medium, double wavelength);
// Precompute error code of a Mie launch whose order bound was too small (not a reference code).
#define CLR_ERR_CODE_ORDER_CAP 90

// Scratch of the allocation-free Mie/phase entry point: file-scope __device__ arrays (noalloc.cu) of
// CLR_NOALLOC_MAX_BINS bins and CLR_NOALLOC_MAX_THETA angles, their addresses resolved once per device.
struct NoallocScratch {
    double *ab, *pdf, *x, *qabs, *qback, *albedo;
    float *theta_f, *cdf_f;
    int *nstop, *err;
};
// Resolves (once per device, with that device current) and returns the scratch addresses.
cudaError_t noalloc_scratch(int device, NoallocScratch* out);

// Enqueue the whole precompute on `stream`. Host inputs are copied in; error codes land in pb.err.
// `ab_scratch` may supply the Mie a_n/b_n scratch (n*CLR_MIE_MAX_ORDER*4 doubles); when null, pb.ab is used.
cudaError_t enqueue_particle_precompute(ParticleBuffers& pb, const clr_scene_params& sp, const clr_particle_spec& ps,
                                        const clr_sediment_spec& ss, double* ab_scratch, cudaStream_t stream);
// The meridional advection-diffusion field of sediment model 3 (one cooperative launch, a CTA per bin)
// into pb.sed_grid and pb.grid_max; pb.merid_* must be allocated (meridional_coef_doubles coefficients).
size_t meridional_coef_doubles(int n, int nr, int nz);
cudaError_t enqueue_meridional_solve(ParticleBuffers& pb, const clr_scene_params& sp, const clr_sediment_spec& ss,
                                     cudaStream_t stream);
// The part of it after the Mie tables (rates, sediment, node tables); pb's Mie outputs must be ready.
cudaError_t enqueue_scene_rates(ParticleBuffers& pb, const clr_scene_params& sp, const clr_particle_spec& ps,
                                const clr_sediment_spec& ss, cudaStream_t stream);
// The same for n scenarios at once (one launch each for the one-thread rate and majorant kernels);
// d_scratch: scene_rates_batch_scratch(n) bytes of device memory.
size_t scene_rates_batch_scratch(int n);
cudaError_t enqueue_scene_rates_batch(ParticleBuffers* const* pbs, const clr_scene_params* sps,
                                      const clr_particle_spec* pss, const clr_sediment_spec* sss, int n,
                                      void* d_scratch, cudaStream_t stream);

}  // namespace clr
