// C ABI of libclaritas_gb.so (declared in include/claritas_gb.h).
//
// A context owns one CUDA stream, the resident particle tables of the current
// scene, and the small per-run buffers (work counter, device tallies). All
// entry points return 0 or a negative CLR_ERR_* code; clr_last_error() gives
// the message. Configuration errors that the reference raises as ValueError in
// its constructor are rejected by the Python layer before reaching here; the
// checks below guard the ABI itself.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdarg>
#include <string>
#include <vector>
#include <algorithm>
#include <cuda_runtime.h>
#include "claritas_gb.h"
#include "kernels.h"

using namespace clr;

struct clr_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    bool scene_set = false, built = false;
    clr_scene_params sp{};
    ParticleBuffers pb{};
    std::vector<void*> allocs;
    // per-run device buffers (single scenario)
    DevScene* d_scene = nullptr;
    long long* d_chunk_begin = nullptr;
    DevTally* d_tally = nullptr;
    unsigned long long* d_work = nullptr;
    int num_sms = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_kernel_ms = 0.0f;
    // wavefront engine pool (allocated on first use)
    unsigned wave_cap = 0;
    void *wave_ray = nullptr, *wave_lane = nullptr;
    SlotMeta* wave_meta = nullptr;
    uint32_t* wave_q = nullptr;
    WaveCtl* wave_ctl = nullptr;
    long long* wave_begin = nullptr;
    unsigned* wave_live = nullptr;  // pinned
    cudaEvent_t wave_ev = nullptr;
    cudaEvent_t tail_ev[2] = {nullptr, nullptr};  // timing events around the tail kernel
    clr_engine_config engine = {};  // zeros: defaults
    int last_passes = 0;
    int last_tail = 0;
    unsigned last_tail_photons = 0;
    float last_tail_ms = 0.0f;
    long long last_launches = 0;
    int run_cap = 0;  // runs the per-run buffers hold
    // scenario sweep (clr_sweep_build): scene parameters and tables of every scenario, carved from one
    // arena; the Mie scratch (a_n/b_n rows and phase pdf of one chunk of bins) is kept between builds
    std::vector<clr_scene_params> sw_sp;
    std::vector<ParticleBuffers> sw_pb;
    void* sw_arena = nullptr;
    size_t sw_arena_bytes = 0;
    void* sw_scratch = nullptr;
    size_t sw_scratch_bytes = 0;
    void* sw_jobs = nullptr;  // job descriptions of the batched rate kernels
    size_t sw_jobs_bytes = 0;
    // light-history diagnostics (clr_set_light_diagnostics): host description, its device copy, buffers
    bool light_on = false;
    clr_light_config light_cfg{};
    LightDiag light{};
    LightDiag* d_light = nullptr;
    std::vector<void*> light_allocs;
    // particle-event provenance partitions (clr_set_path_provenance): the partitions and the per-slot state
    bool prov_on = false;
    clr_path_provenance* d_prov = nullptr;
    uint4* wave_prov = nullptr;
    uint4* d_prov_rec = nullptr;  // per-ray provenance of the last single-run trace with records
    long long prov_rec_cap = 0, prov_rec_n = 0;
};

static int fail(clr_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}
#define CU(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(ctx, CLR_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

static int run_buffers_ready(clr_ctx* ctx, int n);

static cudaError_t dalloc(clr_ctx* ctx, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e == cudaSuccess) ctx->allocs.push_back(*p);
    return e;
}
static void free_particles(clr_ctx* ctx) {
    for (void* p : ctx->allocs) cudaFree(p);
    ctx->allocs.clear();
    ctx->pb = ParticleBuffers{};
    ctx->built = false;
}

extern "C" {

const char* clr_version(void) { return "claritas_gb 0.1 (sm_103a)"; }

const char* clr_last_error(const clr_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int clr_create(clr_ctx** out, int device) {
    if (!out) return CLR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= device || device < 0) return CLR_ERR_CUDA;
    clr_ctx* ctx = new clr_ctx();
    ctx->device = device;
    CU(cudaSetDevice(device));
    CU(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    CU(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
    CU(cudaMalloc(&ctx->d_work, sizeof(unsigned long long)));
    {
        const int rc = run_buffers_ready(ctx, 1);
        if (rc != CLR_OK) return rc;
    }
    CU(cudaEventCreate(&ctx->ev0));
    CU(cudaEventCreate(&ctx->ev1));
    *out = ctx;
    return CLR_OK;
}

int clr_destroy(clr_ctx* ctx) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_particles(ctx);
    cudaFree(ctx->d_scene);
    cudaFree(ctx->d_chunk_begin);
    cudaFree(ctx->d_tally);
    cudaFree(ctx->d_work);
    cudaFree(ctx->wave_ray);
    cudaFree(ctx->wave_lane);
    cudaFree(ctx->wave_meta);
    cudaFree(ctx->wave_q);
    cudaFree(ctx->wave_ctl);
    cudaFree(ctx->wave_begin);
    cudaFree(ctx->sw_arena);
    cudaFree(ctx->sw_scratch);
    cudaFree(ctx->sw_jobs);
    for (void* p : ctx->light_allocs) cudaFree(p);
    cudaFree(ctx->d_prov);
    cudaFree(ctx->wave_prov);
    cudaFree(ctx->d_prov_rec);
    if (ctx->wave_live) cudaFreeHost(ctx->wave_live);
    if (ctx->wave_ev) cudaEventDestroy(ctx->wave_ev);
    for (cudaEvent_t e : ctx->tail_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return CLR_OK;
}

}  // extern "C"

static int check_scene(clr_ctx* ctx, const clr_scene_params& s) {
    if (!(0 < s.rin && s.rin < s.rout && s.rout < s.ring_in && s.ring_in < s.throat_out &&
          s.throat_out <= s.source_r && s.source_r <= s.ring_out))
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "TARDIIS radial/source geometry is inconsistent");
    if (!(s.zwall_top > s.zmean && s.zmean > s.zmin))
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "wall top must lie above the water domain");
    if (s.free_surface_model < 0 || s.free_surface_model > 3 || s.sediment_model < 0 || s.sediment_model > 3 ||
        s.event_model < 0 || s.event_model > 5)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "model code out of range");
    if (s.source_kind != CLR_SOURCE_REFERENCE_LED && s.source_kind != CLR_SOURCE_COLLIMATED_DISC)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "unknown source_kind %d", s.source_kind);
    if (s.free_surface_model == 3 && s.vortex_delta_h > 0.0f && !(s.vortex_core_radius > 0.0f))
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "the Rankine vortex surface needs a positive core radius");
    if (s.free_surface_model == 3 && (s.sediment_model == 1 || s.sediment_model == 2))
        return fail(ctx, CLR_ERR_UNSUPPORTED,
                    "the analytic drift-diffusion sediment fields are defined for the reference's free surfaces; "
                    "with the Rankine vortex use a uniform or a supplied (r, z) field");
    if (!(s.water_absorption >= 0.0f) || !std::isfinite(s.water_absorption))
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "water_absorption must be finite and nonnegative");
    return CLR_OK;
}

static bool hybrid_model(const clr_scene_params& sp) {
    return sp.event_model == 3 || sp.event_model == 4 || sp.event_model == 5;
}

// Argument checks of a particle build for scene sp (including the reference's sediment precompute
// error codes 31-33, :3958-3967).
static int check_particles(clr_ctx* ctx, const clr_scene_params& sp, const clr_particle_spec* ps,
                           const clr_sediment_spec* ss) {
    const int n = ps->n_bins;
    if (n < 1 || n > CLR_MAX_BINS) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "n_bins must be 1..%d", CLR_MAX_BINS);
    if (hybrid_model(sp) && ps->n_theta < 257) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "n_theta must be >= 257");
    if (!ps->diameter_m || !ps->weight || !ps->n_real || !ps->k_imag)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "particle arrays must not be null");
    if (ps->table_arithmetic != CLR_TABLES_REFERENCE && ps->table_arithmetic != CLR_TABLES_FAST)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "unknown table_arithmetic %d", ps->table_arithmetic);
    if (ss->n_radial < 65 || ss->n_quad < 64) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "sediment lookup sizes too small");
    if (sp.sediment_model != 0) {
        if (!(ss->particle_density > ss->water_density) || !(ss->water_density > 0.0) || !(ss->water_viscosity > 0.0) ||
            !(ss->gravity > 0.0) || !(ss->eddy_diffusivity > 0.0) || !(sp.rin > 0.0f))
            return fail(ctx, CLR_ERR_PRECOMPUTE, "sediment transport precompute failed with error code 31");
        if ((sp.vortex_delta_h > 0.0f && sp.free_surface_model == 0) ||
            (sp.free_surface_model == 2 && !(sp.vortex_core_radius > 0.0f)))
            return fail(ctx, CLR_ERR_PRECOMPUTE, "sediment transport precompute failed with error code 32");
        if (!((double)sp.zmean - (double)sp.zmin > 0.0))
            return fail(ctx, CLR_ERR_PRECOMPUTE, "sediment transport precompute failed with error code 33");
        if (sp.sediment_model == 3 && ss->grid && (ss->grid_nr < 2 || ss->grid_nz < 2))
            return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "a supplied model-3 grid needs at least 2 x 2 cells");
        if (sp.sediment_model == 3 && !ss->grid && sp.free_surface_model == 3)
            return fail(ctx, CLR_ERR_UNSUPPORTED,
                        "the meridional field solver follows the reference's free surfaces; with the Rankine vortex "
                        "supply the (r, z) field");
        if (sp.sediment_model == 3 && !ss->grid) {
            // the reference's constructor rules for the solver settings (:5867-5887)
            if (ss->meridional_nr < 16 || ss->meridional_nz < 32)
                return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "meridional grid must be at least 16 x 32 cells");
            if (ss->solver_max_iterations < 250 || ss->solver_check_interval < 10)
                return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "meridional solver needs >= 250 iterations, checks every >= 10");
            if (!(ss->solver_tolerance > 0.0 && ss->solver_tolerance < 1e-2))
                return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "meridional_solver_tolerance must be in (0,1e-2)");
            if (!(ss->solver_sor >= 1.0 && ss->solver_sor < 1.95))
                return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "meridional_solver_sor must be in [1,1.95)");
            if (!(ss->meridional_peak_speed >= 0.0) || !(ss->grid_zmax > (double)sp.zmin))
                return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "meridional peak speed and grid top must be valid");
            if ((size_t)ss->meridional_nr * ss->meridional_nz * 9 > 200 * 1024)
                return fail(ctx, CLR_ERR_UNSUPPORTED, "meridional grid of %d x %d cells exceeds one CTA's shared memory",
                            ss->meridional_nr, ss->meridional_nz);
            if (n > 152) return fail(ctx, CLR_ERR_UNSUPPORTED, "meridional solver runs one CTA per bin (<= 152)");
        }
    }
    return CLR_OK;
}

// The sediment spec with its FP64 geometry filled from the scene where the caller left it zero.
static clr_sediment_spec filled_sediment(const clr_scene_params& sp, const clr_sediment_spec& ss) {
    clr_sediment_spec o = ss;
    if (!(o.rin > 0.0)) {
        o.rin = (double)sp.rin; o.zmin = (double)sp.zmin; o.zmean = (double)sp.zmean;
        o.vortex_delta_h = (double)sp.vortex_delta_h; o.vortex_core_radius = (double)sp.vortex_core_radius;
    }
    return o;
}

// The (r, z) grid of a model-3 scene: the supplied one's shape or the solver's.
static bool solves_grid(const clr_scene_params& sp, const clr_sediment_spec& ss) {
    return sp.sediment_model == 3 && !ss.grid;
}
static int grid_nr_of(const clr_scene_params& sp, const clr_sediment_spec& ss) {
    return sp.sediment_model != 3 ? 2 : (ss.grid ? ss.grid_nr : ss.meridional_nr);
}
static int grid_nz_of(const clr_scene_params& sp, const clr_sediment_spec& ss) {
    return sp.sediment_model != 3 ? 2 : (ss.grid ? ss.grid_nz : ss.meridional_nz);
}

// Node tables pay off (and are exact) for a model-3 grid with no negative value and a moderate size.
// (A solved field is positive everywhere: the solver clamps at 1e-14 and extends from liquid cells.)
static bool wants_node_tables(const clr_scene_params& sp, const clr_sediment_spec& ss, int n, size_t grid_cells) {
    if (sp.sediment_model != 3) return false;
    bool nonneg = ss.grid_zmax > (double)sp.zmin;
    if (ss.grid)
        for (size_t c = 0; c < grid_cells && nonneg; ++c) nonneg = ss.grid[c] >= 0.0;
    const size_t plane = (size_t)grid_nr_of(sp, ss) * grid_nz_of(sp, ss);
    return nonneg && 2 * plane * n * sizeof(int2) <= (size_t(1) << 30);
}

extern "C" {

int clr_set_scene(clr_ctx* ctx, const clr_scene_params* scene) {
    if (!ctx || !scene) return CLR_ERR_INVALID_ARGUMENT;
    const clr_scene_params& s = *scene;
    const int rc = check_scene(ctx, s);
    if (rc != CLR_OK) return rc;
    ctx->sp = s;
    ctx->scene_set = true;
    ctx->built = false;
    return CLR_OK;
}

int clr_build_particles(clr_ctx* ctx, const clr_particle_spec* ps, const clr_sediment_spec* ss_in) {
    if (!ctx || !ps || !ss_in) return CLR_ERR_INVALID_ARGUMENT;
    if (!ctx->scene_set) return fail(ctx, CLR_ERR_NOT_READY, "clr_set_scene must be called first");
    const clr_scene_params& sp = ctx->sp;
    {
        const int rc = check_particles(ctx, sp, ps, ss_in);
        if (rc != CLR_OK) return rc;
    }
    const clr_sediment_spec sse = filled_sediment(sp, *ss_in);
    const clr_sediment_spec* ss = &sse;
    const int n = ps->n_bins;
    const int nt = hybrid_model(sp) ? ps->n_theta : 2;
    CU(cudaSetDevice(ctx->device));
    free_particles(ctx);
    ParticleBuffers& pb = ctx->pb;
    pb.n = n; pb.nt = nt; pb.n_radial = ss->n_radial;
    pb.grid_nr = grid_nr_of(sp, *ss);
    pb.grid_nz = grid_nz_of(sp, *ss);
    pb.grid_zmax = ss->grid_zmax;
    auto D = [&](double** p, size_t cnt) { return dalloc(ctx, (void**)p, cnt * sizeof(double)); };
    auto F = [&](float** p, size_t cnt) { return dalloc(ctx, (void**)p, cnt * sizeof(float)); };
    double** darr[] = {&pb.d, &pb.w, &pb.nidx, &pb.kidx, &pb.x, &pb.qext, &pb.qsca, &pb.qabs, &pb.qback, &pb.g,
                       &pb.albedo, &pb.radius, &pb.nden, &pb.mug, &pb.mus, &pb.mue, &pb.muw, &pb.muev, &pb.gcdf,
                       &pb.wcdf, &pb.pcdf, &pb.moment_a, &pb.moment_b, &pb.trace_geom, &pb.trace_wave, &pb.sedA,
                       &pb.sedB, &pb.sed_norm, &pb.sed_max, &pb.grid_max, &pb.sed_ws};
    for (double** p : darr) CU(D(p, n));
    float** farr[] = {&pb.gcdf_f, &pb.wcdf_f, &pb.pn_f, &pb.pk_f, &pb.prad_f};
    for (float** p : farr) CU(F(p, n));
    CU(dalloc(ctx, (void**)&pb.nstop, n * sizeof(int)));
    CU(dalloc(ctx, (void**)&pb.moment_mode, n));
    CU(dalloc(ctx, (void**)&pb.err, sizeof(int)));
    CU(D(&pb.ab, (size_t)n * CLR_MIE_MAX_ORDER * 4));
    CU(D(&pb.theta, nt));
    CU(F(&pb.theta_f, nt));
    CU(D(&pb.pdf, (size_t)n * nt));
    CU(D(&pb.phase_cdf, (size_t)n * nt));
    CU(F(&pb.phase_cdf_f, (size_t)n * nt));
    CU(dalloc(ctx, (void**)&pb.phase_guide, (size_t)n * (kPhaseGuide + 1) * sizeof(int)));
    CU(D(&pb.muscal, 8));
    CU(D(&pb.sed_major, 4));
    CU(D(&pb.sed_radial_log, (size_t)n * ss->n_radial));
    CU(D(&pb.sed_wr, (size_t)n * ss->n_radial));
    CU(D(&pb.sed_terms, (size_t)n * ss->n_quad));
    const size_t grid_cells = (size_t)pb.grid_nr * pb.grid_nz * (sp.sediment_model == 3 ? n : 1);
    CU(D(&pb.sed_grid, grid_cells));
    cudaStream_t st = ctx->stream;
    CU(cudaMemcpyAsync(pb.d, ps->diameter_m, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(pb.w, ps->weight, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(pb.nidx, ps->n_real, n * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(pb.kidx, ps->k_imag, n * sizeof(double), cudaMemcpyHostToDevice, st));
    std::vector<double> ma(n, 1.0), mb(n, 0.0);
    std::vector<uint8_t> mm(n, 0);
    pb.any_moment = 0;
    if (ps->moment_enabled && ps->moment_a && ps->moment_b && ps->moment_mode) {
        for (int i = 0; i < n; ++i) {
            ma[i] = ps->moment_a[i]; mb[i] = ps->moment_b[i]; mm[i] = ps->moment_mode[i];
            pb.any_moment |= mm[i] ? 1 : 0;
        }
    }
    CU(cudaMemcpyAsync(pb.moment_a, ma.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(pb.moment_b, mb.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(pb.moment_mode, mm.data(), n, cudaMemcpyHostToDevice, st));
    if (sp.sediment_model == 3) {
        const size_t plane = (size_t)pb.grid_nr * pb.grid_nz;
        if (wants_node_tables(sp, *ss, n, grid_cells)) {
            pb.node_tables = 1;
            CU(dalloc(ctx, (void**)&pb.node_mu, plane * sizeof(float2)));
            CU(dalloc(ctx, (void**)&pb.node_alias, 2 * plane * n * sizeof(int2)));
            CU(dalloc(ctx, (void**)&pb.node_major, sizeof(float)));
        }
        if (ss->grid) {
            CU(cudaMemcpyAsync(pb.sed_grid, ss->grid, grid_cells * sizeof(double), cudaMemcpyHostToDevice, st));
        } else {
            CU(D(&pb.merid_coef, meridional_coef_doubles(n, pb.grid_nr, pb.grid_nz)));
            CU(D(&pb.merid_residual, 2 * (size_t)n + 1));
            CU(dalloc(ctx, (void**)&pb.merid_bar, 2 * sizeof(unsigned)));
            CU(dalloc(ctx, (void**)&pb.merid_stats, sizeof(int)));
        }
    } else {
        const double one[4] = {1.0, 1.0, 1.0, 1.0};
        CU(cudaMemcpyAsync(pb.sed_grid, one, sizeof(double), cudaMemcpyHostToDevice, st));
    }
    CU(enqueue_particle_precompute(pb, sp, *ps, *ss, nullptr, st));  // ss: FP64 geometry filled
    int herr = 0;
    CU(cudaMemcpyAsync(&herr, pb.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (pb.node_tables)
        CU(cudaMemcpyAsync(&pb.node_major_host, pb.node_major, sizeof(float), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(pb.muscal_host, pb.muscal, 8 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(pb.sed_major_host, pb.sed_major, 4 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (pb.merid_coef) {
        CU(cudaMemcpyAsync(&pb.solver_iterations, pb.merid_stats, sizeof(int), cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(&pb.solver_max_residual, pb.merid_residual + 2 * (size_t)n, sizeof(double),
                           cudaMemcpyDeviceToHost, st));
    }
    CU(cudaStreamSynchronize(st));
    if (herr) return fail(ctx, CLR_ERR_PRECOMPUTE, "particle precompute failed with error code %d", herr);
    if (pb.merid_coef && pb.solver_max_residual > ss->solver_tolerance)
        return fail(ctx, CLR_ERR_PRECOMPUTE,
                    "meridional transport solver did not converge: max residual=%.6g after %d iterations",
                    pb.solver_max_residual, pb.solver_iterations);
    ctx->built = true;
    return CLR_OK;
}

int clr_read_sediment_field(clr_ctx* ctx, double* grid_out, int32_t* nr, int32_t* nz, int32_t* iterations,
                            double* max_residual) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    if (!ctx->built) return fail(ctx, CLR_ERR_NOT_READY, "particles not built");
    const ParticleBuffers& pb = ctx->pb;
    if (ctx->sp.sediment_model != 3) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "the scene has no (r,z) field");
    if (nr) *nr = pb.grid_nr;
    if (nz) *nz = pb.grid_nz;
    if (iterations) *iterations = pb.merid_coef ? pb.solver_iterations : 0;
    if (max_residual) *max_residual = pb.merid_coef ? pb.solver_max_residual : 0.0;
    if (grid_out) {
        CU(cudaSetDevice(ctx->device));
        CU(cudaMemcpyAsync(grid_out, pb.sed_grid, (size_t)pb.n * pb.grid_nr * pb.grid_nz * sizeof(double),
                           cudaMemcpyDeviceToHost, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
    }
    return CLR_OK;
}

}  // extern "C"

static int read_physics(clr_ctx* ctx, const ParticleBuffers& pb, clr_particle_physics* o) {
    const int n = pb.n;
    CU(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    struct Pair { double* dst; const double* src; size_t cnt; };
    Pair pairs[] = {{o->size_parameter, pb.x, (size_t)n}, {o->qext, pb.qext, (size_t)n}, {o->qsca, pb.qsca, (size_t)n},
                    {o->qabs, pb.qabs, (size_t)n}, {o->qback, pb.qback, (size_t)n}, {o->asym_g, pb.g, (size_t)n},
                    {o->albedo, pb.albedo, (size_t)n}, {o->radius, pb.radius, (size_t)n},
                    {o->number_density, pb.nden, (size_t)n}, {o->mu_geom_bin, pb.mug, (size_t)n},
                    {o->mu_sca_bin, pb.mus, (size_t)n}, {o->mu_ext_bin, pb.mue, (size_t)n},
                    {o->mu_wave_bin, pb.muw, (size_t)n}, {o->mu_event_bin, pb.muev, (size_t)n},
                    {o->trace_geom_bin, pb.trace_geom, (size_t)n}, {o->trace_wave_bin, pb.trace_wave, (size_t)n},
                    {o->geometric_cdf, pb.gcdf, (size_t)n}, {o->wave_cdf, pb.wcdf, (size_t)n},
                    {o->particle_event_cdf, pb.pcdf, (size_t)n}, {o->mu_scalars, pb.muscal, 8},
                    {o->sed_majorants, pb.sed_major, 4}, {o->theta, pb.theta, (size_t)pb.nt},
                    {o->phase_cdf, pb.phase_cdf, (size_t)n * pb.nt}};
    for (const Pair& p : pairs)
        if (p.dst) CU(cudaMemcpyAsync(p.dst, p.src, p.cnt * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (o->nstop) CU(cudaMemcpyAsync(o->nstop, pb.nstop, n * sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return CLR_OK;
}

extern "C" int clr_read_particle_physics(clr_ctx* ctx, clr_particle_physics* o) {
    if (!ctx || !o) return CLR_ERR_INVALID_ARGUMENT;
    if (!ctx->built) return fail(ctx, CLR_ERR_NOT_READY, "particles not built");
    return read_physics(ctx, ctx->pb, o);
}

// Fill the device scene description for the current tables and a run.
static void fill_scene(const clr_scene_params& sp, const ParticleBuffers& pb, const clr_run_params* run, DevScene* s) {
    memset(s, 0, sizeof *s);
    s->P = sp;
    s->gcdf = pb.gcdf_f; s->wcdf = pb.wcdf_f; s->phase_cdf = pb.phase_cdf_f; s->theta = pb.theta_f;
    s->phase_guide = pb.phase_guide;
    s->pn = pb.pn_f; s->pk = pb.pk_f; s->prad = pb.prad_f;
    s->k = pb.kidx; s->qsca = pb.qsca; s->qext = pb.qext;
    s->moment_a = pb.moment_a; s->moment_b = pb.moment_b; s->moment_mode = pb.moment_mode;
    s->trace_geom = pb.trace_geom; s->trace_wave = pb.trace_wave;
    s->sedA = pb.sedA; s->sedB = pb.sedB; s->sed_norm = pb.sed_norm; s->sed_radial_log = pb.sed_radial_log;
    s->sed_grid = pb.sed_grid; s->mu_channels = pb.muscal; s->sed_major = pb.sed_major;
    s->n_bins = pb.n; s->nt = pb.nt; s->n_radial = pb.n_radial; s->grid_nr = pb.grid_nr; s->grid_nz = pb.grid_nz;
    s->any_moment = pb.any_moment; s->grid_zmax = (float)pb.grid_zmax;
    const bool node = pb.node_tables && !(run->flags & CLR_RUN_EXACT_SAMPLERS);
    s->node_mu = node ? pb.node_mu : nullptr;
    s->node_alias = node ? pb.node_alias : nullptr;
    s->node_major = pb.node_major_host;
    s->mu_geom_f = (float)pb.muscal_host[0]; s->mu_wave_f = (float)pb.muscal_host[1];
    s->coherent_f = (float)pb.muscal_host[7];
    s->sed_major_f[0] = (float)pb.sed_major_host[0]; s->sed_major_f[1] = (float)pb.sed_major_host[1];
    s->seed0 = run->seed0; s->seed1 = run->seed1; s->seed2 = run->seed2; s->det_seed = run->detector_seed;
    s->ray_offset = run->ray_offset; s->scenario_id = run->scenario_id; s->philox_key = run->philox_key;
    s->n_rays = run->n_rays; s->weight_mode = run->weight_mode;
    s->roulette_threshold = run->roulette_threshold; s->roulette_survival = run->roulette_survival;
}

static void tally_to_host(const DevTally& d, clr_tallies* out, int64_t n_rays) {
    const TallyCore& t = d.c;
    memset(out, 0, sizeof *out);
    out->n_rays = n_rays;
    for (int j = 0; j < CLR_N_DETECTORS; ++j) {
        out->hw_native[j] = (int64_t)t.hw[0][j]; out->hw_mirror[j] = (int64_t)t.hw[1][j];
        out->hw_native_direct[j] = (int64_t)t.hw[2][j]; out->hw_mirror_direct[j] = (int64_t)t.hw[3][j];
        out->hw_native_stray[j] = (int64_t)t.hw[4][j]; out->hw_mirror_stray[j] = (int64_t)t.hw[5][j];
        out->hw_native_face[j] = (int64_t)t.hw[6][j]; out->hw_mirror_face[j] = (int64_t)t.hw[7][j];
        out->legacy_native[j] = (int64_t)t.hw[8][j]; out->legacy_mirror[j] = (int64_t)t.hw[9][j];
        out->photodiode_native[j] = t.sums[0][j]; out->photodiode_mirror[j] = t.sums[1][j];
        out->incidence_native_sum[j] = t.sums[2][j]; out->incidence_mirror_sum[j] = t.sums[3][j];
        out->weight_native[j] = t.sums[4][j]; out->weight_mirror[j] = t.sums[5][j];
        out->weight_sq_native[j] = t.sums[6][j]; out->weight_sq_mirror[j] = t.sums[7][j];
    }
    for (int k = 0; k < CLR_N_STATUS; ++k) out->status_counts[k] = (int64_t)t.status[k];
    for (int k = 0; k < CLR_N_FAILURE_CODES; ++k) out->failure_code_counts[k] = (int64_t)t.failure[k];
    for (int k = 0; k < CLR_N_EVENT_COUNTERS; ++k) out->event_counts[k] = (int64_t)t.events[k];
    out->event_counts[CLR_EV_ROULETTE_KILLS] = (int64_t)t.status[CLR_STATUS_ROULETTE];
    for (int k = 0; k < CLR_N_CONDITIONAL_STATS; ++k) out->conditional_stats[k] = t.cstats[k];
    for (int k = 0; k < 16; ++k) { out->entered_sums[k] = (int64_t)t.entered_sums[k]; out->ray_flags[k] = (int64_t)t.ray_flags[k]; }
    for (int k = 0; k < CLR_N_SUBCODES; ++k) out->failure_subcode_counts[k] = (int64_t)t.subcodes[k];
    for (int k = 0; k < CLR_IC_HIST; ++k) out->ic_hist[k] = (int64_t)d.ic_hi[k] + (k < 64 ? (int64_t)t.ic_lo[k] : 0);
    for (int k = 0; k < 16; ++k) out->sched_stats[k] = (int64_t)d.sched[k];
    for (int side = 0; side < 2; ++side)
        for (int j = 0; j < CLR_N_DETECTORS; ++j) {
            for (int o = 0; o < 6; ++o) {
                out->order_hits[side][o][j] = (int64_t)d.pd.order[side][o][j];
                out->geometric_order_hits[side][o][j] = (int64_t)d.pd.geom_order[side][o][j];
            }
            for (int k = 0; k < CLR_N_PATH_SUMS; ++k) out->path_sums[k][side][j] = (int64_t)d.pd.sums[k][side][j];
            for (int k = 0; k < CLR_N_PATH_MASKS; ++k) out->path_mask_hits[side][k][j] = (int64_t)d.pd.masks[side][k][j];
            for (int k = 0; k < 5; ++k) out->acrylic_order_hits[side][k][j] = (int64_t)d.pd.acrylic_order[side][k][j];
        }
    out->device_error = (t.n_done == (unsigned long long)n_rays) ? 0 : 1;
}

// Photon pool of the wavefront engine: 2^21 slots (about 640 MB with the queue rings), allocated once per context.
static int wave_pool_ready(clr_ctx* ctx) {
    if (ctx->wave_cap) return CLR_OK;
    const unsigned cap = 1u << 21;
    const size_t lane = std::max(wave_lane_bytes(CLR_RNG_PHILOX), wave_lane_bytes(CLR_RNG_REFERENCE_XORSHIFT));
    CU(cudaMalloc(&ctx->wave_ray, (size_t)cap * wave_ray_bytes()));
    CU(cudaMalloc(&ctx->wave_lane, (size_t)cap * lane));
    CU(cudaMalloc(&ctx->wave_meta, (size_t)cap * sizeof(SlotMeta)));
    CU(cudaMalloc(&ctx->wave_q, (size_t)CLR_WQ_COUNT * 2 * cap * sizeof(uint32_t)));  // rings of 2 * cap
    CU(cudaMalloc(&ctx->wave_ctl, sizeof(WaveCtl)));
    CU(cudaHostAlloc((void**)&ctx->wave_live, 4 * sizeof(unsigned), cudaHostAllocDefault));
    CU(cudaEventCreateWithFlags(&ctx->wave_ev, cudaEventDisableTiming));
    CU(cudaEventCreate(&ctx->tail_ev[0]));
    CU(cudaEventCreate(&ctx->tail_ev[1]));
    ctx->wave_cap = cap;
    return CLR_OK;
}

// Per-run buffers (scene descriptions, work-chunk and photon prefixes, tallies) for up to n runs.
static int run_buffers_ready(clr_ctx* ctx, int n) {
    if (n <= ctx->run_cap) return CLR_OK;
    int cap = std::max(n, 2 * ctx->run_cap);
    cudaFree(ctx->d_scene); cudaFree(ctx->d_chunk_begin); cudaFree(ctx->d_tally); cudaFree(ctx->wave_begin);
    ctx->d_scene = nullptr; ctx->d_chunk_begin = nullptr; ctx->d_tally = nullptr; ctx->wave_begin = nullptr;
    ctx->run_cap = 0;
    CU(cudaMalloc(&ctx->d_scene, (size_t)cap * sizeof(DevScene)));
    CU(cudaMalloc(&ctx->d_chunk_begin, (size_t)(cap + 1) * sizeof(long long)));
    CU(cudaMalloc(&ctx->d_tally, (size_t)cap * sizeof(DevTally)));
    CU(cudaMalloc(&ctx->wave_begin, (size_t)(cap + 1) * sizeof(long long)));
    ctx->run_cap = cap;
    return CLR_OK;
}

// The scene and tables a run traces.
struct SceneRef {
    const clr_scene_params* sp;
    const ParticleBuffers* pb;
};

// Traces n runs in one engine execution (one launch of the persistent kernel or one sequence of
// wavefront passes), each run with its own scene, photon range, seeds and tallies.
static int trace_runs(clr_ctx* ctx, const SceneRef* refs, const clr_run_params* runs, int n, clr_tallies* outs,
                      clr_ray_record* d_records, const LightDiag* d_light = nullptr, bool prov = false) {
    if (!ctx || !runs || !outs || n < 1) return CLR_ERR_INVALID_ARGUMENT;
    if (d_records && n != 1) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "per-ray records need a single run");
    const clr_run_params& r0 = runs[0];
    for (int i = 0; i < n; ++i) {
        const clr_run_params* run = runs + i;
        if (run->n_rays < 0 || (uint64_t)run->ray_offset + (uint64_t)run->n_rays > (1ull << 32))
            return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "run %d: ray range exceeds uint32 global ids", i);
        if (run->rng_mode != CLR_RNG_REFERENCE_XORSHIFT && run->rng_mode != CLR_RNG_PHILOX)
            return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "run %d: unknown rng_mode %d", i, run->rng_mode);
        if (run->weight_mode != CLR_WEIGHT_ANALOG && run->weight_mode != CLR_WEIGHT_IMPLICIT)
            return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "run %d: unknown weight_mode %d", i, run->weight_mode);
        if (run->weight_mode == CLR_WEIGHT_IMPLICIT && run->rng_mode != CLR_RNG_PHILOX)
            return fail(ctx, CLR_ERR_UNSUPPORTED, "implicit-capture weighting runs on the Philox stream only");
        if (run->weight_mode == CLR_WEIGHT_IMPLICIT &&
            !(run->roulette_threshold >= 0.0f && run->roulette_survival > run->roulette_threshold &&
              run->roulette_survival <= 1.0f))
            return fail(ctx, CLR_ERR_INVALID_ARGUMENT,
                        "run %d: Russian roulette needs 0 <= roulette_threshold < roulette_survival <= 1 (got %g, %g)",
                        i, (double)run->roulette_threshold, (double)run->roulette_survival);
        if (run->rng_mode != r0.rng_mode || run->weight_mode != r0.weight_mode || run->flags != r0.flags)
            return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "runs of one call must share rng_mode, weight_mode and flags");
        // closure trials draw from substreams numbered in 14 bits of a counter word on the Philox stream
        if (run->rng_mode == CLR_RNG_PHILOX && refs[i].sp && refs[i].sp->conditional_retries > 16384)
            return fail(ctx, CLR_ERR_UNSUPPORTED, "run %d: the Philox stream allows at most 16384 closure trials "
                        "(conditional_retries %d)", i, refs[i].sp->conditional_retries);
    }
    const bool persistent = (r0.flags & CLR_RUN_PERSISTENT_KERNEL) != 0;
    if (prov && persistent)
        return fail(ctx, CLR_ERR_UNSUPPORTED, "particle-event provenance is counted by the wavefront engine only");
    CU(cudaSetDevice(ctx->device));
    int rc = run_buffers_ready(ctx, n);
    if (rc != CLR_OK) return rc;
    cudaStream_t st = ctx->stream;
    if (prov) CU(cudaMemsetAsync(ctx->d_prov, 0, sizeof(clr_path_provenance), st));
    ctx->prov_rec_n = 0;
    if (prov && d_records) {  // per-ray provenance beside the per-ray records
        const long long need = std::max((long long)r0.n_rays, 1LL);
        if (ctx->prov_rec_cap < need) {
            cudaFree(ctx->d_prov_rec);
            ctx->d_prov_rec = nullptr;
            ctx->prov_rec_cap = 0;
            CU(cudaMalloc((void**)&ctx->d_prov_rec, (size_t)need * sizeof(uint4)));
            ctx->prov_rec_cap = need;
        }
        ctx->prov_rec_n = r0.n_rays;
    }
    std::vector<DevScene> hs(n);
    std::vector<long long> cb(n + 1), rb(n + 1);
    const int chunk = r0.rays_per_item > 0 ? r0.rays_per_item : 256;
    cb[0] = 0; rb[0] = 0;
    long long max_iter = 0;
    for (int i = 0; i < n; ++i) {
        fill_scene(*refs[i].sp, *refs[i].pb, runs + i, &hs[i]);
        hs[i].light = d_light;
        hs[i].prov = prov ? ctx->d_prov : nullptr;
        max_iter = std::max(max_iter, (long long)refs[i].sp->max_iterations);
        cb[i + 1] = cb[i] + (runs[i].n_rays + chunk - 1) / chunk;
        rb[i + 1] = rb[i] + runs[i].n_rays;
    }
    const long long total = rb[n];
    CU(cudaMemcpyAsync(ctx->d_scene, hs.data(), n * sizeof(DevScene), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(ctx->d_chunk_begin, cb.data(), (n + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(ctx->d_tally, 0, n * sizeof(DevTally), st));
    CU(cudaMemsetAsync(ctx->d_work, 0, sizeof(unsigned long long), st));
    LaunchArgs a;
    a.scenes = ctx->d_scene; a.chunk_begin = ctx->d_chunk_begin; a.n_scen = n; a.n_chunks = cb[n];
    a.chunk_rays = chunk; a.work = ctx->d_work; a.tallies = ctx->d_tally; a.records = d_records;
    a.stream = st; a.rng_mode = r0.rng_mode; a.weighted = r0.weight_mode == CLR_WEIGHT_IMPLICIT;
    int occ = photon_kernel_occupancy(a.rng_mode, d_records != nullptr, a.weighted);
    if (occ < 1) occ = 1;
    long long want = (long long)ctx->num_sms * occ;
    long long blocks_needed = (cb[n] * 32 + CLR_TRACE_THREADS - 1) / CLR_TRACE_THREADS;  // a chunk per warp at most
    a.grid = (int)std::max(1LL, std::min(want, blocks_needed));
    if (r0.max_blocks > 0) a.grid = std::max(1, std::min(a.grid, r0.max_blocks));
    WaveLaunch w{};
    if (!persistent) {
        rc = wave_pool_ready(ctx);
        if (rc != CLR_OK) return rc;
        CU(cudaMemcpyAsync(ctx->wave_begin, rb.data(), (n + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
        w.scenes = ctx->d_scene; w.n_scen = n; w.ray_begin = ctx->wave_begin; w.total = (unsigned long long)total;
        w.tallies = ctx->d_tally; w.records = d_records;
        w.ray = ctx->wave_ray; w.lane = ctx->wave_lane; w.meta = ctx->wave_meta; w.qbuf = ctx->wave_q;
        w.ctl = ctx->wave_ctl; w.cap = ctx->wave_cap; w.host_live = ctx->wave_live; w.flag_event = ctx->wave_ev;
        w.tail_begin = ctx->tail_ev[0]; w.tail_end = ctx->tail_ev[1];
        const clr_engine_config& ec = ctx->engine;
        w.flight_steps = ec.flight_steps > 0 ? ec.flight_steps : CLR_ENGINE_DEFAULT_FLIGHT_STEPS;
        w.tail_photons = ec.tail_photons > 0 ? (unsigned)ec.tail_photons : CLR_ENGINE_DEFAULT_TAIL_PHOTONS;
        w.rare_batch = ec.rare_batch > 0 ? (unsigned)ec.rare_batch : CLR_ENGINE_DEFAULT_RARE_BATCH;
        for (int q = 0; q < CLR_N_STAGES; ++q) w.stage_blocks[q] = std::max(0, ec.stage_blocks[q]);
        w.pass_batch = ec.pass_batch > 0 ? ec.pass_batch : CLR_ENGINE_DEFAULT_PASS_BATCH;
        w.acr_budget = ec.acr_budget > 0 ? ec.acr_budget : CLR_ENGINE_DEFAULT_ACR_BUDGET;
        w.light = d_light != nullptr;
        w.prov = prov ? ctx->wave_prov : nullptr;
        w.prov_rec = ctx->prov_rec_n > 0 ? ctx->d_prov_rec : nullptr;
    }
    CU(cudaEventRecord(ctx->ev0, st));
    ctx->last_passes = 0;
    ctx->last_launches = 0;
    ctx->last_tail = 0;
    ctx->last_tail_photons = 0;
    ctx->last_tail_ms = 0.0f;
    if (persistent) {
        if (cb[n] > 0) CU(launch_photon_kernel(a));
        ctx->last_launches = cb[n] > 0 ? 1 : 0;
    } else if (total > 0) {
        const long long max_passes = 100000 + 8LL * max_iter;
        WaveRunInfo info;
        cudaError_t e = a.rng_mode == CLR_RNG_PHILOX ? wave_run_philox(w, ctx->num_sms, st, max_passes, &info)
                                                     : wave_run_xor(w, ctx->num_sms, st, max_passes, &info);
        if (e == cudaErrorLaunchTimeout)
            return fail(ctx, CLR_ERR_DEVICE_TIMEOUT, "wavefront engine did not drain within %lld passes", max_passes);
        CU(e);
        ctx->last_passes = info.passes;
        ctx->last_tail = info.tail;
        ctx->last_tail_photons = info.tail_photons;
        ctx->last_launches = 1 + (long long)info.passes * (1 + CLR_WQ_COUNT) + info.tail;
    }
    CU(cudaEventRecord(ctx->ev1, st));
    std::vector<DevTally> ht(n);
    CU(cudaMemcpyAsync(ht.data(), ctx->d_tally, n * sizeof(DevTally), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    CU(cudaEventElapsedTime(&ctx->last_kernel_ms, ctx->ev0, ctx->ev1));
    if (ctx->last_tail) CU(cudaEventElapsedTime(&ctx->last_tail_ms, ctx->tail_ev[0], ctx->tail_ev[1]));
    for (int i = 0; i < n; ++i) tally_to_host(ht[i], outs + i, runs[i].n_rays);
    return CLR_OK;
}

// Runs of the current scene (clr_set_scene + clr_build_particles).
static int trace_current(clr_ctx* ctx, const clr_run_params* runs, int n, clr_tallies* outs, clr_ray_record* d_records) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    if (!ctx->built) return fail(ctx, CLR_ERR_NOT_READY, "clr_build_particles must succeed before clr_trace");
    if (n < 1) return CLR_ERR_INVALID_ARGUMENT;
    std::vector<SceneRef> refs(n, SceneRef{&ctx->sp, &ctx->pb});
    return trace_runs(ctx, refs.data(), runs, n, outs, d_records, ctx->light_on ? ctx->d_light : nullptr,
                      ctx->prov_on);
}

// Zero the light-diagnostic buffers (trajectory coordinates to NaN and orders to -1, as the reference).
static int light_reset(clr_ctx* ctx) {
    {
        const LightDiag& L = ctx->light;
        const size_t vox = (size_t)L.nx * L.ny * L.nz, traj = (size_t)std::max(L.rep_rays * L.max_segments, 1);
        const size_t heat = (size_t)std::max(L.vis * L.vis, 1), reps = (size_t)std::max(L.rep_rays, 1);
        cudaStream_t st = ctx->stream;
        CU(cudaMemsetAsync(L.total, 0, vox * 4, st)); CU(cudaMemsetAsync(L.post, 0, vox * 4, st));
        CU(cudaMemsetAsync(L.event_weight, 0, vox * 4, st)); CU(cudaMemsetAsync(L.event_count, 0, vox * 4, st));
        CU(cudaMemsetAsync(L.seg_total, 0, 8, st)); CU(cudaMemsetAsync(L.dep_total, 0, 8, st));
        CU(cudaMemsetAsync(L.seg_count, 0, 8, st)); CU(cudaMemsetAsync(L.event_total, 0, 8, st));
        CU(cudaMemsetAsync(L.err_count, 0, 4, st)); CU(cudaMemsetAsync(L.adj_count, 0, 4, st));
        CU(cudaMemsetAsync(L.outside, 0, 32, st));
        for (float* p : {L.tx0, L.ty0, L.tz0, L.tx1, L.ty1, L.tz1}) CU(cudaMemsetAsync(p, 0xFF, traj * 4, st));
        CU(cudaMemsetAsync(L.torder, 0xFF, traj * 4, st));
        CU(cudaMemsetAsync(L.tcount, 0, reps * 4, st)); CU(cudaMemsetAsync(L.toverflow, 0, reps * 4, st));
        CU(cudaMemsetAsync(L.heat_xy, 0, heat * 4, st)); CU(cudaMemsetAsync(L.heat_zy, 0, heat * 4, st));
        CU(cudaStreamSynchronize(st));
    }
    return CLR_OK;
}

static int trace_impl(clr_ctx* ctx, const clr_run_params* run, clr_tallies* out, clr_ray_record* d_records) {
    return trace_current(ctx, run, 1, out, d_records);
}

// ---------------- scenario sweep: many scenes built and traced together ----------------
// Every scenario keeps its own ParticleBuffers, but each per-bin array is one slice of a sweep-wide
// array (scenario i's bins start at bin_off[i]), so the Mie coefficient, phase pdf and phase CDF
// kernels run over the bins of many scenarios per launch. The scene-dependent rest of the precompute
// (rates, sediment coefficients, majorants) stays per scenario.

// Bump allocator over one device arena; with base 0 it only measures.
struct Arena {
    uintptr_t base = 0;
    size_t off = 0;
    template <class T>
    T* take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base + off);
        off += std::max<size_t>(count * sizeof(T), 16);
        return p;
    }
};

static double* ParticleBuffers::* const kBinF64[] = {
    &ParticleBuffers::d, &ParticleBuffers::w, &ParticleBuffers::nidx, &ParticleBuffers::kidx, &ParticleBuffers::x,
    &ParticleBuffers::qext, &ParticleBuffers::qsca, &ParticleBuffers::qabs, &ParticleBuffers::qback,
    &ParticleBuffers::g, &ParticleBuffers::albedo, &ParticleBuffers::radius, &ParticleBuffers::nden,
    &ParticleBuffers::mug, &ParticleBuffers::mus, &ParticleBuffers::mue, &ParticleBuffers::muw,
    &ParticleBuffers::muev, &ParticleBuffers::gcdf, &ParticleBuffers::wcdf, &ParticleBuffers::pcdf,
    &ParticleBuffers::moment_a, &ParticleBuffers::moment_b, &ParticleBuffers::trace_geom,
    &ParticleBuffers::trace_wave, &ParticleBuffers::sedA, &ParticleBuffers::sedB, &ParticleBuffers::sed_norm,
    &ParticleBuffers::sed_max, &ParticleBuffers::grid_max, &ParticleBuffers::sed_ws};
static float* ParticleBuffers::* const kBinF32[] = {&ParticleBuffers::gcdf_f, &ParticleBuffers::wcdf_f,
                                                   &ParticleBuffers::pn_f, &ParticleBuffers::pk_f,
                                                   &ParticleBuffers::prad_f};

struct SweepLayout {
    std::vector<long long> bin_off, tab_off, rad_off, quad_off, cell_off;
    long long bins = 0, tabs = 0, rads = 0, quads = 0, cells = 0;
    std::vector<int> group_first;  // first scenario of each run of scenarios with one Mie key, + sentinel
};

// Two scenarios whose Mie inputs other than the particles agree (their bins can share one launch).
static bool same_mie_key(const ParticleBuffers& a, const clr_particle_spec& pa, const ParticleBuffers& b,
                         const clr_particle_spec& pb) {
    return a.nt == b.nt && pa.n_medium == pb.n_medium && pa.wavelength_m == pb.wavelength_m;
}

static void sweep_carve(Arena& A, const SweepLayout& L, std::vector<ParticleBuffers>& pbs) {
    const int ns = (int)pbs.size();
    for (auto mp : kBinF64) {
        double* b = A.take<double>(L.bins);
        for (int i = 0; i < ns; ++i) pbs[i].*mp = b + L.bin_off[i];
    }
    for (auto mp : kBinF32) {
        float* b = A.take<float>(L.bins);
        for (int i = 0; i < ns; ++i) pbs[i].*mp = b + L.bin_off[i];
    }
    int* nstop = A.take<int>(L.bins);
    uint8_t* mm = A.take<uint8_t>(L.bins);
    double* cdf = A.take<double>(L.tabs);
    float* cdf_f = A.take<float>(L.tabs);
    int* guide = A.take<int>((size_t)L.bins * (kPhaseGuide + 1));
    double* muscal = A.take<double>(8 * (size_t)ns);
    double* smaj = A.take<double>(4 * (size_t)ns);
    float* nmaj = A.take<float>(ns);
    double* srl = A.take<double>(L.rads);
    double* swr = A.take<double>(L.rads);
    double* sterm = A.take<double>(L.quads);
    double* grid = A.take<double>(L.cells);
    int* err = A.take<int>(1);
    for (int i = 0; i < ns; ++i) {
        ParticleBuffers& pb = pbs[i];
        pb.nstop = nstop + L.bin_off[i];
        pb.moment_mode = mm + L.bin_off[i];
        pb.phase_cdf = cdf + L.tab_off[i];
        pb.phase_cdf_f = cdf_f + L.tab_off[i];
        pb.phase_guide = guide + (size_t)L.bin_off[i] * (kPhaseGuide + 1);
        pb.muscal = muscal + 8 * (size_t)i;
        pb.sed_major = smaj + 4 * (size_t)i;
        pb.node_major = nmaj + i;
        pb.sed_radial_log = srl + L.rad_off[i];
        pb.sed_wr = swr + L.rad_off[i];
        pb.sed_terms = sterm + L.quad_off[i];
        pb.sed_grid = grid + L.cell_off[i];
        pb.err = err;
        pb.ab = nullptr;
        pb.pdf = nullptr;
        if (pb.node_tables) {
            const size_t plane = (size_t)pb.grid_nr * pb.grid_nz;
            pb.node_mu = A.take<float2>(plane);
            pb.node_alias = A.take<int2>(2 * plane * pb.n);
        }
        if (pb.solver_iterations < 0) {  // marks a scenario whose model-3 field is solved
            pb.merid_coef = A.take<double>(meridional_coef_doubles(pb.n, pb.grid_nr, pb.grid_nz));
            pb.merid_residual = A.take<double>(2 * (size_t)pb.n + 1);
            pb.merid_bar = A.take<unsigned>(2);
            pb.merid_stats = A.take<int>(1);
        }
    }
    for (size_t g = 0; g + 1 < L.group_first.size(); ++g) {
        const int nt = pbs[L.group_first[g]].nt;
        double* th = A.take<double>(nt);
        float* th_f = A.take<float>(nt);
        for (int i = L.group_first[g]; i < L.group_first[g + 1]; ++i) { pbs[i].theta = th; pbs[i].theta_f = th_f; }
    }
}

// Bins per Mie launch of a sweep: bounds the a_n/b_n and pdf scratch (at most ~0.5 GB of a_n/b_n rows).
constexpr int kSweepChunkBins = 4096;

static int sweep_build(clr_ctx* ctx, int ns, const clr_scene_params* sps, const clr_particle_spec* pss,
                       const clr_sediment_spec* sss_in) {
    ctx->sw_sp.clear();
    ctx->sw_pb.clear();
    if (ns < 1 || !sps || !pss || !sss_in) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "clr_sweep_build: no scenarios");
    std::vector<clr_sediment_spec> fss(ns);
    for (int i = 0; i < ns; ++i) fss[i] = filled_sediment(sps[i], sss_in[i]);
    const clr_sediment_spec* sss = fss.data();
    std::vector<ParticleBuffers> pbs(ns);
    SweepLayout L;
    L.bin_off.resize(ns + 1); L.tab_off.resize(ns + 1); L.rad_off.resize(ns + 1); L.quad_off.resize(ns + 1);
    L.cell_off.resize(ns + 1);
    for (int i = 0; i < ns; ++i) {
        const clr_scene_params& sp = sps[i];
        int rc = check_scene(ctx, sp);
        if (rc == CLR_OK) rc = check_particles(ctx, sp, pss + i, sss + i);
        if (rc == CLR_OK && pss[i].table_arithmetic != pss[0].table_arithmetic)
            rc = fail(ctx, CLR_ERR_INVALID_ARGUMENT, "every scenario of a sweep must share table_arithmetic");
        if (rc != CLR_OK) {
            ctx->err = "scenario " + std::to_string(i) + ": " + ctx->err;
            return rc;
        }
        ParticleBuffers& pb = pbs[i];
        const int n = pss[i].n_bins;
        pb.n = n;
        pb.nt = hybrid_model(sp) ? pss[i].n_theta : 2;
        pb.n_radial = sss[i].n_radial;
        pb.grid_nr = grid_nr_of(sp, sss[i]);
        pb.grid_nz = grid_nz_of(sp, sss[i]);
        pb.grid_zmax = sss[i].grid_zmax;
        if (solves_grid(sp, sss[i])) pb.solver_iterations = -1;
        const long long cells = sp.sediment_model == 3 ? (long long)pb.grid_nr * pb.grid_nz * n : 1;
        pb.node_tables = wants_node_tables(sp, sss[i], n, (size_t)cells) ? 1 : 0;
        L.bin_off[i] = L.bins; L.bins += n;
        L.tab_off[i] = L.tabs; L.tabs += (long long)n * pb.nt;
        L.rad_off[i] = L.rads; L.rads += (long long)n * pb.n_radial;
        L.quad_off[i] = L.quads; L.quads += (long long)n * sss[i].n_quad;
        L.cell_off[i] = L.cells; L.cells += cells;
        if (i == 0 || !same_mie_key(pbs[i - 1], pss[i - 1], pb, pss[i])) L.group_first.push_back(i);
    }
    L.group_first.push_back(ns);
    L.bin_off[ns] = L.bins; L.tab_off[ns] = L.tabs; L.rad_off[ns] = L.rads; L.quad_off[ns] = L.quads;
    L.cell_off[ns] = L.cells;
    CU(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    {
        Arena probe;
        std::vector<ParticleBuffers> tmp = pbs;
        sweep_carve(probe, L, tmp);
        if (probe.off > ctx->sw_arena_bytes) {
            CU(cudaStreamSynchronize(st));
            cudaFree(ctx->sw_arena);
            ctx->sw_arena = nullptr;
            ctx->sw_arena_bytes = 0;
            CU(cudaMalloc(&ctx->sw_arena, probe.off));
            ctx->sw_arena_bytes = probe.off;
        }
    }
    Arena A;
    A.base = reinterpret_cast<uintptr_t>(ctx->sw_arena);
    sweep_carve(A, L, pbs);
    // host staging of the inputs, in the sweep's bin order
    std::vector<double> hd(L.bins), hw(L.bins), hn(L.bins), hk(L.bins), ma(L.bins, 1.0), mb(L.bins, 0.0);
    std::vector<uint8_t> mm(L.bins, 0);
    std::vector<double> cells(L.cells, 1.0);
    for (int i = 0; i < ns; ++i) {
        const clr_particle_spec& ps = pss[i];
        const long long o = L.bin_off[i];
        std::copy(ps.diameter_m, ps.diameter_m + ps.n_bins, hd.begin() + o);
        std::copy(ps.weight, ps.weight + ps.n_bins, hw.begin() + o);
        std::copy(ps.n_real, ps.n_real + ps.n_bins, hn.begin() + o);
        std::copy(ps.k_imag, ps.k_imag + ps.n_bins, hk.begin() + o);
        if (ps.moment_enabled && ps.moment_a && ps.moment_b && ps.moment_mode) {
            for (int b = 0; b < ps.n_bins; ++b) {
                ma[o + b] = ps.moment_a[b]; mb[o + b] = ps.moment_b[b]; mm[o + b] = ps.moment_mode[b];
                pbs[i].any_moment |= ps.moment_mode[b] ? 1 : 0;
            }
        }
        if (sps[i].sediment_model == 3 && sss[i].grid)
            std::copy(sss[i].grid, sss[i].grid + (L.cell_off[i + 1] - L.cell_off[i]), cells.begin() + L.cell_off[i]);
    }
    const ParticleBuffers& P0 = pbs[0];  // per-bin arrays start at scenario 0's slices
    CU(cudaEventRecord(ctx->ev0, st));
    CU(cudaMemcpyAsync(P0.d, hd.data(), L.bins * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P0.w, hw.data(), L.bins * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P0.nidx, hn.data(), L.bins * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P0.kidx, hk.data(), L.bins * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P0.moment_a, ma.data(), L.bins * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P0.moment_b, mb.data(), L.bins * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P0.moment_mode, mm.data(), L.bins, cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(P0.sed_grid, cells.data(), L.cells * sizeof(double), cudaMemcpyHostToDevice, st));
    CU(cudaMemsetAsync(P0.err, 0, sizeof(int), st));
    // Mie tables: chunks of at most kSweepChunkBins bins within each run of scenarios sharing the key
    struct Chunk { int s0; long long b0, b1; int cap; };
    std::vector<Chunk> chunks;
    size_t scratch = 0;
    for (size_t g = 0; g + 1 < L.group_first.size(); ++g) {
        const int s0 = L.group_first[g], s1 = L.group_first[g + 1];
        const clr_particle_spec& ps = pss[s0];
        for (long long b0 = L.bin_off[s0]; b0 < L.bin_off[s1]; b0 += kSweepChunkBins) {
            const long long b1 = std::min(b0 + kSweepChunkBins, L.bin_off[s1]);
            const int cap = mie_order_bound(hd.data() + b0, hn.data() + b0, hk.data() + b0, (int)(b1 - b0),
                                            ps.n_medium, ps.wavelength_m);
            chunks.push_back({s0, b0, b1, cap});
            const size_t ab = (size_t)(b1 - b0) * cap * 4 * sizeof(double);
            const size_t pdf = hybrid_model(sps[s0]) ? (size_t)(b1 - b0) * pbs[s0].nt * sizeof(double) : 0;
            scratch = std::max(scratch, ((ab + 255) & ~(size_t)255) + pdf);
        }
    }
    if (scratch > ctx->sw_scratch_bytes) {
        CU(cudaStreamSynchronize(st));
        cudaFree(ctx->sw_scratch);
        ctx->sw_scratch = nullptr;
        ctx->sw_scratch_bytes = 0;
        CU(cudaMalloc(&ctx->sw_scratch, scratch));
        ctx->sw_scratch_bytes = scratch;
    }
    for (const Chunk& c : chunks) {
        const ParticleBuffers& G = pbs[c.s0];
        const long long nb = c.b1 - c.b0;
        const long long tab = L.tab_off[c.s0] + (c.b0 - L.bin_off[c.s0]) * G.nt;
        MiePhaseBuffers b;
        b.ab = static_cast<double*>(ctx->sw_scratch);
        b.pdf = reinterpret_cast<double*>(static_cast<char*>(ctx->sw_scratch) +
                                          (((size_t)nb * c.cap * 4 * sizeof(double) + 255) & ~(size_t)255));
        b.nstop = P0.nstop + c.b0; b.x = P0.x + c.b0; b.qext = P0.qext + c.b0; b.qsca = P0.qsca + c.b0;
        b.qabs = P0.qabs + c.b0; b.qback = P0.qback + c.b0; b.g = P0.g + c.b0; b.albedo = P0.albedo + c.b0;
        b.theta = G.theta; b.theta_f = G.theta_f;
        b.cdf = P0.phase_cdf + tab; b.cdf_f = P0.phase_cdf_f + tab; b.err = P0.err;
        b.guide = P0.phase_guide + (size_t)c.b0 * (kPhaseGuide + 1);
        CU(enqueue_mie_tables(P0.d + c.b0, P0.nidx + c.b0, P0.kidx + c.b0, (int)nb, pss[c.s0].n_medium,
                              pss[c.s0].wavelength_m, G.nt, hybrid_model(sps[c.s0]), c.cap, b, st,
                              pss[c.s0].table_arithmetic == CLR_TABLES_FAST));
    }
    {
        const size_t need = scene_rates_batch_scratch(ns);
        if (need > ctx->sw_jobs_bytes) {
            CU(cudaStreamSynchronize(st));
            cudaFree(ctx->sw_jobs);
            ctx->sw_jobs = nullptr;
            ctx->sw_jobs_bytes = 0;
            CU(cudaMalloc(&ctx->sw_jobs, need));
            ctx->sw_jobs_bytes = need;
        }
        std::vector<ParticleBuffers*> pp(ns);
        for (int i = 0; i < ns; ++i) pp[i] = &pbs[i];
        CU(enqueue_scene_rates_batch(pp.data(), sps, pss, sss, ns, ctx->sw_jobs, st));
    }
    int herr = 0;
    std::vector<double> hmu(8 * (size_t)ns), hsm(4 * (size_t)ns);
    std::vector<float> hnm(ns);
    CU(cudaMemcpyAsync(&herr, P0.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(hmu.data(), P0.muscal, hmu.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(hsm.data(), P0.sed_major, hsm.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(hnm.data(), P0.node_major, hnm.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
    for (int i = 0; i < ns; ++i)
        if (pbs[i].merid_coef) {
            CU(cudaMemcpyAsync(&pbs[i].solver_iterations, pbs[i].merid_stats, sizeof(int), cudaMemcpyDeviceToHost, st));
            CU(cudaMemcpyAsync(&pbs[i].solver_max_residual, pbs[i].merid_residual + 2 * (size_t)pbs[i].n,
                               sizeof(double), cudaMemcpyDeviceToHost, st));
        }
    CU(cudaEventRecord(ctx->ev1, st));
    CU(cudaStreamSynchronize(st));
    CU(cudaEventElapsedTime(&ctx->last_kernel_ms, ctx->ev0, ctx->ev1));
    if (herr) return fail(ctx, CLR_ERR_PRECOMPUTE, "sweep particle precompute failed with error code %d", herr);
    for (int i = 0; i < ns; ++i)
        if (pbs[i].merid_coef && pbs[i].solver_max_residual > sss[i].solver_tolerance)
            return fail(ctx, CLR_ERR_PRECOMPUTE,
                        "scenario %d: meridional transport solver did not converge: max residual=%.6g after %d iterations",
                        i, pbs[i].solver_max_residual, pbs[i].solver_iterations);
    for (int i = 0; i < ns; ++i) {
        std::copy(hmu.begin() + 8 * i, hmu.begin() + 8 * i + 8, pbs[i].muscal_host);
        std::copy(hsm.begin() + 4 * i, hsm.begin() + 4 * i + 4, pbs[i].sed_major_host);
        pbs[i].node_major_host = hnm[i];
    }
    ctx->sw_sp.assign(sps, sps + ns);
    ctx->sw_pb = std::move(pbs);
    ctx->last_passes = 0;
    ctx->last_launches = 0;
    return CLR_OK;
}

extern "C" {

int clr_trace(clr_ctx* ctx, const clr_run_params* run, clr_tallies* out, clr_ray_record* records) {
    return trace_impl(ctx, run, out, records);
}

int clr_trace_batch(clr_ctx* ctx, const clr_run_params* runs, int n_runs, clr_tallies* outs) {
    return trace_current(ctx, runs, n_runs, outs, nullptr);
}

int clr_set_light_diagnostics(clr_ctx* ctx, const clr_light_config* cfg) {
    if (!ctx || !cfg) return CLR_ERR_INVALID_ARGUMENT;
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(ctx->stream));
    for (void* p : ctx->light_allocs) cudaFree(p);
    ctx->light_allocs.clear();
    ctx->light_on = false;
    ctx->light = LightDiag{};
    if (cfg->heatmap_size < 0) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "heatmap_size must be >= 0");
    if (!cfg->enabled && cfg->heatmap_size == 0) return CLR_OK;
    // the reference's configuration rules (:7246-7252) and allocation cap (:7266-7275)
    const bool vx = cfg->enabled != 0;
    if (vx && cfg->max_rays < 1) return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "light diagnostic max_rays must be >=1");
    if (vx && std::min(cfg->nx, std::min(cfg->ny, cfg->nz)) < 4)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "light diagnostic grid dimensions must each be >=4");
    const int rep = vx ? std::min(cfg->representative_rays, cfg->max_rays) : 0;
    if (vx && (rep < 0 || cfg->max_segments_per_ray < 1))
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "invalid representative-ray diagnostic configuration");
    const size_t vox = vx ? (size_t)cfg->nx * cfg->ny * cfg->nz : 1;
    const size_t traj = (size_t)std::max(rep * (vx ? cfg->max_segments_per_ray : 1), 1), reps = (size_t)std::max(rep, 1);
    const size_t bytes = vox * 20 + traj * 32 + reps * 8 + 8;
    if (bytes > 1000000000ull)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "light diagnostic allocation is too large (%.3g GB)", bytes / 1e9);
    const size_t heat = (size_t)std::max(cfg->heatmap_size * cfg->heatmap_size, 1);
    LightDiag& L = ctx->light;
    L.voxels = vx ? 1 : 0;
    L.nx = vx ? cfg->nx : 1; L.ny = vx ? cfg->ny : 1; L.nz = vx ? cfg->nz : 1; L.max_rays = vx ? cfg->max_rays : 0;
    L.rep_rays = rep; L.max_segments = vx ? cfg->max_segments_per_ray : 0; L.vis = cfg->heatmap_size;
    L.zmax = cfg->zmax;
    L.zvis = cfg->heat_zmax;
    auto A = [&](void** p, size_t b) {
        cudaError_t e = cudaMalloc(p, b);
        if (e == cudaSuccess) ctx->light_allocs.push_back(*p);
        return e;
    };
    CU(A((void**)&L.total, vox * 4)); CU(A((void**)&L.post, vox * 4)); CU(A((void**)&L.event_weight, vox * 4));
    CU(A((void**)&L.event_count, vox * 4));
    CU(A((void**)&L.seg_total, 8)); CU(A((void**)&L.dep_total, 8)); CU(A((void**)&L.seg_count, 8));
    CU(A((void**)&L.event_total, 8)); CU(A((void**)&L.err_count, 4)); CU(A((void**)&L.adj_count, 4));
    CU(A((void**)&L.outside, 32));
    for (float** p : {&L.tx0, &L.ty0, &L.tz0, &L.tx1, &L.ty1, &L.tz1}) CU(A((void**)p, traj * 4));
    CU(A((void**)&L.torder, traj * 4)); CU(A((void**)&L.tcount, reps * 4)); CU(A((void**)&L.toverflow, reps * 4));
    CU(A((void**)&L.heat_xy, heat * 4)); CU(A((void**)&L.heat_zy, heat * 4));
    CU(A((void**)&ctx->d_light, sizeof(LightDiag)));
    CU(cudaMemcpy(ctx->d_light, &L, sizeof L, cudaMemcpyHostToDevice));
    ctx->light_cfg = *cfg;
    const int rc = light_reset(ctx);
    if (rc != CLR_OK) return rc;
    ctx->light_on = true;
    return CLR_OK;
}

int clr_set_path_provenance(clr_ctx* ctx, int enabled) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    CU(cudaSetDevice(ctx->device));
    CU(cudaStreamSynchronize(ctx->stream));
    ctx->prov_on = false;
    if (!enabled) return CLR_OK;
    int rc = wave_pool_ready(ctx);
    if (rc != CLR_OK) return rc;
    if (!ctx->d_prov) CU(cudaMalloc((void**)&ctx->d_prov, sizeof(clr_path_provenance)));
    if (!ctx->wave_prov) CU(cudaMalloc((void**)&ctx->wave_prov, (size_t)ctx->wave_cap * sizeof(uint4)));
    CU(cudaMemset(ctx->d_prov, 0, sizeof(clr_path_provenance)));
    ctx->prov_on = true;
    return CLR_OK;
}

int clr_read_path_provenance(clr_ctx* ctx, clr_path_provenance* out) {
    if (!ctx || !out) return CLR_ERR_INVALID_ARGUMENT;
    if (!ctx->prov_on) return fail(ctx, CLR_ERR_NOT_READY, "particle-event provenance is off");
    CU(cudaSetDevice(ctx->device));
    CU(cudaMemcpyAsync(out, ctx->d_prov, sizeof(clr_path_provenance), cudaMemcpyDeviceToHost, ctx->stream));
    CU(cudaStreamSynchronize(ctx->stream));
    return CLR_OK;
}

int clr_read_path_provenance_records(clr_ctx* ctx, uint32_t* out, int64_t n_rays) {
    if (!ctx || !out || n_rays < 0) return CLR_ERR_INVALID_ARGUMENT;
    if (!ctx->prov_on || n_rays > ctx->prov_rec_n)
        return fail(ctx, CLR_ERR_NOT_READY, "no per-ray provenance for %lld rays (the last trace kept %lld)",
                    (long long)n_rays, ctx->prov_rec_n);
    CU(cudaSetDevice(ctx->device));
    if (n_rays) CU(cudaMemcpy(out, ctx->d_prov_rec, (size_t)n_rays * sizeof(uint4), cudaMemcpyDeviceToHost));
    return CLR_OK;
}

int clr_read_light_diagnostics(clr_ctx* ctx, clr_light_result* o) {
    if (!ctx || !o) return CLR_ERR_INVALID_ARGUMENT;
    if (!ctx->light_on) return fail(ctx, CLR_ERR_NOT_READY, "light diagnostics are off");
    CU(cudaSetDevice(ctx->device));
    const LightDiag& L = ctx->light;
    cudaStream_t st = ctx->stream;
    const size_t vox = (size_t)L.nx * L.ny * L.nz, traj = (size_t)L.rep_rays * L.max_segments;
    const size_t heat = (size_t)L.vis * L.vis, reps = (size_t)L.rep_rays;
    struct Cp { void* dst; const void* src; size_t bytes; };
    const Cp cps[] = {{o->track_length, L.total, vox * 4}, {o->post_scatter_track_length, L.post, vox * 4},
                      {o->scatter_event_weight, L.event_weight, vox * 4}, {o->scatter_event_count, L.event_count, vox * 4},
                      {o->heatmap_xy, L.heat_xy, heat * 4}, {o->heatmap_zy, L.heat_zy, heat * 4},
                      {o->trajectory_x0, L.tx0, traj * 4}, {o->trajectory_y0, L.ty0, traj * 4},
                      {o->trajectory_z0, L.tz0, traj * 4}, {o->trajectory_x1, L.tx1, traj * 4},
                      {o->trajectory_y1, L.ty1, traj * 4}, {o->trajectory_z1, L.tz1, traj * 4},
                      {o->trajectory_order, L.torder, traj * 4}, {o->trajectory_count, L.tcount, reps * 4},
                      {o->trajectory_overflow, L.toverflow, reps * 4}};
    for (const Cp& c : cps)
        if (c.dst && c.bytes) CU(cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, st));
    unsigned long long sc = 0, et = 0;
    unsigned err = 0, adj = 0, outside[8] = {0};
    CU(cudaMemcpyAsync(&o->segment_length_total, L.seg_total, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&o->deposited_length_total, L.dep_total, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&sc, L.seg_count, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&et, L.event_total, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&err, L.err_count, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&adj, L.adj_count, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(outside, L.outside, 32, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    o->segment_count = (int64_t)sc; o->scatter_event_total = (int64_t)et;
    o->error_count = err; o->boundary_adjustment_count = adj; o->event_outside_count = outside[0];
    for (int k = 0; k < 3; ++k) memcpy(&o->first_outside_xyz_tol[k], &outside[1 + k], 4);
    memcpy(&o->first_outside_xyz_tol[3], &outside[5], 4);
    o->first_outside_ray = outside[4]; o->first_outside_set = outside[6];
    return CLR_OK;
}

int clr_sweep_build(clr_ctx* ctx, int n_scenarios, const clr_scene_params* scenes, const clr_particle_spec* particles,
                    const clr_sediment_spec* sediments) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    return sweep_build(ctx, n_scenarios, scenes, particles, sediments);
}

int clr_sweep_trace(clr_ctx* ctx, const clr_run_params* runs, int n_runs, clr_tallies* outs) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    if (ctx->sw_pb.empty()) return fail(ctx, CLR_ERR_NOT_READY, "clr_sweep_build must succeed before clr_sweep_trace");
    if (n_runs != (int)ctx->sw_pb.size())
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "clr_sweep_trace: %d runs for %d scenarios", n_runs,
                    (int)ctx->sw_pb.size());
    std::vector<SceneRef> refs(n_runs);
    for (int i = 0; i < n_runs; ++i) refs[i] = SceneRef{&ctx->sw_sp[i], &ctx->sw_pb[i]};
    return trace_runs(ctx, refs.data(), runs, n_runs, outs, nullptr);
}

int clr_sweep_read_particle_physics(clr_ctx* ctx, int scenario, clr_particle_physics* out) {
    if (!ctx || !out) return CLR_ERR_INVALID_ARGUMENT;
    if (scenario < 0 || scenario >= (int)ctx->sw_pb.size())
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "scenario %d outside the built sweep", scenario);
    return read_physics(ctx, ctx->sw_pb[scenario], out);
}

int clr_trace_host_records(clr_ctx* ctx, const clr_run_params* run, clr_tallies* out, clr_ray_record* host_records) {
    if (!ctx || !run || !out) return CLR_ERR_INVALID_ARGUMENT;
    if (!host_records) return trace_impl(ctx, run, out, nullptr);
    CU(cudaSetDevice(ctx->device));
    clr_ray_record* d = nullptr;
    const size_t bytes = (size_t)run->n_rays * sizeof(clr_ray_record);
    CU(cudaMalloc(&d, bytes ? bytes : 16));
    int rc = trace_impl(ctx, run, out, d);
    if (rc == CLR_OK) {
        cudaError_t e = cudaMemcpy(host_records, d, bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = fail(ctx, CLR_ERR_CUDA, "record copy: %s", cudaGetErrorString(e));
    }
    cudaFree(d);
    return rc;
}

int clr_mie_phase_noalloc(clr_ctx* ctx, const double* d_diameter_m, const double* d_n_real, const double* d_k_imag,
                          int n_bins, double n_medium, double wavelength_m, int n_theta, double* d_qext,
                          double* d_qsca, double* d_asym_g, double* d_theta, double* d_phase_cdf, void* stream) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    if (n_bins < 1 || n_bins > CLR_NOALLOC_MAX_BINS || n_theta < 2 || n_theta > CLR_NOALLOC_MAX_THETA)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT,
                    "clr_mie_phase_noalloc: n_bins must be 1..%d and n_theta 2..%d (its fixed scratch), got %d and %d",
                    CLR_NOALLOC_MAX_BINS, CLR_NOALLOC_MAX_THETA, n_bins, n_theta);
    if (!d_diameter_m || !d_n_real || !d_k_imag || !d_qext || !d_qsca || !d_asym_g || !d_theta || !d_phase_cdf)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "clr_mie_phase_noalloc: null buffer");
    if (!(wavelength_m > 0.0) || !(n_medium > 0.0))
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "clr_mie_phase_noalloc: wavelength and medium index must be positive");
    CU(cudaSetDevice(ctx->device));
    NoallocScratch sc;
    CU(noalloc_scratch(ctx->device, &sc));
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    MiePhaseBuffers b;
    b.ab = sc.ab; b.nstop = sc.nstop; b.x = sc.x; b.qext = d_qext; b.qsca = d_qsca; b.qabs = sc.qabs;
    b.qback = sc.qback; b.g = d_asym_g; b.albedo = sc.albedo; b.theta = d_theta; b.theta_f = sc.theta_f;
    b.pdf = sc.pdf; b.cdf = d_phase_cdf; b.cdf_f = sc.cdf_f; b.err = sc.err;
    CU(enqueue_mie_phase(d_diameter_m, d_n_real, d_k_imag, n_bins, n_medium, wavelength_m, n_theta, b, st));
    int herr = 0;
    CU(cudaMemcpyAsync(&herr, sc.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (herr) return fail(ctx, CLR_ERR_PRECOMPUTE, "clr_mie_phase_noalloc failed with error code %d", herr);
    return CLR_OK;
}

int clr_last_launches(const clr_ctx* ctx, int64_t* launches, int64_t* passes) {
    if (!ctx || !launches || !passes) return CLR_ERR_INVALID_ARGUMENT;
    *passes = ctx->last_passes;
    *launches = ctx->last_launches;
    return CLR_OK;
}

int clr_set_engine_config(clr_ctx* ctx, const clr_engine_config* config) {
    if (!ctx) return CLR_ERR_INVALID_ARGUMENT;
    if (!config) {
        ctx->engine = clr_engine_config{};
        return CLR_OK;
    }
    const clr_engine_config& c = *config;
    if (c.flight_steps < 0 || c.flight_steps > 64 || c.tail_photons < 0 || c.tail_photons > (1 << 23) ||
        c.rare_batch < 0 || c.rare_batch > (1 << 21) || c.pass_batch < 0 || c.pass_batch > 64)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT,
                    "engine config: flight_steps 0..64, tail_photons 0..8388608, rare_batch 0..2097152, "
                    "pass_batch 0..64");
    for (int q = 0; q < CLR_N_STAGES; ++q)
        if (c.stage_blocks[q] < 0 || c.stage_blocks[q] > 32)
            return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "engine config: stage_blocks must be 0..32");
    if (c.acr_budget < 0 || c.acr_budget > 16384 || c.acr_budget % CLR_ENGINE_ACR_BUDGET_STEP)
        return fail(ctx, CLR_ERR_INVALID_ARGUMENT, "engine config: acr_budget must be a multiple of %d up to 16384",
                    CLR_ENGINE_ACR_BUDGET_STEP);
    ctx->engine = c;
    return CLR_OK;
}

int clr_last_engine_stats(const clr_ctx* ctx, double* out, int n) {
    if (!ctx || !out || n < 1) return CLR_ERR_INVALID_ARGUMENT;
    const double v[5] = {(double)ctx->last_passes, (double)ctx->last_launches, (double)ctx->last_tail_photons,
                         (double)ctx->last_tail_ms, (double)ctx->last_kernel_ms};
    for (int i = 0; i < n && i < 5; ++i) out[i] = v[i];
    return CLR_OK;
}

int clr_last_kernel_ms(const clr_ctx* ctx, float* ms) {
    if (!ctx || !ms) return CLR_ERR_INVALID_ARGUMENT;
    *ms = ctx->last_kernel_ms;
    return CLR_OK;
}

int clr_calibrate(clr_ctx* ctx, int which, double* ops_per_second) {
    if (!ctx || !ops_per_second || which < 0 || which > 1) return CLR_ERR_INVALID_ARGUMENT;
    CU(cudaSetDevice(ctx->device));
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        double ops = 0.0;
        CU(cudaEventRecord(ctx->ev0, ctx->stream));
        CU(launch_calibration(which, ctx->num_sms, ctx->stream, &ops));
        CU(cudaEventRecord(ctx->ev1, ctx->stream));
        CU(cudaStreamSynchronize(ctx->stream));
        float ms = 0.0f;
        CU(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        if (rep > 0 && ms > 0.0f) best = std::max(best, ops / (ms * 1e-3));
    }
    *ops_per_second = best;
    return CLR_OK;
}

/* sizes of the ABI structs as compiled, for the Python mirror's self-check */
int64_t clr_abi_sizeof(int which) {
    switch (which) {
        case 0: return (int64_t)sizeof(clr_scene_params);
        case 1: return (int64_t)sizeof(clr_particle_spec);
        case 2: return (int64_t)sizeof(clr_sediment_spec);
        case 3: return (int64_t)sizeof(clr_run_params);
        case 4: return (int64_t)sizeof(clr_ray_record);
        case 5: return (int64_t)sizeof(clr_tallies);
        case 6: return (int64_t)sizeof(clr_particle_physics);
        case 7: return (int64_t)sizeof(clr_path_provenance);
        case 8: return (int64_t)sizeof(clr_engine_config);
        default: return -1;
    }
}

}  // extern "C"
