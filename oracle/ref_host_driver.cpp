/* Host driver for the reference's own device code (test infrastructure only).
 *
 * Builds into oracle/_ref/libclaritas_ref_host.so (recipe: oracle/Makefile).
 * It #includes the reference's CUDA_SRC, extracted unmodified by
 * oracle/ref_extract.py, through oracle/ref_host_shim.h, and reproduces the
 * host orchestration of the reference around it:
 *   - the precompute sequence of ClaritasForwardModel._prepare_gpu_particle_physics
 *     (CLARITAS/CLARITAS.py:6036-6965): PSD normalisation (:6147-6169), Mie
 *     coefficients (:6186-6220), theta grid / phase pdf / phase cdf or the dummy
 *     table (:6221-6255), transport rates (:6278-6325), channel rate arrays
 *     (:6362-6375), sediment coefficients (:6399-6449), and for model 3 either the
 *     meridional solver's launch sequence (:6451-6725) or the grid
 *     finalisation/majorants (:6694-6725) on a caller-supplied grid;
 *   - one simulate() chunk (CLARITAS/CLARITAS.py:7631-7864): trace_kernel with
 *     the exact 234-argument list (:7638-7758), then score_detectors_kernel
 *     (:7783-7847), with every GPU thread replaced by one loop iteration.
 * Rays run in parallel under OpenMP; each iteration sets the thread-local
 * blockIdx/threadIdx the kernel reads, so ray ids and RNG seeding are exactly
 * the reference's. Tallies are accumulated as in simulate (:7849-7862).
 */
#include "ref_host_shim.h"

#include <cstdio>
#include <cstdlib>
#include <vector>
#include <string>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "claritas_gb.h"
#include "tally_extras.h"

thread_local ref_dim3 threadIdx = {0, 0, 0};
thread_local ref_dim3 blockIdx = {0, 0, 0};
thread_local ref_dim3 blockDim = {1, 1, 1};

#include "_ref/claritas_cuda_src.inc"

namespace {

struct RefState {
    clr_scene_params sp;
    int n = 0, nt = 0;
    std::vector<double> d, w_in, wd, nidx, kidx;
    std::vector<double> agg_scalars;
    std::vector<int> nstop;
    std::vector<double> x, qext, qsca, qabs, qback, g, albedo;
    std::vector<double> theta, phase_cdf;
    std::vector<double> radius, pmass, srcw, nden, sg, ssca, sext, swave, sevent;
    std::vector<double> mug, mus, mue, muw, muev, pew, gew, wew, gcdf, wcdf, pcdf, muscal;
    std::vector<double> moment_a, moment_b;
    std::vector<unsigned char> moment_mode;
    std::vector<double> trace_geom, trace_wave;
    std::vector<double> sed_tau, sed_ws, sed_sre, sed_sdrag, sed_A, sed_B, sed_norm, sed_max, sed_min;
    std::vector<double> sed_rmax, sed_rre, sed_rcenter, sed_radial_log, sed_radial_wr;
    std::vector<double> sed_sc, sed_sw, sed_bc, sed_bw, sed_major;
    std::vector<double> sed_grid;
    int grid_nr = 2, grid_nz = 2, n_radial = 65;
    int solver_iterations = 0;
    double solver_residual = 0.0;
    float grid_zmax = 0.f;
    std::string err;
};

inline void set_index(unsigned bdim, unsigned i) {
    blockDim.x = bdim; blockIdx.x = i / bdim; threadIdx.x = i % bdim;
    blockDim.y = blockDim.z = 1; blockIdx.y = blockIdx.z = 0; threadIdx.y = threadIdx.z = 0;
}

}  // namespace

extern "C" {

struct clref_state;

const char* clref_last_error(clref_state* h) {
    return h ? reinterpret_cast<RefState*>(h)->err.c_str() : "null state";
}

void clref_free(clref_state* h) { delete reinterpret_cast<RefState*>(h); }

/* Precompute; returns 0 or the reference error code (positive) / -1 on bad input. */
int clref_prepare(const clr_scene_params* sp, const clr_particle_spec* ps, const clr_sediment_spec* ss,
                  clref_state** out) {
    if (!sp || !ps || !ss || !out) return -1;
    RefState* S = new RefState();
    *out = reinterpret_cast<clref_state*>(S);
    S->sp = *sp;
    const int n = ps->n_bins;
    S->n = n;
    if (n < 1 || n > CLR_MAX_BINS) { S->err = "bad n_bins"; return -1; }
    S->d.assign(ps->diameter_m, ps->diameter_m + n);
    S->w_in.assign(ps->weight, ps->weight + n);
    S->nidx.assign(ps->n_real, ps->n_real + n);
    S->kidx.assign(ps->k_imag, ps->k_imag + n);
    S->wd.assign(n, 0.0);
    S->agg_scalars.assign(10, 0.0);
    int err = 0;
    set_index(1, 0);
    orthokinetic_compact_aggregation_kernel(S->d.data(), S->w_in.data(), n, ps->concentration_kg_m3,
                                            ps->density_kg_m3, 0.0, 0.2, 200000, S->wd.data(),
                                            S->agg_scalars.data(), &err);
    if (err) { S->err = "PSD normalisation error"; return err; }
    const int M = 4096;
    std::vector<double> Dre((size_t)n * M), Dim((size_t)n * M), ar((size_t)n * M), ai((size_t)n * M),
        br((size_t)n * M), bi((size_t)n * M);
    S->nstop.assign(n, 0);
    S->x.assign(n, 0); S->qext.assign(n, 0); S->qsca.assign(n, 0); S->qabs.assign(n, 0);
    S->qback.assign(n, 0); S->g.assign(n, 0); S->albedo.assign(n, 0);
    for (int p = 0; p < n; ++p) {
        set_index(128, p);
        mie_coefficients_efficiencies_kernel(S->d.data(), S->nidx.data(), S->kidx.data(), ps->n_medium,
                                             ps->wavelength_m, n, Dre.data(), Dim.data(), ar.data(), ai.data(),
                                             br.data(), bi.data(), S->nstop.data(), S->x.data(), S->qext.data(),
                                             S->qsca.data(), S->qabs.data(), S->qback.data(), S->g.data(),
                                             S->albedo.data(), &err);
    }
    if (err) { S->err = "Mie precompute error"; return err; }
    const int em = sp->event_model;
    if (em == 3 || em == 4 || em == 5) {
        const int nt = ps->n_theta;
        S->nt = nt;
        S->theta.assign(nt, 0.0);
        std::vector<double> pdf((size_t)n * nt);
        S->phase_cdf.assign((size_t)n * nt, 0.0);
        for (int j = 0; j < nt; ++j) { set_index(128, j); build_theta_grid_kernel(S->theta.data(), nt); }
#pragma omp parallel for schedule(static)
        for (long long idx = 0; idx < (long long)n * nt; ++idx) {
            set_index(128, (unsigned)idx);
            mie_phase_pdf_kernel(S->theta.data(), nt, n, S->nstop.data(), ar.data(), ai.data(), br.data(),
                                 bi.data(), pdf.data());
        }
        for (int p = 0; p < n; ++p) {
            set_index(1, p);
            mie_phase_cdf_kernel(S->theta.data(), pdf.data(), nt, n, S->phase_cdf.data(), &err);
        }
    } else {
        S->nt = 2;
        S->theta.assign(2, 0.0);
        S->phase_cdf.assign((size_t)2 * n, 0.0);
        for (int p = 0; p < std::max(n, 1); ++p) {
            set_index(128, p);
            dummy_phase_kernel(S->theta.data(), S->phase_cdf.data(), n);
        }
    }
    if (err) { S->err = "phase CDF error"; return err; }
    auto arr = [n]() { return std::vector<double>(n, 0.0); };
    S->radius = arr(); S->pmass = arr(); S->srcw = arr(); S->nden = arr(); S->sg = arr(); S->ssca = arr();
    S->sext = arr(); S->swave = arr(); S->sevent = arr(); S->mug = arr(); S->mus = arr(); S->mue = arr();
    S->muw = arr(); S->muev = arr(); S->pew = arr(); S->gew = arr(); S->wew = arr(); S->gcdf = arr();
    S->wcdf = arr(); S->pcdf = arr(); S->muscal.assign(8, 0.0);
    set_index(1, 0);
    transport_precompute_kernel(S->d.data(), S->wd.data(), S->qext.data(), S->qsca.data(), S->kidx.data(), n,
                                ps->concentration_kg_m3, ps->density_kg_m3, ps->weight_mode, em,
                                ps->hybrid_wave_scale, ps->n_medium, ps->wavelength_m, ps->wave_rms_height_m,
                                S->radius.data(), S->pmass.data(), S->srcw.data(), S->nden.data(), S->sg.data(),
                                S->ssca.data(), S->sext.data(), S->swave.data(), S->sevent.data(), S->mug.data(),
                                S->mus.data(), S->mue.data(), S->muw.data(), S->muev.data(), S->pew.data(),
                                S->gew.data(), S->wew.data(), S->gcdf.data(), S->wcdf.data(), S->pcdf.data(),
                                S->muscal.data(), &err);
    if (err) { S->err = "transport precompute error"; return err; }
    S->moment_a.assign(n, 1.0); S->moment_b.assign(n, 0.0); S->moment_mode.assign(n, 0);
    if (ps->moment_enabled && ps->moment_a && ps->moment_b && ps->moment_mode) {
        for (int i = 0; i < n; ++i) {
            S->moment_a[i] = ps->moment_a[i]; S->moment_b[i] = ps->moment_b[i]; S->moment_mode[i] = ps->moment_mode[i];
        }
    }
    S->trace_geom = arr(); S->trace_wave = arr();
    for (int i = 0; i < n; ++i) {
        if (em == 3) { S->trace_geom[i] = S->mug[i]; S->trace_wave[i] = S->muw[i]; }
        else if (em == 4 || em == 5) { S->trace_geom[i] = std::max(S->muev[i] - S->muw[i], 0.0); S->trace_wave[i] = S->muw[i]; }
        else { S->trace_geom[i] = S->muev[i]; S->trace_wave[i] = 0.0; }
    }
    const int NR = ss->n_radial;
    S->n_radial = NR;
    S->sed_tau = arr(); S->sed_ws = arr(); S->sed_sre = arr(); S->sed_sdrag = arr(); S->sed_A = arr();
    S->sed_B = arr(); S->sed_norm = arr(); S->sed_max = arr(); S->sed_min.assign(n, NAN); S->sed_rmax = arr();
    S->sed_rre = arr(); S->sed_rcenter = arr(); S->sed_radial_log.assign((size_t)n * NR, 0.0);
    S->sed_radial_wr.assign((size_t)n * NR, 0.0); S->sed_sc = arr(); S->sed_sw = arr(); S->sed_bc = arr();
    S->sed_bw = arr(); S->sed_major.assign(4, 0.0);
    set_index(1, 0);
    // FP64 geometry as the reference's host passes it (:6413-6418), else the scene's FP32 values widened
    const bool g64 = ss->rin > 0.0;
    const double GR = g64 ? ss->rin : (double)sp->rin, GZMIN = g64 ? ss->zmin : (double)sp->zmin;
    const double GZMEAN = g64 ? ss->zmean : (double)sp->zmean;
    const double GDH = g64 ? ss->vortex_delta_h : (double)sp->vortex_delta_h;
    const double GCORE = g64 ? ss->vortex_core_radius : (double)sp->vortex_core_radius;
    sediment_transport_precompute_kernel(
        S->d.data(), n, sp->sediment_model, ss->particle_density, ss->water_density, ss->water_viscosity,
        ss->gravity, ss->eddy_diffusivity, GR, GZMIN, GZMEAN,
        sp->free_surface_model, GDH, GCORE, ss->n_quad, NR,
        S->trace_geom.data(), S->trace_wave.data(), S->sed_tau.data(), S->sed_ws.data(), S->sed_sre.data(),
        S->sed_sdrag.data(), S->sed_A.data(), S->sed_B.data(), S->sed_norm.data(), S->sed_max.data(),
        S->sed_rmax.data(), S->sed_rre.data(), S->sed_rcenter.data(), S->sed_radial_log.data(),
        S->sed_radial_wr.data(), S->sed_sc.data(), S->sed_sw.data(), S->sed_bc.data(), S->sed_bw.data(),
        S->sed_major.data(), &err);
    if (err) { S->err = "sediment precompute error"; return err; }
    S->sed_grid.assign(1, 1.0);
    S->grid_nr = 2; S->grid_nz = 2; S->grid_zmax = (float)ss->grid_zmax;
    if (sp->sediment_model == 3 && !ss->grid) {
        // the reference's meridional solver kernels in its host's launch sequence (:6451-6725); a launch of
        // T threads becomes a loop over t, a <<<n, 1>>> launch a loop over the bins
        const int GNR = ss->meridional_nr, GNZ = ss->meridional_nz, FSM = sp->free_surface_model;
        const int max_it = ss->solver_max_iterations, every = ss->solver_check_interval;
        if (GNR < 2 || GNZ < 2 || max_it < 1 || every < 1) { S->err = "bad meridional solver settings"; return -1; }
        const long long plane = (long long)GNR * GNZ, total = plane * n;
        const double ZG = ss->grid_zmax;
        S->grid_nr = GNR; S->grid_nz = GNZ;
        S->sed_grid.assign((size_t)total, 0.0);
        std::vector<unsigned char> active((size_t)plane, 0);
        std::vector<double> ap((size_t)total), ae((size_t)total), aw((size_t)total), an((size_t)total),
            as((size_t)total), res(n, 0.0);
        double* G = S->sed_grid.data();
        auto each = [](long long T, auto&& f) {
#pragma omp parallel for schedule(static)
            for (long long t = 0; t < T; ++t) { set_index(256, (unsigned)t); f(); }
            set_index(1, 0);
        };
        auto per_bin = [&](auto&& f) {
            for (int p = 0; p < n; ++p) { set_index(1, p); f(); }
            set_index(1, 0);
        };
        each(plane, [&] { meridional_active_mask_kernel(GNR, GNZ, GR, GZMIN, ZG, GZMEAN, FSM, GDH, GCORE,
                                                        active.data()); });
        each(total, [&] { meridional_grid_initialize_kernel(n, GNR, GNZ, GR, GZMIN, ZG, FSM, GCORE, S->sed_A.data(),
                                                            S->sed_B.data(), S->sed_norm.data(),
                                                            S->sed_radial_log.data(), NR, active.data(), G); });
        each(total, [&] { meridional_build_coefficients_kernel(n, GNR, GNZ, GR, GZMIN, ZG, GZMEAN, FSM, GDH, GCORE,
                                                               ss->meridional_peak_speed, ss->eddy_diffusivity,
                                                               S->sed_ws.data(), S->sed_radial_wr.data(), NR,
                                                               active.data(), ap.data(), ae.data(), aw.data(),
                                                               an.data(), as.data()); });
        auto normalize = [&] {
            per_bin([&] { meridional_normalize_kernel(n, GNR, GNZ, GR, GZMIN, ZG, GZMEAN, active.data(), G, &err); });
        };
        auto relax = [&](int parity) {
            each(total, [&] { meridional_relax_kernel(n, GNR, GNZ, parity, ss->solver_sor, active.data(), ap.data(),
                                                      ae.data(), aw.data(), an.data(), as.data(), G); });
        };
        normalize();
        if (err) { S->err = "meridional initial normalization error"; return err; }
        const int min_it = max_it < 1000 ? max_it : 1000;
        int iters = 0, last = 0;
        for (int it = 1; it <= max_it; ++it) {
            relax(0);
            relax(1);
            if (it % 20 == 0) normalize();
            if (it % every == 0 || it == max_it) {
                normalize();
                per_bin([&] { meridional_residual_kernel(n, GNR, GNZ, active.data(), ap.data(), ae.data(), aw.data(),
                                                         an.data(), as.data(), G, res.data()); });
                if (err) { S->err = "meridional normalization error"; return err; }
                last = it;
                double mx = 0.0;
                for (double v : res) mx = v > mx ? v : mx;
                if (it >= min_it && mx <= ss->solver_tolerance) { iters = it; break; }
            }
        }
        if (iters == 0) iters = last ? last : max_it;
        double mx = 0.0;
        for (double v : res) mx = v > mx ? v : mx;
        S->solver_iterations = iters;
        S->solver_residual = mx;
        if (mx > ss->solver_tolerance) { S->err = "meridional transport solver did not converge"; return -7; }
        each((long long)n * GNR, [&] { meridional_extend_grid_kernel(n, GNR, GNZ, active.data(), G); });
        per_bin([&] { meridional_finalize_kernel(n, GNR, GNZ, GR, GZMIN, ZG, active.data(), G, S->sed_norm.data(),
                                                 S->sed_max.data(), S->sed_min.data(), S->sed_sc.data(),
                                                 S->sed_sw.data(), S->sed_bc.data(), S->sed_bw.data()); });
        meridional_majorants_kernel(n, S->trace_geom.data(), S->trace_wave.data(), S->sed_max.data(),
                                    S->sed_major.data());
    } else if (sp->sediment_model == 3) {
        if (!ss->grid || ss->grid_nr < 2 || ss->grid_nz < 2) { S->err = "model 3 needs a grid"; return -1; }
        S->grid_nr = ss->grid_nr; S->grid_nz = ss->grid_nz;
        const size_t plane = (size_t)ss->grid_nr * ss->grid_nz;
        S->sed_grid.assign(ss->grid, ss->grid + plane * n);
        std::vector<unsigned char> active(plane, 1);
        for (int p = 0; p < n; ++p) {
            set_index(1, p);
            meridional_finalize_kernel(n, ss->grid_nr, ss->grid_nz, GR, GZMIN,
                                       ss->grid_zmax, active.data(), S->sed_grid.data(), S->sed_norm.data(),
                                       S->sed_max.data(), S->sed_min.data(), S->sed_sc.data(), S->sed_sw.data(),
                                       S->sed_bc.data(), S->sed_bw.data());
        }
        set_index(1, 0);
        meridional_majorants_kernel(n, S->trace_geom.data(), S->trace_wave.data(), S->sed_max.data(),
                                    S->sed_major.data());
    }
    return 0;
}

int clref_read_physics(clref_state* h, clr_particle_physics* o) {
    RefState* S = reinterpret_cast<RefState*>(h);
    if (!S || !o) return -1;
    auto cp = [](double* dst, const std::vector<double>& v) { if (dst) std::copy(v.begin(), v.end(), dst); };
    cp(o->size_parameter, S->x); cp(o->qext, S->qext); cp(o->qsca, S->qsca); cp(o->qabs, S->qabs);
    cp(o->qback, S->qback); cp(o->asym_g, S->g); cp(o->albedo, S->albedo);
    if (o->nstop) std::copy(S->nstop.begin(), S->nstop.end(), o->nstop);
    cp(o->radius, S->radius); cp(o->number_density, S->nden);
    cp(o->mu_geom_bin, S->mug); cp(o->mu_sca_bin, S->mus); cp(o->mu_ext_bin, S->mue); cp(o->mu_wave_bin, S->muw);
    cp(o->mu_event_bin, S->muev); cp(o->trace_geom_bin, S->trace_geom); cp(o->trace_wave_bin, S->trace_wave);
    cp(o->geometric_cdf, S->gcdf); cp(o->wave_cdf, S->wcdf); cp(o->particle_event_cdf, S->pcdf);
    cp(o->mu_scalars, S->muscal); cp(o->sed_majorants, S->sed_major); cp(o->theta, S->theta);
    cp(o->phase_cdf, S->phase_cdf);
    return 0;
}

int clref_n_theta(clref_state* h) { return h ? reinterpret_cast<RefState*>(h)->nt : 0; }

int clref_read_sediment_field(clref_state* h, double* grid, int* nr, int* nz, int* iterations, double* max_residual) {
    RefState* S = reinterpret_cast<RefState*>(h);
    if (!S) return -1;
    if (nr) *nr = S->grid_nr;
    if (nz) *nz = S->grid_nz;
    if (iterations) *iterations = S->solver_iterations;
    if (max_residual) *max_residual = S->solver_residual;
    if (grid) std::copy(S->sed_grid.begin(), S->sed_grid.end(), grid);
    return 0;
}

/* Trace + score run->n_rays rays starting at global id run->ray_offset.
 * records (host memory, nullable) receives one clr_ray_record per ray. */
static int trace_impl(clref_state* h, const clr_run_params* run, clr_tallies* T, clr_ray_record* records,
                      int32_t* prov, float* defl, int n_threads);

int clref_trace(clref_state* h, const clr_run_params* run, clr_tallies* T, clr_ray_record* records,
                int n_threads) {
    return trace_impl(h, run, T, records, nullptr, nullptr, n_threads);
}

/* As clref_trace, and per ray the reference's provenance outputs: prov [n_rays][13] = its int outputs
 * first_particle_event_type .. particle_after_acrylic_return_count (trace_kernel :4601-4603), defl
 * [n_rays][5] = first_particle_deflection_deg .. water_path_after_last_particle_event (:4580). */
int clref_trace_provenance(clref_state* h, const clr_run_params* run, clr_tallies* T, clr_ray_record* records,
                           int32_t* prov, float* defl, int n_threads) {
    return trace_impl(h, run, T, records, prov, defl, n_threads);
}

static int trace_impl(clref_state* h, const clr_run_params* run, clr_tallies* T, clr_ray_record* records,
                      int32_t* prov, float* defl, int n_threads) {
    RefState* S = reinterpret_cast<RefState*>(h);
    if (!S || !run || !T) return -1;
    if (run->rng_mode != CLR_RNG_REFERENCE_XORSHIFT || run->weight_mode != CLR_WEIGHT_ANALOG) {
        S->err = "the reference supports only xorshift streams and analog weights";
        return -4;
    }
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    std::memset(T, 0, sizeof *T);
    const clr_scene_params& P = S->sp;
    const int64_t total = run->n_rays;
    const int64_t CH = 65536;
    std::vector<std::vector<float>> outf(71, std::vector<float>(CH));
    std::vector<std::vector<int>> outi(58, std::vector<int>(CH));
    std::vector<unsigned long long> cstats(10, 0ULL);
    float hxy[1] = {0}, hzy[1] = {0};
    float lt[1] = {0}, lp[1] = {0}, lew[1] = {0};
    unsigned int lec[1] = {0}, lac[1] = {0};
    double lst[1] = {0}, ldt[1] = {0};
    unsigned long long lsc[1] = {0}, let[1] = {0}, lat[1] = {0};
    unsigned int lerr[1] = {0}, lbadj[1] = {0}, lout[32] = {0};
    float ltx0[1], lty0[1], ltz0[1], ltx1[1], lty1[1], ltz1[1];
    int ltorder[1], ltevent[1], ltcount[1], ltover[1];
    const int threads = 256;
    for (int64_t start = 0; start < total; start += CH) {
        const int n = (int)std::min<int64_t>(CH, total - start);
        const unsigned global_start = run->ray_offset + (unsigned)start;
        for (int k = 0; k < 71; ++k) std::fill(outf[k].begin(), outf[k].begin() + n, NAN);
        for (int k = 0; k < 58; ++k) std::fill(outi[k].begin(), outi[k].begin() + n, 0);
        float** F = (float**)alloca(71 * sizeof(float*));
        int** I = (int**)alloca(58 * sizeof(int*));
        for (int k = 0; k < 71; ++k) F[k] = outf[k].data();
        for (int k = 0; k < 58; ++k) I[k] = outi[k].data();
#pragma omp parallel for schedule(dynamic, 1024)
        for (int i = 0; i < n; ++i) {
            set_index(threads, i);
            trace_kernel(
                P.max_iterations, S->muscal.data(), P.n_water, P.n_acrylic, P.n_air, P.wavelength, P.rough_alpha,
                P.spheroid_aspect, P.orientation_model, P.orientation_kappa, P.max_particle_bounces,
                P.max_cell_bounces, P.rin, P.rout, P.zmin, P.zmean, P.zwall_top, P.free_surface_model,
                P.vortex_delta_h, P.vortex_core_radius, P.bottom_disc_thickness, P.bottom_external_n,
                P.max_axial_bounces, P.ring_in, P.throat_out, P.ring_out, P.source_r, P.throat_r, P.counterbore_r,
                P.beam_sigma, 0, P.alpha1, P.alpha2, P.source_angular_model, P.source_bore_model, P.bore_n,
                P.max_bore_bounces, n, S->gcdf.data(), S->wcdf.data(), S->phase_cdf.data(), S->theta.data(), S->nt,
                S->nidx.data(), S->kidx.data(), S->radius.data(), S->n, S->qsca.data(), S->qext.data(),
                (P.event_model == 4 || P.event_model == 5) ? 1 : 0, P.conditional_retries, cstats.data(),
                S->moment_a.data(), S->moment_b.data(), S->moment_mode.data(), P.sediment_model,
                S->trace_geom.data(), S->trace_wave.data(), S->sed_A.data(), S->sed_B.data(), S->sed_norm.data(),
                S->sed_radial_log.data(), S->n_radial, S->sed_major.data(), S->sed_grid.data(), S->grid_nr,
                S->grid_nz, S->grid_zmax, hxy, hzy, 0, 0u, 1, 1, 1, P.zmean, lt, lp, lew, lec, lac, lst, ldt, lsc,
                let, lat, lerr, lbadj, lout, 0, 1, ltx0, lty0, ltz0, ltx1, lty1, ltz1, ltorder, ltevent, ltcount,
                ltover,
                F[0], F[1], F[2], F[3], F[4], F[5], F[6], F[7], F[8], F[9], F[10], F[11], F[12], F[13], F[14], F[15],
                F[16], F[17], F[18], F[19], F[20], F[21], F[22], F[23], F[24], F[25], F[26], F[27], F[28], F[29],
                F[30], F[31], F[32], F[33], F[34], F[35], F[36], F[37], F[38], F[39], F[40], F[41], F[42], F[43],
                F[44], F[45], F[46], F[47], F[48], F[49], F[50], F[51], F[52], F[53], F[54], F[55], F[56], F[57],
                F[58], F[59], F[60], F[61], F[62], F[63], F[64], F[65], F[66], F[67], F[68], F[69], F[70],
                I[0], I[1], I[2], I[3], I[4], I[5], I[6], I[7], I[8], I[9], I[10], I[11], I[12], I[13], I[14], I[15],
                I[16], I[17], I[18], I[19], I[20], I[21], I[22], I[23], I[24], I[25], I[26], I[27], I[28], I[29],
                I[30], I[31], I[32], I[33], I[34], I[35], I[36], I[37], I[38], I[39], I[40], I[41], I[42], I[43],
                I[44], I[45], I[46], I[47], I[48], I[49], I[50], I[51], I[52], I[53], I[54], I[55], I[56], I[57],
                run->seed0, run->seed1, run->seed2, global_start);
        }
        int hn[18] = {0}, hm[18] = {0}, hnd[18] = {0}, hmd[18] = {0}, hns[18] = {0}, hms[18] = {0}, hnf[18] = {0},
            hmf[18] = {0}, ln[18] = {0}, lm[18] = {0};
        float pdn[18] = {0}, pdm[18] = {0}, ian[18] = {0}, iam[18] = {0};
        std::vector<int> nid(n), mid(n), nbc(n), mbc(n), nfc(n), mfc(n);
#pragma omp parallel for schedule(dynamic, 1024)
        for (int i = 0; i < n; ++i) {
            set_index(threads, i);
            score_detectors_kernel(F[0], F[1], F[2], F[3], F[4], F[5], I[20], I[0], n, P.rout, P.ring_in,
                                   P.throat_out, P.ring_out, P.throat_r, P.counterbore_r, P.legacy_accept_deg,
                                   P.detector_bore_model, P.n_air, P.bore_n, P.max_bore_bounces, P.ring_face_model,
                                   P.ring_face_n, P.n_acrylic, P.max_ring_face_bounces, P.photodiode_model,
                                   run->detector_seed, global_start, hn, hm, hnd, hmd, hns, hms, hnf, hmf, pdn, pdm,
                                   ian, iam, ln, lm, nid.data(), mid.data(), nbc.data(), mbc.data(), nfc.data(),
                                   mfc.data());
        }
        for (int j = 0; j < 18; ++j) {
            T->hw_native[j] += hn[j]; T->hw_mirror[j] += hm[j];
            T->hw_native_direct[j] += hnd[j]; T->hw_mirror_direct[j] += hmd[j];
            T->hw_native_stray[j] += hns[j]; T->hw_mirror_stray[j] += hms[j];
            T->hw_native_face[j] += hnf[j]; T->hw_mirror_face[j] += hmf[j];
            T->legacy_native[j] += ln[j]; T->legacy_mirror[j] += lm[j];
            T->photodiode_native[j] += pdn[j]; T->photodiode_mirror[j] += pdm[j];
            T->incidence_native_sum[j] += ian[j]; T->incidence_mirror_sum[j] += iam[j];
            T->weight_native[j] += hn[j]; T->weight_mirror[j] += hm[j];
            T->weight_sq_native[j] += hn[j]; T->weight_sq_mirror[j] += hm[j];
        }
        for (int i = 0; i < n; ++i) {
            int st = I[20][i];
            if (st >= 0 && st < CLR_N_STATUS) T->status_counts[st]++;
            int pf = I[21][i];
            if (pf >= 0 && pf < CLR_N_FAILURE_CODES) T->failure_code_counts[pf]++;
            for (int k = 0; k < 20; ++k) T->event_counts[k] += I[k][i];
        }
        {
            for (int i = 0; i < n; ++i) {
                clr_ray_record tmp;
                memset(&tmp, 0, sizeof tmp);
                clr_ray_record& r = tmp;
                int32_t* ri = &r.status;
                /* record order: status, then outi[0..19], then failure code/subcode */
                ri[0] = I[20][i];
                for (int k = 0; k < 20; ++k) ri[1 + k] = I[k][i];
                r.failure_code = I[21][i]; r.failure_subcode = I[22][i];
                r.native_id = nid[i]; r.mirror_id = mid[i]; r.native_bounces = nbc[i]; r.mirror_bounces = mbc[i];
                r.air_x = F[0][i]; r.air_y = F[1][i]; r.air_z = F[2][i];
                r.air_vx = F[3][i]; r.air_vy = F[4][i]; r.air_vz = F[5][i];
                r.water_path = F[6][i]; r.acrylic_path = F[7][i];
                clr_tally_add_ray_stats(T, &r);
                if (records) records[start + i] = tmp;
                if (prov)
                    for (int k = 0; k < 13; ++k) prov[(start + i) * 13 + k] = I[35 + k][i];
                if (defl)
                    for (int k = 0; k < 5; ++k) defl[(start + i) * 5 + k] = F[8 + k][i];
            }
        }
    }
    T->n_rays = total;
    for (int k = 0; k < 10; ++k) T->conditional_stats[k] = cstats[k];
    return 0;
}

}  /* extern "C" */
