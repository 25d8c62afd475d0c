// GPU driver for the reference's own device code (test infrastructure only).
//
// Built on a GPU machine into oracle/_ref/libclaritas_ref_gpu.so by
// tests/golden/make_gpu_fixtures.py (nvcc, sm_103a) from the reference source
// extracted by oracle/ref_extract.py. It replays the reference host's launch
// sequence: the precompute of _prepare_gpu_particle_physics
// (CLARITAS/CLARITAS.py:6147-6449, the meridional solver :6451-6725 or a supplied model-3 grid) and,
// per chunk, trace_kernel with its 234 arguments (:7638-7758) followed by
// score_detectors_kernel (:7783-7847) on 256-thread blocks. Its per-ray
// outputs are the bit-exact target for the library's xorshift parity mode.
#include <cstdio>
#include <cstring>
#include <vector>
#include <string>
#include <cuda_runtime.h>
#include "claritas_gb.h"
#include "tally_extras.h"

#include "_ref/claritas_cuda_src.inc"

namespace {

struct RefGpu {
    clr_scene_params sp;
    int n = 0, nt = 0, n_radial = 65, grid_nr = 2, grid_nz = 2;
    float grid_zmax = 0.f;
    std::vector<void*> allocs;
    double *d, *w_in, *wd, *nidx, *kidx, *agg, *x, *qext, *qsca, *qabs, *qback, *g, *albedo;
    int* nstop;
    double *theta, *phase_cdf, *radius, *pmass, *srcw, *nden, *sg, *ssca, *sext, *swave, *sevent, *mug, *mus, *mue,
        *muw, *muev, *pew, *gew, *wew, *gcdf, *wcdf, *pcdf, *muscal, *moment_a, *moment_b, *trace_geom, *trace_wave;
    unsigned char* moment_mode;
    double *sed_tau, *sed_ws, *sed_sre, *sed_sdrag, *sed_A, *sed_B, *sed_norm, *sed_max, *sed_min, *sed_rmax, *sed_rre,
        *sed_rcenter, *sed_radial_log, *sed_radial_wr, *sed_sc, *sed_sw, *sed_bc, *sed_bw, *sed_major, *sed_grid;
    int* err;
    int solver_iterations = 0;
    double solver_residual = 0.0;
    std::string msg;
};

template <class T>
cudaError_t dmalloc(RefGpu* S, T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) S->allocs.push_back(*p);
    return e;
}

int check(RefGpu* S, const char* what) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) { S->msg = std::string(what) + ": " + cudaGetErrorString(e); return -2; }
    int h = 0;
    cudaMemcpy(&h, S->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (h) { S->msg = std::string(what) + " error code " + std::to_string(h); return h; }
    return 0;
}

}  // namespace

extern "C" {

const char* clrefgpu_last_error(void* h) { return h ? ((RefGpu*)h)->msg.c_str() : "null"; }

void clrefgpu_free(void* h) {
    RefGpu* S = (RefGpu*)h;
    if (!S) return;
    for (void* p : S->allocs) cudaFree(p);
    delete S;
}

int clrefgpu_n_theta(void* h) { return h ? ((RefGpu*)h)->nt : 0; }

int clrefgpu_prepare(const clr_scene_params* sp, const clr_particle_spec* ps, const clr_sediment_spec* ss, void** out) {
    RefGpu* S = new RefGpu();
    *out = S;
    S->sp = *sp;
    const int n = ps->n_bins, M = 4096;
    S->n = n;
#define A(p, c) if (dmalloc(S, &S->p, c) != cudaSuccess) { S->msg = "alloc"; return -2; }
    A(d, n) A(w_in, n) A(wd, n) A(nidx, n) A(kidx, n) A(agg, 10) A(x, n) A(qext, n) A(qsca, n) A(qabs, n) A(qback, n)
    A(g, n) A(albedo, n) A(nstop, n) A(err, 1)
    cudaMemcpy(S->d, ps->diameter_m, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(S->w_in, ps->weight, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(S->nidx, ps->n_real, n * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(S->kidx, ps->k_imag, n * 8, cudaMemcpyHostToDevice);
    cudaMemset(S->err, 0, sizeof(int));
    orthokinetic_compact_aggregation_kernel<<<1, 1>>>(S->d, S->w_in, n, ps->concentration_kg_m3, ps->density_kg_m3, 0.0,
                                                      0.2, 200000, S->wd, S->agg, S->err);
    int rc = check(S, "PSD normalisation");
    if (rc) return rc;
    double *Dre, *Dim, *ar, *ai, *br, *bi;
    dmalloc(S, &Dre, (size_t)n * M); dmalloc(S, &Dim, (size_t)n * M); dmalloc(S, &ar, (size_t)n * M);
    dmalloc(S, &ai, (size_t)n * M); dmalloc(S, &br, (size_t)n * M); dmalloc(S, &bi, (size_t)n * M);
    const int threads = 128;
    mie_coefficients_efficiencies_kernel<<<(n + threads - 1) / threads, threads>>>(
        S->d, S->nidx, S->kidx, ps->n_medium, ps->wavelength_m, n, Dre, Dim, ar, ai, br, bi, S->nstop, S->x, S->qext,
        S->qsca, S->qabs, S->qback, S->g, S->albedo, S->err);
    rc = check(S, "Mie");
    if (rc) return rc;
    const int em = sp->event_model;
    if (em == 3 || em == 4 || em == 5) {
        const int nt = ps->n_theta;
        S->nt = nt;
        A(theta, nt) A(phase_cdf, (size_t)n * nt)
        double* pdf;
        dmalloc(S, &pdf, (size_t)n * nt);
        build_theta_grid_kernel<<<(nt + threads - 1) / threads, threads>>>(S->theta, nt);
        const long long total = (long long)n * nt;
        mie_phase_pdf_kernel<<<(unsigned)((total + threads - 1) / threads), threads>>>(S->theta, nt, n, S->nstop, ar, ai,
                                                                                        br, bi, pdf);
        mie_phase_cdf_kernel<<<n, 1>>>(S->theta, pdf, nt, n, S->phase_cdf, S->err);
    } else {
        S->nt = 2;
        A(theta, 2) A(phase_cdf, (size_t)2 * n)
        dummy_phase_kernel<<<(n + threads - 1) / threads > 0 ? (n + threads - 1) / threads : 1, threads>>>(S->theta, S->phase_cdf, n);
    }
    rc = check(S, "phase table");
    if (rc) return rc;
    A(radius, n) A(pmass, n) A(srcw, n) A(nden, n) A(sg, n) A(ssca, n) A(sext, n) A(swave, n) A(sevent, n) A(mug, n)
    A(mus, n) A(mue, n) A(muw, n) A(muev, n) A(pew, n) A(gew, n) A(wew, n) A(gcdf, n) A(wcdf, n) A(pcdf, n)
    A(muscal, 8)
    transport_precompute_kernel<<<1, 1>>>(S->d, S->wd, S->qext, S->qsca, S->kidx, n, ps->concentration_kg_m3,
                                          ps->density_kg_m3, ps->weight_mode, em, ps->hybrid_wave_scale, ps->n_medium,
                                          ps->wavelength_m, ps->wave_rms_height_m, S->radius, S->pmass, S->srcw,
                                          S->nden, S->sg, S->ssca, S->sext, S->swave, S->sevent, S->mug, S->mus, S->mue,
                                          S->muw, S->muev, S->pew, S->gew, S->wew, S->gcdf, S->wcdf, S->pcdf, S->muscal,
                                          S->err);
    rc = check(S, "transport precompute");
    if (rc) return rc;
    A(moment_a, n) A(moment_b, n) A(moment_mode, n)
    {
        std::vector<double> ma(n, 1.0), mb(n, 0.0);
        std::vector<unsigned char> mm(n, 0);
        if (ps->moment_enabled && ps->moment_a && ps->moment_b && ps->moment_mode)
            for (int i = 0; i < n; ++i) { ma[i] = ps->moment_a[i]; mb[i] = ps->moment_b[i]; mm[i] = ps->moment_mode[i]; }
        cudaMemcpy(S->moment_a, ma.data(), n * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(S->moment_b, mb.data(), n * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(S->moment_mode, mm.data(), n, cudaMemcpyHostToDevice);
    }
    A(trace_geom, n) A(trace_wave, n)
    {
        std::vector<double> mug(n), muw(n), muev(n), tg(n), tw(n);
        cudaMemcpy(mug.data(), S->mug, n * 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(muw.data(), S->muw, n * 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(muev.data(), S->muev, n * 8, cudaMemcpyDeviceToHost);
        for (int i = 0; i < n; ++i) {
            if (em == 3) { tg[i] = mug[i]; tw[i] = muw[i]; }
            else if (em == 4 || em == 5) { tg[i] = muev[i] - muw[i] > 0.0 ? muev[i] - muw[i] : 0.0; tw[i] = muw[i]; }
            else { tg[i] = muev[i]; tw[i] = 0.0; }
        }
        cudaMemcpy(S->trace_geom, tg.data(), n * 8, cudaMemcpyHostToDevice);
        cudaMemcpy(S->trace_wave, tw.data(), n * 8, cudaMemcpyHostToDevice);
    }
    const int NR = ss->n_radial;
    S->n_radial = NR;
    A(sed_tau, n) A(sed_ws, n) A(sed_sre, n) A(sed_sdrag, n) A(sed_A, n) A(sed_B, n) A(sed_norm, n) A(sed_max, n)
    A(sed_min, n) A(sed_rmax, n) A(sed_rre, n) A(sed_rcenter, n) A(sed_radial_log, (size_t)n * NR)
    A(sed_radial_wr, (size_t)n * NR) A(sed_sc, n) A(sed_sw, n) A(sed_bc, n) A(sed_bw, n) A(sed_major, 4)
    cudaMemset(S->sed_major, 0, 4 * 8);
    cudaMemset(S->err, 0, sizeof(int));
    // FP64 geometry as the reference's host passes it (:6413-6418), else the scene's FP32 values widened
    const bool g64 = ss->rin > 0.0;
    const double GR = g64 ? ss->rin : (double)sp->rin, GZMIN = g64 ? ss->zmin : (double)sp->zmin;
    const double GZMEAN = g64 ? ss->zmean : (double)sp->zmean;
    const double GDH = g64 ? ss->vortex_delta_h : (double)sp->vortex_delta_h;
    const double GCORE = g64 ? ss->vortex_core_radius : (double)sp->vortex_core_radius;
    sediment_transport_precompute_kernel<<<1, 1>>>(
        S->d, n, sp->sediment_model, ss->particle_density, ss->water_density, ss->water_viscosity, ss->gravity,
        ss->eddy_diffusivity, GR, GZMIN, GZMEAN, sp->free_surface_model,
        GDH, GCORE, ss->n_quad, NR, S->trace_geom, S->trace_wave,
        S->sed_tau, S->sed_ws, S->sed_sre, S->sed_sdrag, S->sed_A, S->sed_B, S->sed_norm, S->sed_max, S->sed_rmax,
        S->sed_rre, S->sed_rcenter, S->sed_radial_log, S->sed_radial_wr, S->sed_sc, S->sed_sw, S->sed_bc, S->sed_bw,
        S->sed_major, S->err);
    rc = check(S, "sediment precompute");
    if (rc) return rc;
    S->grid_zmax = (float)ss->grid_zmax;
    if (sp->sediment_model == 3 && !ss->grid) {
        // the reference's meridional solver, launched as its host does (:6451-6725)
        const int GNR = ss->meridional_nr, GNZ = ss->meridional_nz, FSM = sp->free_surface_model;
        S->grid_nr = GNR; S->grid_nz = GNZ;
        const size_t plane = (size_t)GNR * GNZ, total = plane * n;
        A(sed_grid, total)
        unsigned char* active;
        double *ap, *ae, *aw, *an, *as, *residual;
        dmalloc(S, &active, plane);
        dmalloc(S, &ap, total); dmalloc(S, &ae, total); dmalloc(S, &aw, total); dmalloc(S, &an, total);
        dmalloc(S, &as, total); dmalloc(S, &residual, n);
        const int th = 256, bp = (int)((plane + th - 1) / th), bt = (int)((total + th - 1) / th);
        const double ZG = ss->grid_zmax;
        meridional_active_mask_kernel<<<bp, th>>>(GNR, GNZ, GR, GZMIN, ZG, GZMEAN, FSM, GDH, GCORE, active);
        meridional_grid_initialize_kernel<<<bt, th>>>(n, GNR, GNZ, GR, GZMIN, ZG, FSM, GCORE, S->sed_A, S->sed_B,
                                                      S->sed_norm, S->sed_radial_log, NR, active, S->sed_grid);
        meridional_build_coefficients_kernel<<<bt, th>>>(n, GNR, GNZ, GR, GZMIN, ZG, GZMEAN, FSM, GDH, GCORE,
                                                         ss->meridional_peak_speed, ss->eddy_diffusivity, S->sed_ws,
                                                         S->sed_radial_wr, NR, active, ap, ae, aw, an, as);
        cudaMemset(S->err, 0, sizeof(int));
        meridional_normalize_kernel<<<n, 1>>>(n, GNR, GNZ, GR, GZMIN, ZG, GZMEAN, active, S->sed_grid, S->err);
        rc = check(S, "meridional initial normalization");
        if (rc) return rc;
        const int max_it = ss->solver_max_iterations, every = ss->solver_check_interval;
        const int min_it = max_it < 1000 ? max_it : 1000;
        int iters = 0, last = 0;
        std::vector<double> res(n, 0.0);
        for (int it = 1; it <= max_it; ++it) {
            meridional_relax_kernel<<<bt, th>>>(n, GNR, GNZ, 0, ss->solver_sor, active, ap, ae, aw, an, as, S->sed_grid);
            meridional_relax_kernel<<<bt, th>>>(n, GNR, GNZ, 1, ss->solver_sor, active, ap, ae, aw, an, as, S->sed_grid);
            if (it % 20 == 0)
                meridional_normalize_kernel<<<n, 1>>>(n, GNR, GNZ, GR, GZMIN, ZG, GZMEAN, active, S->sed_grid, S->err);
            if (it % every == 0 || it == max_it) {
                meridional_normalize_kernel<<<n, 1>>>(n, GNR, GNZ, GR, GZMIN, ZG, GZMEAN, active, S->sed_grid, S->err);
                meridional_residual_kernel<<<n, 1>>>(n, GNR, GNZ, active, ap, ae, aw, an, as, S->sed_grid, residual);
                rc = check(S, "meridional normalization");
                if (rc) return rc;
                cudaMemcpy(res.data(), residual, n * 8, cudaMemcpyDeviceToHost);
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
        if (mx > ss->solver_tolerance) { S->msg = "meridional transport solver did not converge"; return -7; }
        meridional_extend_grid_kernel<<<(n * GNR + th - 1) / th, th>>>(n, GNR, GNZ, active, S->sed_grid);
        meridional_finalize_kernel<<<n, 1>>>(n, GNR, GNZ, GR, GZMIN, ZG, active, S->sed_grid, S->sed_norm, S->sed_max,
                                             S->sed_min, S->sed_sc, S->sed_sw, S->sed_bc, S->sed_bw);
        meridional_majorants_kernel<<<1, 1>>>(n, S->trace_geom, S->trace_wave, S->sed_max, S->sed_major);
        rc = check(S, "meridional majorants");
        if (rc) return rc;
    } else if (sp->sediment_model == 3) {
        S->grid_nr = ss->grid_nr; S->grid_nz = ss->grid_nz;
        const size_t plane = (size_t)ss->grid_nr * ss->grid_nz;
        A(sed_grid, plane * n)
        cudaMemcpy(S->sed_grid, ss->grid, plane * n * 8, cudaMemcpyHostToDevice);
        unsigned char* active;
        dmalloc(S, &active, plane);
        cudaMemset(active, 1, plane);
        meridional_finalize_kernel<<<n, 1>>>(n, ss->grid_nr, ss->grid_nz, GR, GZMIN,
                                             ss->grid_zmax, active, S->sed_grid, S->sed_norm, S->sed_max, S->sed_min,
                                             S->sed_sc, S->sed_sw, S->sed_bc, S->sed_bw);
        meridional_majorants_kernel<<<1, 1>>>(n, S->trace_geom, S->trace_wave, S->sed_max, S->sed_major);
        rc = check(S, "grid majorants");
        if (rc) return rc;
    } else {
        A(sed_grid, 1)
        const double one = 1.0;
        cudaMemcpy(S->sed_grid, &one, 8, cudaMemcpyHostToDevice);
    }
    return 0;
#undef A
}

int clrefgpu_read_sediment_field(void* h, double* grid, int* nr, int* nz, int* iterations, double* max_residual) {
    RefGpu* S = (RefGpu*)h;
    if (nr) *nr = S->grid_nr;
    if (nz) *nz = S->grid_nz;
    if (iterations) *iterations = S->solver_iterations;
    if (max_residual) *max_residual = S->solver_residual;
    if (grid) cudaMemcpy(grid, S->sed_grid, (size_t)S->n * S->grid_nr * S->grid_nz * 8, cudaMemcpyDeviceToHost);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
}

int clrefgpu_read_physics(void* h, clr_particle_physics* o) {
    RefGpu* S = (RefGpu*)h;
    const int n = S->n;
    auto cp = [](double* dst, const double* src, size_t c) { if (dst) cudaMemcpy(dst, src, c * 8, cudaMemcpyDeviceToHost); };
    cp(o->size_parameter, S->x, n); cp(o->qext, S->qext, n); cp(o->qsca, S->qsca, n); cp(o->qabs, S->qabs, n);
    cp(o->qback, S->qback, n); cp(o->asym_g, S->g, n); cp(o->albedo, S->albedo, n);
    if (o->nstop) cudaMemcpy(o->nstop, S->nstop, n * 4, cudaMemcpyDeviceToHost);
    cp(o->radius, S->radius, n); cp(o->number_density, S->nden, n);
    cp(o->mu_geom_bin, S->mug, n); cp(o->mu_sca_bin, S->mus, n); cp(o->mu_ext_bin, S->mue, n);
    cp(o->mu_wave_bin, S->muw, n); cp(o->mu_event_bin, S->muev, n);
    cp(o->trace_geom_bin, S->trace_geom, n); cp(o->trace_wave_bin, S->trace_wave, n);
    cp(o->geometric_cdf, S->gcdf, n); cp(o->wave_cdf, S->wcdf, n); cp(o->particle_event_cdf, S->pcdf, n);
    cp(o->mu_scalars, S->muscal, 8); cp(o->sed_majorants, S->sed_major, 4); cp(o->theta, S->theta, S->nt);
    cp(o->phase_cdf, S->phase_cdf, (size_t)n * S->nt);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -2;
}

int clrefgpu_trace(void* h, const clr_run_params* run, clr_tallies* T, clr_ray_record* records) {
    RefGpu* S = (RefGpu*)h;
    const clr_scene_params& P = S->sp;
    memset(T, 0, sizeof *T);
    const long long total = run->n_rays;
    const int CH = 250000;  // CHUNK_SIZE, CLARITAS/CLARITAS.py:233
    std::vector<float*> F(71);
    std::vector<int*> I(58);
    for (int k = 0; k < 71; ++k) dmalloc(S, &F[k], CH);
    for (int k = 0; k < 58; ++k) dmalloc(S, &I[k], CH);
    unsigned long long* cstats; dmalloc(S, &cstats, 10); cudaMemset(cstats, 0, 80);
    float *hxy, *hzy, *lt, *lp, *lew, *ltx0, *lty0, *ltz0, *ltx1, *lty1, *ltz1;
    unsigned int *lec, *lac, *lerr, *lbadj, *lout;
    double *lst, *ldt;
    unsigned long long *lsc, *let, *lat;
    int *ltorder, *ltevent, *ltcount, *ltover;
    dmalloc(S, &hxy, 1); dmalloc(S, &hzy, 1); dmalloc(S, &lt, 1); dmalloc(S, &lp, 1); dmalloc(S, &lew, 1);
    dmalloc(S, &ltx0, 1); dmalloc(S, &lty0, 1); dmalloc(S, &ltz0, 1); dmalloc(S, &ltx1, 1); dmalloc(S, &lty1, 1);
    dmalloc(S, &ltz1, 1); dmalloc(S, &lec, 1); dmalloc(S, &lac, 1); dmalloc(S, &lerr, 1); dmalloc(S, &lbadj, 1);
    dmalloc(S, &lout, 32); dmalloc(S, &lst, 1); dmalloc(S, &ldt, 1); dmalloc(S, &lsc, 1); dmalloc(S, &let, 1);
    dmalloc(S, &lat, 1); dmalloc(S, &ltorder, 1); dmalloc(S, &ltevent, 1); dmalloc(S, &ltcount, 1);
    dmalloc(S, &ltover, 1);
    cudaMemset(lout, 0, 32 * 4);
    int *hn, *hm, *hnd, *hmd, *hns, *hms, *hnf, *hmf, *ln, *lm, *nid, *mid, *nbc, *mbc, *nfc, *mfc;
    float *pdn, *pdm, *ian, *iam;
    dmalloc(S, &hn, 18); dmalloc(S, &hm, 18); dmalloc(S, &hnd, 18); dmalloc(S, &hmd, 18); dmalloc(S, &hns, 18);
    dmalloc(S, &hms, 18); dmalloc(S, &hnf, 18); dmalloc(S, &hmf, 18); dmalloc(S, &ln, 18); dmalloc(S, &lm, 18);
    dmalloc(S, &pdn, 18); dmalloc(S, &pdm, 18); dmalloc(S, &ian, 18); dmalloc(S, &iam, 18);
    dmalloc(S, &nid, CH); dmalloc(S, &mid, CH); dmalloc(S, &nbc, CH); dmalloc(S, &mbc, CH); dmalloc(S, &nfc, CH);
    dmalloc(S, &mfc, CH);
    const int threads = 256;
    const float nanf_ = __builtin_nanf("");
    std::vector<float> nanbuf(CH, nanf_);
    std::vector<int> hi[58];
    std::vector<float> hf[8];
    std::vector<int> hnid(CH), hmid(CH), hnbc(CH), hmbc(CH);
    for (long long start = 0; start < total; start += CH) {
        const int n = (int)((total - start) < CH ? (total - start) : CH);
        const unsigned gstart = run->ray_offset + (unsigned)start;
        for (int k = 0; k < 71; ++k) cudaMemcpy(F[k], nanbuf.data(), n * 4, cudaMemcpyHostToDevice);
        for (int k = 0; k < 58; ++k) cudaMemset(I[k], 0, n * 4);
        const int blocks = (n + threads - 1) / threads;
        trace_kernel<<<blocks, threads>>>(
            P.max_iterations, S->muscal, P.n_water, P.n_acrylic, P.n_air, P.wavelength, P.rough_alpha, P.spheroid_aspect,
            P.orientation_model, P.orientation_kappa, P.max_particle_bounces, P.max_cell_bounces, P.rin, P.rout, P.zmin,
            P.zmean, P.zwall_top, P.free_surface_model, P.vortex_delta_h, P.vortex_core_radius, P.bottom_disc_thickness,
            P.bottom_external_n, P.max_axial_bounces, P.ring_in, P.throat_out, P.ring_out, P.source_r, P.throat_r,
            P.counterbore_r, P.beam_sigma, 0, P.alpha1, P.alpha2, P.source_angular_model, P.source_bore_model, P.bore_n,
            P.max_bore_bounces, n, S->gcdf, S->wcdf, S->phase_cdf, S->theta, S->nt, S->nidx, S->kidx, S->radius, S->n,
            S->qsca, S->qext, (P.event_model == 4 || P.event_model == 5) ? 1 : 0, P.conditional_retries, cstats,
            S->moment_a, S->moment_b, S->moment_mode, P.sediment_model, S->trace_geom, S->trace_wave, S->sed_A,
            S->sed_B, S->sed_norm, S->sed_radial_log, S->n_radial, S->sed_major, S->sed_grid, S->grid_nr, S->grid_nz,
            S->grid_zmax, hxy, hzy, 0, 0u, 1, 1, 1, P.zmean, lt, lp, lew, lec, lac, lst, ldt, lsc, let, lat, lerr, lbadj,
            lout, 0, 1, ltx0, lty0, ltz0, ltx1, lty1, ltz1, ltorder, ltevent, ltcount, ltover,
            F[0], F[1], F[2], F[3], F[4], F[5], F[6], F[7], F[8], F[9], F[10], F[11], F[12], F[13], F[14], F[15],
            F[16], F[17], F[18], F[19], F[20], F[21], F[22], F[23], F[24], F[25], F[26], F[27], F[28], F[29], F[30],
            F[31], F[32], F[33], F[34], F[35], F[36], F[37], F[38], F[39], F[40], F[41], F[42], F[43], F[44], F[45],
            F[46], F[47], F[48], F[49], F[50], F[51], F[52], F[53], F[54], F[55], F[56], F[57], F[58], F[59], F[60],
            F[61], F[62], F[63], F[64], F[65], F[66], F[67], F[68], F[69], F[70],
            I[0], I[1], I[2], I[3], I[4], I[5], I[6], I[7], I[8], I[9], I[10], I[11], I[12], I[13], I[14], I[15],
            I[16], I[17], I[18], I[19], I[20], I[21], I[22], I[23], I[24], I[25], I[26], I[27], I[28], I[29], I[30],
            I[31], I[32], I[33], I[34], I[35], I[36], I[37], I[38], I[39], I[40], I[41], I[42], I[43], I[44], I[45],
            I[46], I[47], I[48], I[49], I[50], I[51], I[52], I[53], I[54], I[55], I[56], I[57],
            run->seed0, run->seed1, run->seed2, gstart);
        int* zero18[] = {hn, hm, hnd, hmd, hns, hms, hnf, hmf, ln, lm};
        for (int* p : zero18) cudaMemset(p, 0, 18 * 4);
        float* zf18[] = {pdn, pdm, ian, iam};
        for (float* p : zf18) cudaMemset(p, 0, 18 * 4);
        score_detectors_kernel<<<blocks, threads>>>(
            F[0], F[1], F[2], F[3], F[4], F[5], I[20], I[0], n, P.rout, P.ring_in, P.throat_out, P.ring_out, P.throat_r,
            P.counterbore_r, P.legacy_accept_deg, P.detector_bore_model, P.n_air, P.bore_n, P.max_bore_bounces,
            P.ring_face_model, P.ring_face_n, P.n_acrylic, P.max_ring_face_bounces, P.photodiode_model,
            run->detector_seed, gstart, hn, hm, hnd, hmd, hns, hms, hnf, hmf, pdn, pdm, ian, iam, ln, lm, nid, mid, nbc,
            mbc, nfc, mfc);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { S->msg = cudaGetErrorString(e); return -2; }
        int h18[10][18];
        float f18[4][18];
        for (int k = 0; k < 10; ++k) cudaMemcpy(h18[k], zero18[k], 72, cudaMemcpyDeviceToHost);
        for (int k = 0; k < 4; ++k) cudaMemcpy(f18[k], zf18[k], 72, cudaMemcpyDeviceToHost);
        for (int j = 0; j < 18; ++j) {
            T->hw_native[j] += h18[0][j]; T->hw_mirror[j] += h18[1][j];
            T->hw_native_direct[j] += h18[2][j]; T->hw_mirror_direct[j] += h18[3][j];
            T->hw_native_stray[j] += h18[4][j]; T->hw_mirror_stray[j] += h18[5][j];
            T->hw_native_face[j] += h18[6][j]; T->hw_mirror_face[j] += h18[7][j];
            T->legacy_native[j] += h18[8][j]; T->legacy_mirror[j] += h18[9][j];
            T->photodiode_native[j] += f18[0][j]; T->photodiode_mirror[j] += f18[1][j];
            T->incidence_native_sum[j] += f18[2][j]; T->incidence_mirror_sum[j] += f18[3][j];
            T->weight_native[j] += h18[0][j]; T->weight_mirror[j] += h18[1][j];
        }
        for (int k = 0; k < 23; ++k) { hi[k].resize(n); cudaMemcpy(hi[k].data(), I[k], n * 4, cudaMemcpyDeviceToHost); }
        for (int k = 0; k < 8; ++k) { hf[k].resize(n); cudaMemcpy(hf[k].data(), F[k], n * 4, cudaMemcpyDeviceToHost); }
        cudaMemcpy(hnid.data(), nid, n * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(hmid.data(), mid, n * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(hnbc.data(), nbc, n * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(hmbc.data(), mbc, n * 4, cudaMemcpyDeviceToHost);
        for (int i = 0; i < n; ++i) {
            int st = hi[20][i];
            if (st >= 0 && st < CLR_N_STATUS) T->status_counts[st]++;
            int pf = hi[21][i];
            if (pf >= 0 && pf < CLR_N_FAILURE_CODES) T->failure_code_counts[pf]++;
            for (int k = 0; k < 20; ++k) T->event_counts[k] += hi[k][i];
            {
                clr_ray_record tmp;
                memset(&tmp, 0, sizeof tmp);
                clr_ray_record& r = tmp;
                int32_t* ri = &r.status;
                ri[0] = st;
                for (int k = 0; k < 20; ++k) ri[1 + k] = hi[k][i];
                r.failure_code = pf; r.failure_subcode = hi[22][i];
                r.native_id = hnid[i]; r.mirror_id = hmid[i]; r.native_bounces = hnbc[i]; r.mirror_bounces = hmbc[i];
                r.air_x = hf[0][i]; r.air_y = hf[1][i]; r.air_z = hf[2][i];
                r.air_vx = hf[3][i]; r.air_vy = hf[4][i]; r.air_vz = hf[5][i];
                r.water_path = hf[6][i]; r.acrylic_path = hf[7][i];
                clr_tally_add_ray_stats(T, &r);
                if (records) records[start + i] = tmp;
            }
        }
    }
    unsigned long long hc[10];
    cudaMemcpy(hc, cstats, 80, cudaMemcpyDeviceToHost);
    for (int k = 0; k < 10; ++k) T->conditional_stats[k] = hc[k];
    T->n_rays = total;
    // release the per-run buffers (they were appended to the allocation list)
    return 0;
}

}  // extern "C"
