/* CPU oracle API (test infrastructure only).
 *
 * A plain-C restatement of the reference's photon-transport hot path: the
 * particle-physics precompute of ClaritasForwardModel._prepare_gpu_particle_physics
 * (CLARITAS/CLARITAS.py:6036-6965), trace_kernel (:4551-5104) and
 * score_detectors_kernel (:4378-4436), evaluated ray by ray on the host.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * always as the checker. The product library never links it.
 */
#ifndef CLARITAS_ORACLE_H
#define CLARITAS_ORACLE_H

#include "claritas_gb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct clo_state clo_state;

int clo_prepare(const clr_scene_params* scene, const clr_particle_spec* particles, const clr_sediment_spec* sediment,
                clo_state** out);
int clo_read_physics(clo_state* st, clr_particle_physics* out);
int clo_n_theta(clo_state* st);
/* as clo_trace, and per ray the provenance outputs of the reference (prov [n][13]: first/last event type,
 * last event order, first backscatter, first source hemisphere, first/last particle, geometric and wave
 * bin, acrylic returns after a particle event, particle events after a return; defl [n][5]: first/last
 * deflection in degrees, path and optical path inside particles, water path after the last event) */
int clo_trace_provenance(clo_state* st, const clr_run_params* run, clr_tallies* out, clr_ray_record* records,
                         int32_t* prov, float* defl, int n_threads);
/* the sediment coefficients of models 1-3 per bin: radial log coefficient (A), vertical inverse length (B),
 * normalisation, settling velocity, radial log lookup and (models 2, 3) radial slip velocity
 * [n_bins][n_radial] (any pointer may be NULL) */
int clo_read_sediment(clo_state* st, double* A, double* B, double* norm, double* ws, double* radial_log,
                      double* radial_slip);
/* the meridional secondary-circulation velocity (ur returned, uz through the pointer) at (r, z) */
double clo_meridional_velocity(int fsm, double r, double z, double zmin, double zmean, double R, double dh, double core,
                               double upeak, double* uz);
/* free-surface height at (x, y) and, when normal is not NULL, its unit normal (into the water) */
float clo_surface(int fsm, float x, float y, float zmean, float R, float dh, float core, float* normal);
/* first positive crossing of a ray with the free surface (FLT_MAX: none) */
float clo_surface_hit(int fsm, float x, float y, float z, float vx, float vy, float vz, float zmean, float R, float dh,
                      float core);
/* the sediment concentration scale of bin pidx at a point, as the trace looks it up (FP32 position) */
double clo_local_scale(clo_state* st, int pidx, float x, float y, float z);
/* 1 when (r, z) lies in the liquid (above the bottom, below the free surface) */
int clo_meridional_fluid(int fsm, double r, double z, double zmin, double zmean, double R, double dh, double core);
/* the sediment field [n_bins][nr][nz] of model 3 (solved or supplied) and the solver's iterations / residual */
int clo_read_sediment_field(clo_state* st, double* grid, int* nr, int* nz, int* iterations, double* max_residual);
int clo_trace(clo_state* st, const clr_run_params* run, clr_tallies* out, clr_ray_record* records, int n_threads);
const char* clo_last_error(clo_state* st);
void clo_free(clo_state* st);

/* unit entry points used by the oracle's own tests */
double clo_erfinv(double y);
int clo_philox4x32_10(const uint32_t key[2], const uint32_t ctr[4], uint32_t out[4]);

#ifdef __cplusplus
}
#endif

#endif
