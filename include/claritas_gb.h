/* claritas_gb.h -- C ABI of the GB300 photon-transport library (libclaritas_gb.so).
 *
 * This library replaces the device half of the CLARITAS forward model:
 *   - trace_kernel          CLARITAS/CLARITAS.py:4551-5104 (234 launch arguments, launch :7638-7758)
 *   - score_detectors_kernel CLARITAS/CLARITAS.py:4378-4436 (47 launch arguments, launch :7783-7847)
 *   - the particle-physics precompute launched from
 *     ClaritasForwardModel._prepare_gpu_particle_physics, CLARITAS/CLARITAS.py:6036-6965:
 *     PSD normalisation (:3607-3635), Mie coefficients/efficiencies (:3495-3559),
 *     theta grid (:3488-3493), phase pdf (:3561-3581), phase cdf (:3583-3592),
 *     transport rates (:3845-3921), sediment coefficients and majorants (:3940-4038).
 * The reference binds these through CuPy RawModule launches with positional
 * numpy scalars and CuPy device arrays. Here the whole scene is one POD struct
 * and every call returns an int status (0 = success, negative = error); the text
 * of the last error is available from clr_last_error().
 *
 * Units: metres, kg/m^3 (= g/L), radians unless named otherwise. The coordinate
 * frame is the reference's: z = 0 at the sensor-ring plane, the LED bore at
 * 180 degrees launches along +y, detector j looks along (sin 10j deg, cos 10j deg).
 *
 * Threading: a context owns one CUDA stream and its device allocations; it must
 * not be used from two host threads at once. Calls are synchronous from the
 * caller's point of view.
 */
#ifndef CLARITAS_GB_H
#define CLARITAS_GB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLR_N_DETECTORS 18
#define CLR_MAX_BINS 64            /* AGG_MAX_BINS, CLARITAS/CLARITAS.py:3599 */
#define CLR_MIE_MAX_ORDER 4096     /* MIE_MAX_ORDER, CLARITAS/CLARITAS.py:1136 */
#define CLR_N_STATUS 16
#define CLR_N_FAILURE_CODES 32
#define CLR_N_EVENT_COUNTERS 24
#define CLR_N_CONDITIONAL_STATS 10

/* status codes returned by every entry point */
enum {
    CLR_OK = 0,
    CLR_ERR_INVALID_ARGUMENT = -1,
    CLR_ERR_CUDA = -2,
    CLR_ERR_NOT_READY = -3,
    CLR_ERR_UNSUPPORTED = -4,
    CLR_ERR_PRECOMPUTE = -5,   /* a precompute kernel raised its error word (reference error_flag) */
    CLR_ERR_DEVICE_TIMEOUT = -6
};

/* random-number back-ends */
enum {
    CLR_RNG_REFERENCE_XORSHIFT = 0, /* the reference's per-ray xorshift32 streams, bit-exact parity mode */
    CLR_RNG_PHILOX = 1              /* counter-based Philox4x32-10 keyed by (seed, scenario, photon) */
};

/* run flags */
enum {
    /* the counter-based stream uses the reference's own samplers everywhere, with no
       equivalent-distribution replacement (validates those replacements) */
    CLR_RUN_EXACT_SAMPLERS = 1,
    /* run the single persistent photon kernel instead of the wavefront engine (same per-ray results
       in the xorshift parity mode; kept for comparison and as the record-run fallback) */
    CLR_RUN_PERSISTENT_KERNEL = 2
};

/* photon weighting */
enum {
    CLR_WEIGHT_ANALOG = 0,   /* reference semantics: absorption is terminal, every weight is 1 */
    /* no reference counterpart (counter-based stream only): absorption is never sampled; at an absorbing
       particle the photon scatters and its weight is multiplied by the survival probability (the particle
       albedo in the conditional closure, exp(-alpha chord) per internal chord otherwise, exp(-mu_a d) per
       water flight); below roulette_threshold Russian roulette keeps it with probability
       w / roulette_survival at weight roulette_survival, else ends it with CLR_STATUS_ROULETTE. Detector
       weight sums (clr_tallies.weight_*) are then unbiased estimates of the analog hit counts. */
    CLR_WEIGHT_IMPLICIT = 1
};

/* photon end status (clr_tallies.status_counts): the reference's codes 0..8 (trace_kernel st,
 * CLARITAS/CLARITAS.py:4617-5066: 1 left into the air, 2 water-boundary exit, 3 rejected at the source,
 * 4 failure, 5 absorbed, 6 open top, 7 bottom exterior, 8 trapped), and one of this library's */
#define CLR_STATUS_ROULETTE 9       /* weighted runs: ended by Russian roulette */

/* source models */
enum {
    CLR_SOURCE_REFERENCE_LED = 0,  /* Gaussian spot + Beta angular law through the 180-degree bore */
    CLR_SOURCE_COLLIMATED_DISC = 1 /* uniform disc beam, launched at the inner wall, no collimator */
};

/* Scene description. Field names follow the ClaritasForwardModel constructor
 * (CLARITAS/CLARITAS.py:5577-5652) after its derived quantities
 * (zmin = -sensor_height, zmean = water_height - sensor_height, ... :5671-5699). */
typedef struct clr_scene_params {
    /* refractive indices */
    float n_water, n_acrylic, n_air, bore_n, ring_face_n, bottom_external_n;
    /* cell */
    float rin, rout, zmin, zmean, zwall_top, bottom_disc_thickness;
    /* sensor ring and bores */
    float ring_in, throat_out, ring_out, source_r, throat_r, counterbore_r;
    /* source */
    float beam_sigma, alpha1, alpha2, legacy_accept_deg;
    int32_t source_angular_model;   /* SOURCE_ANGULAR_MODEL_CODES :5553 */
    int32_t source_bore_model;      /* BORE_SURFACE_MODEL_CODES :5558 */
    int32_t detector_bore_model;
    int32_t ring_face_model;        /* RING_FACE_SURFACE_MODEL_CODES :5559 */
    int32_t photodiode_model;       /* PHOTODIODE_RESPONSE_MODEL_CODES :5560 */
    int32_t max_bore_bounces, max_ring_face_bounces;
    /* free surface */
    int32_t free_surface_model;     /* FREE_SURFACE_MODEL_CODES :5565 */
    float vortex_delta_h, vortex_core_radius;
    /* particle event law */
    float wavelength;               /* vacuum wavelength used inside particles */
    float rough_alpha;              /* tan(particle_surface_rms_slope_deg) */
    float spheroid_aspect, orientation_kappa;
    int32_t orientation_model;
    int32_t max_particle_bounces, max_cell_bounces, max_axial_bounces;
    float max_iterations;
    int32_t event_model;            /* EVENT_MODEL_CODES :5544 */
    int32_t conditional_retries;    /* CONDITIONAL_MAX_TRIALS :1117 */
    int32_t sediment_model;         /* SEDIMENT_TRANSPORT_MODEL_CODES :5570 */
    /* new source option (no reference counterpart; ignored when source_kind == CLR_SOURCE_REFERENCE_LED) */
    int32_t source_kind;
    float disc_radius;              /* collimated disc beam radius */
    float disc_height;              /* beam axis height z (same frame) */
    /* absorption coefficient of the water itself (1/m; no reference counterpart, whose water does not
     * absorb; 0 keeps the reference's transport and draw sequence). Analog runs end a photon at an
     * exponential absorption distance (status 5), weighted runs multiply its weight by exp(-mu_a d). */
    float water_absorption;
    int32_t reserved[3];
} clr_scene_params;

/* Particle population and the inputs of the Mie/rate precompute
 * (_prepare_gpu_particle_physics, CLARITAS/CLARITAS.py:6036-6330). */
typedef struct clr_particle_spec {
    int32_t n_bins;                 /* 1..CLR_MAX_BINS */
    int32_t n_theta;                /* mie_phase_grid_size; 2 selects the dummy 2-point table */
    int32_t weight_mode;            /* 0 mass_fraction, 1 number_fraction */
    int32_t moment_enabled;         /* 1 when moment_a/b/mode are supplied */
    const double* diameter_m;
    const double* weight;           /* PSD weights, normalised internally */
    const double* n_real;
    const double* k_imag;
    const double* moment_a;         /* nullable */
    const double* moment_b;         /* nullable */
    const uint8_t* moment_mode;     /* nullable */
    double concentration_kg_m3;
    double density_kg_m3;
    double n_medium;
    double wavelength_m;
    double wave_rms_height_m;
    double hybrid_wave_scale;
    /* Arithmetic of the phase tables (no reference counterpart): CLR_TABLES_REFERENCE (0) keeps the
     * reference's order of operations (bit-identical tables, required by the parity stream's bit-exact
     * contract); CLR_TABLES_FAST (1) evaluates the same sums with fused multiply-adds and two angles per
     * Legendre recurrence, ~4x less FP64 work, tables equal to rounding. */
    int32_t table_arithmetic;
    int32_t reserved_spec;
} clr_particle_spec;
#define CLR_TABLES_REFERENCE 0
#define CLR_TABLES_FAST 1

/* Inputs of the sediment coefficient precompute (CLARITAS/CLARITAS.py:3940-4038) and,
 * for sediment model 3, an externally supplied (r,z) concentration-scale grid laid
 * out [bin][ir][iz] as the reference's SED_GRID (:1537-1558). */
typedef struct clr_sediment_spec {
    double particle_density, water_density, water_viscosity, gravity, eddy_diffusivity;
    int32_t n_quad, n_radial;
    int32_t grid_nr, grid_nz;
    const double* grid;             /* sediment model 3: a supplied field, or NULL to solve it (below) */
    double grid_zmax;               /* top of the (r,z) grid: the free surface at the wall */
    /* FP64 cell geometry of the sediment precompute, as the reference passes it to those kernels
     * (float64 arguments, CLARITAS/CLARITAS.py:6413-6418); rin = 0 widens the scene's FP32 values */
    double rin, zmin, zmean, vortex_delta_h, vortex_core_radius;
    /* sediment model 3 with grid == NULL: the field is solved on the device on meridional_nr x
     * meridional_nz cells, the reference's meridional advection-diffusion solver
     * (CLARITAS/CLARITAS.py:4040-4215 driven by :6451-6725; defaults 48 x 96, 8000 iterations, check
     * every 250, tolerance 1e-6, SOR 1.75; peak speed = circulation ratio x peak azimuthal speed) */
    int32_t meridional_nr, meridional_nz, solver_max_iterations, solver_check_interval;
    double solver_tolerance, solver_sor, meridional_peak_speed;
} clr_sediment_spec;

/* One transport run over a contiguous range of global ray ids. The three
 * transport seeds and the detector seed are the reference's derived seeds
 * (simulate, CLARITAS/CLARITAS.py:7304-7306 and :7780-7782). */
typedef struct clr_run_params {
    int64_t n_rays;
    uint32_t ray_offset;
    uint32_t seed0, seed1, seed2, detector_seed;
    int32_t rng_mode;               /* CLR_RNG_* */
    uint64_t philox_key;            /* CLR_RNG_PHILOX: 64-bit key */
    uint32_t scenario_id;           /* CLR_RNG_PHILOX: folded into the counter */
    int32_t weight_mode;            /* CLR_WEIGHT_* */
    float roulette_threshold;       /* CLR_WEIGHT_IMPLICIT only */
    float roulette_survival;        /* weight given to survivors; probability = w / survival */
    int32_t max_blocks;             /* 0 = occupancy-derived grid; >0 caps the resident blocks (tuning, tests) */
    int32_t rays_per_item;          /* work-queue granularity; 0 = default */
    int32_t flags;                  /* CLR_RUN_* bits */
    int32_t reserved[3];
} clr_run_params;

/* Per-ray record, written only when a record buffer is passed to clr_trace
 * (parity tests). Integer fields are the reference's per-ray outputs
 * (trace_kernel :5070-5103, score_detectors_kernel :4396-4411). air_* are NaN
 * unless status == 1, as in the reference's NaN-initialised outputs (:7635). */
typedef struct clr_ray_record {
    int32_t status, interaction_count, geometric, wave, coherent, morphology;
    int32_t particle_reflections, entry_reflections, internal_reflections, absorptions;
    int32_t cell_inner_reflections, cell_outer_reflections, cell_tir;
    int32_t top_reflections, top_tir, bottom_inner_reflections, bottom_outer_reflections, bottom_tir;
    int32_t source_bore_interactions, source_bore_reflections, entered_water;
    int32_t failure_code, failure_subcode;
    int32_t native_id, mirror_id, native_bounces, mirror_bounces;
    float air_x, air_y, air_z, air_vx, air_vy, air_vz;
    float water_path, acrylic_path;
} clr_ray_record;

/* indices into clr_tallies.path_sums: per-channel sums over detected rays of their interaction,
 * geometric, wave, coherent-wave, morphology-wave, particle entry-reflection and internal-reflection
 * counts (the reference's path_*_sums, CLARITAS/CLARITAS.py:8033-8056) */
#define CLR_N_PATH_SUMS 7
enum { CLR_PS_INTERACTIONS = 0, CLR_PS_GEOMETRIC, CLR_PS_WAVE, CLR_PS_COHERENT, CLR_PS_MORPHOLOGY,
       CLR_PS_ENTRY_REFLECTIONS, CLR_PS_INTERNAL_REFLECTIONS };

/* indices into clr_tallies.path_mask_hits: the reference's per-ray event-history masks
 * (_event_history_masks, CLARITAS/CLARITAS.py:5265-5321, in its key order), predicates over the ray's
 * interaction (ic), geometric (g), wave (w), coherent (coh), morphology (mor) counts and its particle
 * entry-reflection (per), internal-reflection (pir) and absorption (pabs) counts */
#define CLR_N_PATH_MASKS 25
enum {
    CLR_PM_ANY_PARTICLE = 0,        /* ic > 0 */
    CLR_PM_ANY_GEOMETRIC,           /* g > 0 */
    CLR_PM_ANY_WAVE,                /* w > 0 */
    CLR_PM_ANY_COHERENT_WAVE,       /* coh > 0 */
    CLR_PM_ANY_MORPHOLOGY_WAVE,     /* mor > 0 */
    CLR_PM_ANY_ENTRY_REFLECTION,    /* per > 0 */
    CLR_PM_ANY_INTERNAL_REFLECTION, /* pir > 0 */
    CLR_PM_BALLISTIC,               /* ic == 0 */
    CLR_PM_SINGLE,                  /* ic == 1 */
    CLR_PM_SINGLE_ENTRY_REFLECTION, /* ic == 1, per > 0 */
    CLR_PM_MULTIPLE,                /* ic >= 2 */
    CLR_PM_ORDER_2, CLR_PM_ORDER_3, CLR_PM_ORDER_4PLUS,
    CLR_PM_EXACTLY_ONE_GEOMETRIC,   /* ic == 1, g == 1, w == 0 */
    CLR_PM_EXACTLY_ONE_WAVE,        /* ic == 1, g == 0, w == 1 */
    CLR_PM_SINGLE_COHERENT_ESCAPE,  /* ic == 1, coh == 1 */
    CLR_PM_SINGLE_ENTRY_REFLECTION_ESCAPE,    /* ic == 1, per > 0 */
    CLR_PM_SINGLE_INTERNAL_REFLECTION_ESCAPE, /* ic == 1, pir > 0 */
    CLR_PM_SINGLE_TRANSMISSION_ESCAPE,        /* ic == 1, (g > 0 or mor > 0), per == pir == pabs == 0 */
    CLR_PM_MIXED_GEOMETRIC_WAVE,    /* ic >= 2, g > 0, w > 0 */
    CLR_PM_GEOMETRIC_ONLY_MULTIPLE, /* ic >= 2, g > 0, w == 0 */
    CLR_PM_WAVE_ONLY_MULTIPLE,      /* ic >= 2, g == 0, w > 0 */
    CLR_PM_MULTIPLE_ENTRY_REFLECTION,    /* ic >= 2, per > 0 */
    CLR_PM_MULTIPLE_INTERNAL_REFLECTION  /* ic >= 2, pir > 0 */
};

/* indices into clr_tallies.event_counts (sums of per-ray counters over the run) */
enum {
    CLR_EV_INTERACTIONS = 0, CLR_EV_GEOMETRIC, CLR_EV_WAVE, CLR_EV_COHERENT, CLR_EV_MORPHOLOGY,
    CLR_EV_PARTICLE_REFLECTIONS, CLR_EV_ENTRY_REFLECTIONS, CLR_EV_INTERNAL_REFLECTIONS, CLR_EV_ABSORPTIONS,
    CLR_EV_CELL_INNER, CLR_EV_CELL_OUTER, CLR_EV_CELL_TIR, CLR_EV_TOP, CLR_EV_TOP_TIR,
    CLR_EV_BOTTOM_INNER, CLR_EV_BOTTOM_OUTER, CLR_EV_BOTTOM_TIR,
    CLR_EV_SOURCE_BORE_INTERACTIONS, CLR_EV_SOURCE_BORE_REFLECTIONS, CLR_EV_ENTERED_WATER,
    CLR_EV_WATER_STEPS,       /* free-flight steps in water (the unit of the roofline work count) */
    CLR_EV_NULL_COLLISIONS,   /* Woodcock rejections and inaccessible-placement nulls */
    CLR_EV_ROULETTE_KILLS,
    CLR_EV_RESERVED
};

#define CLR_N_SUBCODES 96
#define CLR_IC_HIST 1024

/* indices into clr_tallies.entered_sums (over rays with entered_water > 0) */
enum {
    CLR_ES_IC = 0, CLR_ES_GIC, CLR_ES_WIC, CLR_ES_WCOH, CLR_ES_WMORPH, CLR_ES_PR, CLR_ES_CIR, CLR_ES_COR,
    CLR_ES_TOP, CLR_ES_BIR, CLR_ES_BOR, CLR_ES_CTIR, CLR_ES_TTIR, CLR_ES_BTIR, CLR_ES_PER, CLR_ES_PIR
};
/* indices into clr_tallies.ray_flags */
enum {
    CLR_RF_ENTERED = 0, CLR_RF_BALLISTIC, CLR_RF_ENTRY_REFLECTED, CLR_RF_INTERNAL_REFLECTED, CLR_RF_ABSORBED,
    CLR_RF_CELL_TIR, CLR_RF_TOP_TIR, CLR_RF_BOTTOM_TIR, CLR_RF_SOURCE_ACCEPTED, CLR_RF_SOURCE_DIRECT,
    CLR_RF_SOURCE_REFLECTED, CLR_RF_VALID_AIR, CLR_RF_TRAPPED
};

/* Compact index of a production failure subcode (CLARITAS/CLARITAS.py:1808-1895):
 * 0..47 themselves; 1001..1007 -> 48..54; 1101..1107 -> 55..61; 2001..2002 -> 62..63;
 * 2101..2104 -> 64..67; 3001..3006 -> 68..73; 4001 -> 74; 9001..9003 -> 75..77; other -> 95. */
#define CLR_SUBCODE_INDEX(s)                                                              \
    (((s) >= 0 && (s) < 48) ? (s)                                                         \
     : ((s) >= 1001 && (s) <= 1007) ? 48 + (s) - 1001                                     \
     : ((s) >= 1101 && (s) <= 1107) ? 55 + (s) - 1101                                     \
     : ((s) >= 2001 && (s) <= 2002) ? 62 + (s) - 2001                                     \
     : ((s) >= 2101 && (s) <= 2104) ? 64 + (s) - 2101                                     \
     : ((s) >= 3001 && (s) <= 3006) ? 68 + (s) - 3001                                     \
     : ((s) == 4001) ? 74                                                                 \
     : ((s) >= 9001 && (s) <= 9003) ? 75 + (s) - 9001 : 95)

/* Detector tallies of one run. Integer counts are exact; float sums are FP64. */
typedef struct clr_tallies {
    int64_t n_rays;
    int64_t hw_native[CLR_N_DETECTORS], hw_mirror[CLR_N_DETECTORS];
    int64_t hw_native_direct[CLR_N_DETECTORS], hw_mirror_direct[CLR_N_DETECTORS];
    int64_t hw_native_stray[CLR_N_DETECTORS], hw_mirror_stray[CLR_N_DETECTORS];
    int64_t hw_native_face[CLR_N_DETECTORS], hw_mirror_face[CLR_N_DETECTORS];
    int64_t legacy_native[CLR_N_DETECTORS], legacy_mirror[CLR_N_DETECTORS];
    double photodiode_native[CLR_N_DETECTORS], photodiode_mirror[CLR_N_DETECTORS];
    double incidence_native_sum[CLR_N_DETECTORS], incidence_mirror_sum[CLR_N_DETECTORS];
    double weight_native[CLR_N_DETECTORS], weight_mirror[CLR_N_DETECTORS];
    double weight_sq_native[CLR_N_DETECTORS], weight_sq_mirror[CLR_N_DETECTORS];
    int64_t status_counts[CLR_N_STATUS];
    int64_t failure_code_counts[CLR_N_FAILURE_CODES];
    int64_t event_counts[CLR_N_EVENT_COUNTERS];
    uint64_t conditional_stats[CLR_N_CONDITIONAL_STATS];
    int32_t device_error;           /* nonzero if the kernel did not account for every ray */
    int32_t reserved[7];
    /* per-ray statistics the reference's host derives from its per-ray arrays (simulate,
     * CLARITAS/CLARITAS.py:8659-8735); see CLR_ES_* and CLR_RF_* for the indices */
    int64_t entered_sums[16];       /* sums over rays that entered the water */
    int64_t ray_flags[16];          /* counts of rays satisfying a predicate */
    int64_t failure_subcode_counts[CLR_N_SUBCODES];  /* indexed by clr_subcode_index() */
    int64_t ic_hist[CLR_IC_HIST];   /* interaction count of entered rays; last bin = overflow */
    /* scheduler profile of the photon kernel (no reference counterpart): per phase
     * (0 source, 1 entry, 2 water) the warp iterations [k], the lanes that ran [4+k] and the
     * SM clock cycles spent [8+k]; [11] cycles spent scoring finished histories */
    int64_t sched_stats[16];
    /* detected rays partitioned for the particle-path diagnostics (the reference's host partitions of its
     * per-ray arrays, CLARITAS/CLARITAS.py:8019-8110): index 0 native, 1 mirror detector id */
    int64_t order_hits[2][6][CLR_N_DETECTORS];            /* by particle-interaction count 0,1,2,3,4,5+ */
    int64_t geometric_order_hits[2][6][CLR_N_DETECTORS];  /* by geometric-event count 0,1,2,3,4,5+ */
    int64_t path_sums[CLR_N_PATH_SUMS][2][CLR_N_DETECTORS];  /* sums of per-ray counters (CLR_PS_*) */
    int64_t path_mask_hits[2][CLR_N_PATH_MASKS][CLR_N_DETECTORS];  /* rays satisfying each CLR_PM_* mask */
    /* by acrylic reflection count (cell inner + outer + bottom inner + outer reflections) 0,1,2,3,4+
     * (:8114-8123) */
    int64_t acrylic_order_hits[2][5][CLR_N_DETECTORS];
} clr_tallies;

/* Host copies of the particle-physics tables (diagnostics and parity checks).
 * Arrays are caller-owned; any pointer may be NULL to skip that output. */
typedef struct clr_particle_physics {
    double* size_parameter; double* qext; double* qsca; double* qabs; double* qback;
    double* asym_g; double* albedo; int32_t* nstop;
    double* radius; double* number_density;
    double* mu_geom_bin; double* mu_sca_bin; double* mu_ext_bin; double* mu_wave_bin; double* mu_event_bin;
    double* trace_geom_bin; double* trace_wave_bin;
    double* geometric_cdf; double* wave_cdf; double* particle_event_cdf;
    double* mu_scalars;            /* [8], transport_precompute_kernel :3908-3920 */
    double* sed_majorants;         /* [4] */
    double* theta;                 /* [n_theta] */
    double* phase_cdf;             /* [n_bins * n_theta] */
} clr_particle_physics;

typedef struct clr_ctx clr_ctx;

/* Context lifetime. Replaces ClaritasForwardModel.__init__'s RawModule build
 * (CLARITAS/CLARITAS.py:6000-6033); kernels are compiled ahead of time. */
int clr_create(clr_ctx** out, int device);
int clr_destroy(clr_ctx* ctx);
const char* clr_last_error(const clr_ctx* ctx);
const char* clr_version(void);

/* Store the scene parameters (the scalar half of the trace_kernel/score_detectors_kernel
 * argument lists, CLARITAS/CLARITAS.py:4551-4560 and :4378-4384). */
int clr_set_scene(clr_ctx* ctx, const clr_scene_params* scene);

/* Run the whole particle-physics precompute on the device and keep its tables resident:
 * replaces _prepare_gpu_particle_physics (CLARITAS/CLARITAS.py:6036-6965). */
int clr_build_particles(clr_ctx* ctx, const clr_particle_spec* particles, const clr_sediment_spec* sediment);

/* Copy the resident tables back (CLARITAS/CLARITAS.py:6774, phase_table_diagnostics :7146). */
int clr_read_particle_physics(clr_ctx* ctx, clr_particle_physics* out);

/* Trace n_rays photons and score them: replaces one simulate() chunk loop
 * (CLARITAS/CLARITAS.py:7614-7864). `records` is a DEVICE pointer to n_rays
 * clr_ray_record entries, or NULL for the tally-only hot path. */
int clr_trace(clr_ctx* ctx, const clr_run_params* run, clr_tallies* out, clr_ray_record* records);

/* Light-history diagnostics of the following traces of the current scene (the reference's
 * simulate(light_transport_config=..., heatmap_size=...), CLARITAS/CLARITAS.py:7229-7300): for rays with
 * global id < max_rays every water segment's track length is deposited into an nx x ny x nz voxel grid
 * over x, y in [-rin, rin] and z in [zmin, zmax] by an exact FP64 traversal (also into a second grid
 * once the ray has had a particle event), accepted particle-event sites are counted per voxel, the
 * first representative_rays rays keep up to max_segments_per_ray clipped segments, and (heatmap_size
 * > 0, every ray) every 10 um of water path adds one count to x-y and z-y heat maps. Nothing here draws a random
 * number or changes a history. The buffers are zeroed by this call and accumulate over the following
 * traces of the context until it is called again. */
typedef struct clr_light_config {
    int32_t enabled;                /* voxel grids, events and trajectories; 0 with heatmap_size 0: all off */
    int32_t nx, ny, nz;             /* voxels per axis, each >= 4 */
    int32_t max_rays;               /* >= 1 */
    int32_t representative_rays, max_segments_per_ray;
    int32_t heatmap_size;           /* 0: no heat maps */
    float zmax;                     /* voxel box top: the higher of the free surface's centre and wall heights */
    float heat_zmax;                /* heat-map z range top: the free surface height at the wall */
} clr_light_config;
int clr_set_light_diagnostics(clr_ctx* ctx, const clr_light_config* config);

/* Results of the last trace with light diagnostics on; every array pointer may be NULL. */
typedef struct clr_light_result {
    float* track_length;            /* [nz][ny][nx] */
    float* post_scatter_track_length;
    float* scatter_event_weight;
    uint32_t* scatter_event_count;
    float* heatmap_xy;              /* [heatmap_size][heatmap_size] */
    float* heatmap_zy;
    float *trajectory_x0, *trajectory_y0, *trajectory_z0, *trajectory_x1, *trajectory_y1, *trajectory_z1;
    int32_t* trajectory_order;      /* [representative_rays][max_segments_per_ray]: particle events before */
    int32_t* trajectory_count;      /* [representative_rays] */
    int32_t* trajectory_overflow;   /* [representative_rays] */
    double segment_length_total, deposited_length_total;
    int64_t segment_count, scatter_event_total;
    int64_t error_count, boundary_adjustment_count, event_outside_count;
    float first_outside_xyz_tol[4]; /* first event outside the box: x, y, z, tolerance */
    uint32_t first_outside_ray, first_outside_set;
} clr_light_result;
int clr_read_light_diagnostics(clr_ctx* ctx, clr_light_result* out);

/* Particle-event provenance of detected rays: the reference's causal partitions of its per-ray
 * provenance arrays (first/last particle, geometric and wave bin, first/last event type and deflection,
 * acrylic returns; trace_kernel :4625-4647, :4966-4979, :5005-5058, host :8063-8160, :8470-8481),
 * counted on the device. While enabled (clr_set_path_provenance), every clr_trace / clr_trace_batch of
 * the current scene adds its detected rays into one clr_path_provenance (reset at each call, summed over
 * the runs of the call); the wavefront engine counts them, the persistent kernel refuses the run.
 * Index [side]: 0 the native, 1 the mirrored detector id. Event type codes (:4625-4628): 1 geometric
 * external reflection, 2 geometric transmission/refraction, 3 geometric internal-reflection path,
 * 4 coherent Mie wave, 5..7 the morphology-wave 1..3; 0 none. */
enum { CLR_PB_FIRST_PARTICLE = 0, CLR_PB_LAST_PARTICLE, CLR_PB_FIRST_GEOMETRIC, CLR_PB_LAST_GEOMETRIC,
       CLR_PB_FIRST_WAVE, CLR_PB_LAST_WAVE, CLR_PB_COUNT };
enum { CLR_WALL_ZERO_PARTICLE = 0, CLR_WALL_NO_ACRYLIC_RETURN, CLR_WALL_ACRYLIC_RETURN };
#define CLR_N_EVENT_TYPES 8
#define CLR_N_H170_ANGLE_BINS 6     /* last/first deflection bins [0,30,60,90,120,150,180.0001) deg */
typedef struct clr_path_provenance {
    int64_t bin_hits[CLR_PB_COUNT][2][CLR_MAX_BINS][CLR_N_DETECTORS];  /* rays by first/last bin (CLR_PB_*) */
    int64_t first_type_hits[2][CLR_N_EVENT_TYPES][CLR_N_DETECTORS];   /* by type of the first event */
    int64_t last_type_hits[2][CLR_N_EVENT_TYPES][CLR_N_DETECTORS];    /* by type of the last event */
    int64_t wall_hits[2][3][CLR_N_DETECTORS];           /* CLR_WALL_*: no event / events, no return / return */
    int64_t after_return_hits[2][CLR_N_DETECTORS];      /* a particle event after an acrylic return */
    int64_t first_backscatter_hits[2][CLR_N_DETECTORS]; /* first event turned the ray back (cos < 0) */
    int64_t first_source_hemisphere_hits[2][CLR_N_DETECTORS];  /* leaving the first event with vy < 0 */
    double first_angle_sum[2][CLR_N_DETECTORS];         /* deflection (deg) sums and counts, first event */
    int64_t first_angle_count[2][CLR_N_DETECTORS];
    double last_angle_sum[2][CLR_N_DETECTORS];          /* and last event */
    int64_t last_angle_count[2][CLR_N_DETECTORS];
    double last_type_angle_sum[2][CLR_N_EVENT_TYPES][CLR_N_DETECTORS];  /* last deflection by last type */
    int64_t last_type_angle_count[2][CLR_N_EVENT_TYPES][CLR_N_DETECTORS];
    int64_t h170_last_angle_hits[2][CLR_N_EVENT_TYPES][CLR_N_H170_ANGLE_BINS];  /* detector 17; row 0: all */
    int64_t h170_first_angle_hits[2][CLR_N_H170_ANGLE_BINS];
} clr_path_provenance;
int clr_set_path_provenance(clr_ctx* ctx, int enabled);
int clr_read_path_provenance(clr_ctx* ctx, clr_path_provenance* out);
/* Per-ray provenance of the last single-run trace that wrote per-ray records with provenance on (the
 * reference's per-ray outputs :4601-4603, :4580; parity tests): out [n_rays][4] words per ray,
 *   [0] bytes 0..3: first / last particle bin, first / last geometric bin (0xFF none)
 *   [1] bytes 0, 1: first / last wave bin; bits 16-19 first and 20-23 last event type; bit 24 first event
 *       backscatter; 25 first event into the source hemisphere (vy < 0); 26 an acrylic (or headspace)
 *       return after a particle event; 27 a particle event after such a return
 *   [2], [3]: first / last deflection (deg) as float bits, -1 before any event */
int clr_read_path_provenance_records(clr_ctx* ctx, uint32_t* out, int64_t n_rays);

/* Trace n_runs runs of the current scene in one engine execution (one persistent-kernel launch or
 * one sequence of wavefront passes): each run has its own photon range, seeds and tallies
 * (outs[n_runs]). The runs share rng_mode, weight_mode and flags. Replaces the reference's chunk loop
 * when the caller wants per-batch tallies (batch jackknife, CLARITAS/CLARITAS.py:5244, :7638-7862). */
int clr_trace_batch(clr_ctx* ctx, const clr_run_params* runs, int n_runs, clr_tallies* outs);

/* Scenario sweep (the batched-sweep caller of the reference, run_one_case over many scenarios,
 * CLARITAS/CLARITAS.py:13020): builds the particle tables of n_scenarios scenes, each with its own
 * scene parameters, particles and sediment (scenes[i], particles[i], sediments[i]), with the
 * arithmetic of clr_set_scene + clr_build_particles, so every scenario's tables equal those of a
 * single build. The Mie coefficient and phase-table kernels run over the bins of many scenarios per
 * launch. Replaces the previous sweep of the context (the current single scene is not touched).
 * Errors name the first failing scenario; a precompute error code applies to the whole sweep. */
int clr_sweep_build(clr_ctx* ctx, int n_scenarios, const clr_scene_params* scenes, const clr_particle_spec* particles,
                    const clr_sediment_spec* sediments);

/* Trace every scenario of the built sweep in one engine execution: runs[i] (photon count, seeds,
 * ray offset) traces scenario i, tallies into outs[i]; n_runs must equal the sweep's scenario count
 * and the runs share rng_mode, weight_mode and flags. */
int clr_sweep_trace(clr_ctx* ctx, const clr_run_params* runs, int n_runs, clr_tallies* outs);

/* The resident (r,z) sediment field of the current scene (sediment model 3): grid_out (nullable)
 * receives [bins][nr][nz] doubles (the solved field after the reference's column extension, or the
 * supplied one); iterations and max_residual (nullable) the solver's iteration count and final largest
 * residual (0 for a supplied grid), the reference's meridional_solver_iterations / _max_residual. */
int clr_read_sediment_field(clr_ctx* ctx, double* grid_out, int32_t* nr, int32_t* nz, int32_t* iterations,
                            double* max_residual);

/* clr_read_particle_physics for scenario `scenario` of the built sweep. */
int clr_sweep_read_particle_physics(clr_ctx* ctx, int scenario, clr_particle_physics* out);

/* Same as clr_trace with HOST-resident record memory (copied back inside the call). */
int clr_trace_host_records(clr_ctx* ctx, const clr_run_params* run, clr_tallies* out, clr_ray_record* host_records);

/* Device time of the photon transport in the last clr_trace* / clr_sweep_trace call, or of the
 * precompute in the last clr_sweep_build, measured with CUDA events recorded on the context's stream
 * around its launches and copies (milliseconds). No reference counterpart. */
int clr_last_kernel_ms(const clr_ctx* ctx, float* ms);

/* Kernel launches of the last clr_trace call (the wavefront engine launches one graph of 12 kernel
 * nodes per pass plus one initialisation kernel; the persistent kernel is one launch) and the number
 * of wavefront passes (0 for the persistent kernel). No reference counterpart. */
int clr_last_launches(const clr_ctx* ctx, int64_t* launches, int64_t* passes);

/* Settings of the wavefront engine (no reference counterpart; the reference launches one thread per ray).
 * They change how the work is scheduled, never a photon's draws or arithmetic: integer tallies are the same
 * for any settings. Zero selects the default. stage_blocks[q] caps the resident blocks per SM of the stage
 * kernel of queue q (order GEN, ENTRY, FLIGHT, COND, GEOM, MORPH, TOP, BOTTOM, SIDE, ACRYL, FIN). */
#define CLR_ENGINE_DEFAULT_FLIGHT_STEPS 4
#define CLR_ENGINE_DEFAULT_TAIL_PHOTONS 65536
#define CLR_ENGINE_DEFAULT_RARE_BATCH 8192
#define CLR_ENGINE_DEFAULT_PASS_BATCH 8
#define CLR_ENGINE_DEFAULT_ACR_BUDGET 256
#define CLR_ENGINE_ACR_BUDGET_STEP 64
#define CLR_N_STAGES 11
typedef struct clr_engine_config {
    int32_t flight_steps;           /* water flights per FLIGHT visit, 1..64 */
    int32_t tail_photons;           /* photons in flight at which the single-thread tail kernel takes over */
    int32_t rare_batch;             /* queue length at which a rare stage (MORPH, TOP, BOTTOM) runs */
    int32_t stage_blocks[CLR_N_STAGES];
    int32_t pass_batch;             /* pass graphs queued between two reads of the live flag */
    int32_t acr_budget;             /* bounces per piece of an acrylic traversal while photons are drawn
                                     * (a multiple of CLR_ENGINE_ACR_BUDGET_STEP) */
    int32_t reserved[2];
} clr_engine_config;
/* Use `config` for the following traces of the context (NULL: back to the defaults). */
int clr_set_engine_config(clr_ctx* ctx, const clr_engine_config* config);

/* Engine profile of the last clr_trace* / clr_sweep_trace call (no reference counterpart), the first n of:
 * [0] wavefront pass graphs launched, [1] kernel launches, [2] photons handed to the tail kernel (0 when it
 * did not run), [3] tail-kernel device time (ms, CUDA events around its launch), [4] the call's device time
 * (ms, as clr_last_kernel_ms). */
int clr_last_engine_stats(const clr_ctx* ctx, double* out, int n);

/* Calibration kernels for roofline denominators (no reference counterpart): sustained
 * arithmetic throughput of this device in operations per second, counting a fused
 * multiply-add as two operations. which = 0: FP32 FFMA; which = 1: FP64 DFMA. */
int clr_calibrate(clr_ctx* ctx, int which, double* ops_per_second);

/* Allocation-free Mie tables (no reference counterpart; the reference always allocates through
 * CuPy). For callers that must not allocate device memory: a loop whose device memory belongs to
 * another framework's pool, where a cudaMalloc/cudaFree per iteration would synchronise the device.
 * Computes, for n_bins <= CLR_NOALLOC_MAX_BINS (16) particle bins and
 * 2 <= n_theta <= CLR_NOALLOC_MAX_THETA (4097) angles, the extinction and scattering efficiencies,
 * the asymmetry parameter, the theta grid and the per-bin phase CDF -- the same kernels and values as
 * clr_build_particles -- into caller-owned DEVICE buffers (d_qext, d_qsca, d_asym_g: [n_bins];
 * d_theta: [n_theta]; d_phase_cdf: [n_bins][n_theta]) on `stream` (a cudaStream_t, or NULL for the
 * context's stream). The inputs d_diameter_m, d_n_real, d_k_imag are device arrays of n_bins doubles.
 * No memory is allocated or freed: the scratch is a fixed set of file-scope device arrays (about 3 MB
 * per device, held by every device that loads the library until the process exits) whose addresses
 * are resolved on the first call for each device and kept for the life of the process, so calls after
 * a cudaDeviceReset of that device are not supported. The scratch is shared by every context on a
 * device, so calls that overlap on one device race: serialise them. Only the error word is reset per
 * call; the call then copies it to the host and synchronises `stream`, so it must not be called while
 * `stream` is being captured into a CUDA graph. It returns CLR_ERR_PRECOMPUTE with "error code k" on a
 * Mie failure (the scratch stays usable for the next call), and CLR_ERR_INVALID_ARGUMENT (with the
 * limits in the message) for sizes beyond the scratch. */
#define CLR_NOALLOC_MAX_BINS 16
#define CLR_NOALLOC_MAX_THETA 4097
int clr_mie_phase_noalloc(clr_ctx* ctx, const double* d_diameter_m, const double* d_n_real, const double* d_k_imag,
                          int n_bins, double n_medium, double wavelength_m, int n_theta, double* d_qext,
                          double* d_qsca, double* d_asym_g, double* d_theta, double* d_phase_cdf, void* stream);

/* Sizes of the ABI structs as compiled into the library (0 scene, 1 particle spec, 2 sediment spec,
 * 3 run params, 4 ray record, 5 tallies, 6 particle physics, 7 path provenance, 8 engine config); -1 for an
 * unknown index.
 * No reference counterpart: lets a binding check its struct mirror against the library. */
int64_t clr_abi_sizeof(int which);

/* ---------------------------------------------------------------------------------------------
 * Surrogate network of the detector signals (no reference counterpart: the reference runs a full
 * Monte Carlo for every scenario query). A multilayer perceptron
 *   CLR_MLP_INPUTS -> CLR_MLP_WIDTH (x4 hidden layers, SiLU) -> CLR_MLP_OUTPUTS
 * with BF16 weights and activations and FP32 accumulation; its 256x256 layers (forward,
 * backward-data and weight-gradient products) run on the tensor cores (tcgen05), the rest on CUDA
 * cores. FP32 master weights, Adam (beta1 0.9, beta2 0.999, eps 1e-8), mean-squared-error loss over
 * the outputs. Inputs and targets are device FP32 arrays [n][CLR_MLP_INPUTS] / [n][CLR_MLP_OUTPUTS]
 * in whatever normalisation the caller trains with. Parameters are one flat FP32 vector: W1 [256][6],
 * b1, W2 [256][256], b2, W3, b3, W4, b4, W5 [3][256], b5.
 * ------------------------------------------------------------------------------------------- */
#define CLR_MLP_INPUTS 6
#define CLR_MLP_WIDTH 256
#define CLR_MLP_OUTPUTS 3
#define CLR_MLP_PARAMS 199939
typedef struct clr_mlp clr_mlp;

/* max_batch: rows of the work buffers (a multiple of 128); weights drawn uniform in
 * +-1/sqrt(fan_in) from `seed`. */
int clr_mlp_create(clr_mlp** out, int device, int max_batch, uint64_t seed);
int clr_mlp_destroy(clr_mlp* net);
const char* clr_mlp_last_error(const clr_mlp* net);
int clr_mlp_set_params(clr_mlp* net, const float* host_params, int64_t count);  /* resets Adam */
int clr_mlp_get_params(clr_mlp* net, float* host_params, int64_t count);
/* d_y[n][3] = network(d_x[n][6]) for any n (processed in max_batch chunks) on `stream` (NULL: the
 * network's own), synchronous. */
int clr_mlp_forward(clr_mlp* net, const float* d_x, int64_t n, float* d_y, void* stream);
/* Loss and gradient of one batch of n rows (a multiple of 128, at most max_batch) without an update:
 * grads_host[CLR_MLP_PARAMS] (nullable) and the mean squared error. */
int clr_mlp_gradients(clr_mlp* net, const float* d_x, const float* d_t, int64_t n, float* grads_host, float* loss);
/* Adam steps over d_index[0 .. n_index) in batches of `batch` rows (a multiple of 128): each step
 * gathers its rows of d_x/d_t by index, runs forward and backward and updates; the step is one CUDA
 * graph launch. mean_loss: the mean batch loss of the call. */
int clr_mlp_train(clr_mlp* net, const float* d_x, const float* d_t, const int32_t* d_index, int64_t n_index,
                  int batch, float lr, float* mean_loss);
/* Per-output loss weights for the following clr_mlp_gradients / clr_mlp_train calls: d_w[row][3] on the
 * device, rows indexed like their d_t (the caller keeps it alive); NULL returns to the unweighted loss.
 * The loss becomes sum w (y - t)^2 / (3 n); weights of 1/variance give each label its likelihood weight. */
int clr_mlp_set_loss_weights(clr_mlp* net, const float* d_w);
/* Device time of the last clr_mlp_forward / clr_mlp_train call (CUDA events on its stream), ms. */
int clr_mlp_last_ms(const clr_mlp* net, float* ms);
/* C[M][256] = A[M][K] . B[256][K]^T on the tensor cores: BF16 row-major operands (K a multiple of
 * 64, leading dimensions multiples of 8 elements, 16-byte aligned), FP32 result (ldc >= 256),
 * synchronous on `stream`. */
int clr_bf16_gemm_n256(const void* d_a, int64_t lda, const void* d_b, int64_t ldb, int64_t M, int64_t K, float* d_c,
                       int64_t ldc, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CLARITAS_GB_H */
