// Device-resident description of one scenario: the scene scalars plus pointers
// to its particle tables, as consumed by the photon kernel. Built by the
// precompute path (precompute.cu) and uploaded once per scenario.
#pragma once
#include <cstdint>
#include "claritas_gb.h"

namespace clr {

// Light-history diagnostics of a trace (no effect on any history: no random draw, diagnostic buffers only).
// Voxel grids are [nz][ny][nx] over x, y in [-R, R] and z in [zmin, zmax]; heat maps [vis][vis].
struct LightDiag {
    int voxels;                             // voxel grids, events and trajectories on (heat maps are separate)
    int nx, ny, nz, max_rays, rep_rays, max_segments, vis;
    float zmax, zvis;                       // voxel box top; heat-map z range top (surface height at the wall)
    float *total, *post, *event_weight;     // track length, after >= 1 particle event; scatter-event weight
    unsigned *event_count;                  // scatter events per voxel
    double *seg_total, *dep_total;          // [1] clipped segment length, deposited length
    unsigned long long *seg_count, *event_total;
    unsigned *err_count, *adj_count, *outside;  // [1], [1], [8]: count, first outside x, y, z, gid, tol, set
    float *tx0, *ty0, *tz0, *tx1, *ty1, *tz1;   // [rep_rays][max_segments] representative trajectories
    int *torder, *tcount, *toverflow;           // [rep_rays][max_segments], [rep_rays], [rep_rays]
    float *heat_xy, *heat_zy;                   // [vis][vis] (vis 0: none)
};

// Guide cells per bin of the inverse-CDF phase-angle search: guide[k] is the first angle index whose CDF
// reaches k / kPhaseGuide (k = 0..kPhaseGuide), so a draw u in cell k = floor(u kPhaseGuide) searches only
// [guide[k], guide[k+1]] and finds the index the whole-table search finds.
constexpr int kPhaseGuide = 256;

struct DevScene {
    clr_scene_params P;
    // particle tables (float copies are exact casts of the FP64 tables, which is what the
    // reference compares against: CLARITAS/CLARITAS.py:2628, :2633-2637)
    const float* gcdf;
    const float* wcdf;
    const float* phase_cdf;     // [n_bins][nt]
    const int* phase_guide;     // [n_bins][kPhaseGuide + 1], or null (whole-table search)
    const float* theta;         // [nt]
    const float* pn;            // (float)n_real
    const float* pk;            // (float)k_imag
    const float* prad;          // (float)radius
    const double* k;            // k_imag
    const double* qsca;
    const double* qext;
    const double* moment_a;
    const double* moment_b;
    const uint8_t* moment_mode;
    const double* trace_geom;   // channel rates per bin (:6362-6375)
    const double* trace_wave;
    const double* sedA;
    const double* sedB;
    const double* sed_norm;
    const double* sed_radial_log;
    const double* sed_grid;
    const double* mu_channels;  // [8] transport_precompute_kernel output
    const double* sed_major;    // [4]
    // Node tables of the (r, z) field for the counter-based stream (sediment model 3 only): per node the
    // channel rates summed over bins, and per channel and node an alias table over bins. Null when absent.
    const float2* node_mu;      // [nr*nz] (geometric, wave)
    const int2* node_alias;     // [2][nr*nz][n_bins] (probability bits, alias bin)
    float node_major;           // max over nodes of the summed rate: a majorant of the interpolated field
    // FP32 casts of transport scalars the water step reads every flight (round-to-nearest casts of the
    // FP64 values, identical to casting on the device): mu_channels[0], [1], [7] and sed_major[0], [1]
    float mu_geom_f, mu_wave_f, coherent_f, sed_major_f[2];
    int32_t n_bins, nt, n_radial, grid_nr, grid_nz, any_moment;
    float grid_zmax;
    // run description of this scenario
    uint32_t seed0, seed1, seed2, det_seed, ray_offset, scenario_id;
    uint64_t philox_key;
    int64_t n_rays;
    int32_t weight_mode;
    float roulette_threshold, roulette_survival;
    int32_t pad;
    const LightDiag* light;     // null unless light-history diagnostics are on for this trace
    clr_path_provenance* prov;  // provenance partitions of detected rays; null unless counted for this trace
};

// Tally counters shared by the per-warp shared-memory tally and the per-scenario device tally.
// Layout: hw block, FP64 sums, then a contiguous tail of 64-bit counters.
struct TallyCore {
    unsigned long long hw[10][CLR_N_DETECTORS];   // native, mirror, nat direct, mir direct, nat stray, mir stray,
                                                  // nat face, mir face, legacy native, legacy mirror
    double sums[8][CLR_N_DETECTORS];              // photodiode nat/mir, incidence nat/mir, weight nat/mir, w^2 nat/mir
    unsigned long long status[CLR_N_STATUS];
    unsigned long long failure[CLR_N_FAILURE_CODES];
    unsigned long long events[CLR_N_EVENT_COUNTERS];
    unsigned long long cstats[CLR_N_CONDITIONAL_STATS];
    unsigned long long n_done;
    unsigned long long entered_sums[16];
    unsigned long long ray_flags[16];
    unsigned long long subcodes[CLR_N_SUBCODES];
    unsigned long long ic_lo[64];                 // interaction-count histogram, counts 0..63
};
#define CLR_TALLY_TAIL (CLR_N_STATUS + CLR_N_FAILURE_CODES + CLR_N_EVENT_COUNTERS + CLR_N_CONDITIONAL_STATS + 1 + 16 + 16 + CLR_N_SUBCODES + 64)

// Detector hits partitioned for the particle-path diagnostics of the reference's host
// (CLARITAS/CLARITAS.py:8019-8110: native [0] and mirror [1] detector ids of every detected ray), counted
// on the device instead of from per-ray arrays.
struct PathDiag {
    unsigned long long order[2][6][CLR_N_DETECTORS];       // by particle-interaction count 0,1,2,3,4,5+
    unsigned long long geom_order[2][6][CLR_N_DETECTORS];  // by geometric-event count 0,1,2,3,4,5+
    unsigned long long sums[CLR_N_PATH_SUMS][2][CLR_N_DETECTORS];  // per-ray counter sums (CLR_PS_*)
    unsigned long long masks[2][CLR_N_PATH_MASKS][CLR_N_DETECTORS];  // event-history masks (CLR_PM_*)
    unsigned long long acrylic_order[2][5][CLR_N_DETECTORS];         // by acrylic reflection count 0..3, 4+
};

// Per-scenario tallies in device memory: the core plus the high part of the histogram
// (interaction counts >= 64, clamped to the last bin), updated with global atomics.
struct DevTally {
    TallyCore c;
    unsigned long long ic_hi[CLR_IC_HIST];
    unsigned long long sched[16];
    PathDiag pd;
};

}  // namespace clr
