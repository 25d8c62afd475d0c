"""ctypes mirror of include/claritas_gb.h (the library's C ABI).

Every Structure here has the same field order and C types as its C counterpart;
tests/test_abi.py checks the sizes against the compiled library's own
``clr_abi_sizeof`` export.
"""
from __future__ import annotations

import ctypes as C

N_DETECTORS = 18
MAX_BINS = 64
MIE_MAX_ORDER = 4096
N_STATUS = 16
N_FAILURE_CODES = 32
N_EVENT_COUNTERS = 24
N_CONDITIONAL_STATS = 10
N_SUBCODES = 96
IC_HIST = 1024
N_PATH_SUMS = 7  # CLR_N_PATH_SUMS
# CLR_PM_* in order: the reference's event-history mask keys (CLARITAS/CLARITAS.py:5287-5320)
PATH_MASK_NAMES = (
    "any_particle", "any_geometric", "any_wave", "any_coherent_wave", "any_morphology_wave",
    "any_entry_reflection", "any_internal_reflection", "ballistic", "single_interaction",
    "single_entry_reflection", "multiple_interaction", "interaction_order_2", "interaction_order_3",
    "interaction_order_4plus", "exactly_one_geometric", "exactly_one_wave", "single_coherent_wave_escape",
    "single_external_entry_reflection_escape", "single_internal_reflection_escape",
    "single_surface_transmission_escape", "mixed_geometric_wave", "geometric_only_multiple", "wave_only_multiple",
    "multiple_with_entry_reflection", "multiple_with_internal_reflection")
N_PATH_MASKS = len(PATH_MASK_NAMES)  # CLR_N_PATH_MASKS
ES_NAMES = ["ic", "gic", "wic", "wcoh", "wmorph", "pr", "cir", "cor", "top", "bir", "bor", "ctir", "ttir", "btir",
            "per", "pir"]
RF_NAMES = ["entered", "ballistic", "entry_reflected", "internal_reflected", "absorbed", "cell_tir", "top_tir",
            "bottom_tir", "source_accepted", "source_direct", "source_reflected", "valid_air", "trapped"]


def subcode_index(s: int) -> int:
    """Compact index of a production failure subcode (CLR_SUBCODE_INDEX in include/claritas_gb.h)."""
    if 0 <= s < 48:
        return s
    for lo, hi, base in ((1001, 1007, 48), (1101, 1107, 55), (2001, 2002, 62), (2101, 2104, 64), (3001, 3006, 68),
                         (4001, 4001, 74), (9001, 9003, 75)):
        if lo <= s <= hi:
            return base + s - lo
    return 95


def subcode_of_index(i: int) -> int:
    """Inverse of subcode_index for the named ranges (95 maps to -1: 'other')."""
    if i < 48:
        return i
    for lo, hi, base in ((1001, 1007, 48), (1101, 1107, 55), (2001, 2002, 62), (2101, 2104, 64), (3001, 3006, 68),
                         (4001, 4001, 74), (9001, 9003, 75)):
        if base <= i <= base + hi - lo:
            return lo + i - base
    return -1

CLR_OK = 0
CLR_ERR_INVALID_ARGUMENT = -1
CLR_ERR_CUDA = -2
CLR_ERR_NOT_READY = -3
CLR_ERR_UNSUPPORTED = -4
CLR_ERR_PRECOMPUTE = -5
CLR_ERR_DEVICE_TIMEOUT = -6

RNG_REFERENCE_XORSHIFT = 0
RNG_PHILOX = 1
RUN_EXACT_SAMPLERS = 1
RUN_PERSISTENT_KERNEL = 2
WEIGHT_ANALOG = 0
WEIGHT_IMPLICIT = 1
SOURCE_REFERENCE_LED = 0
SOURCE_COLLIMATED_DISC = 1
STATUS_ABSORBED = 5
STATUS_ROULETTE = 9  # weighted runs: ended by Russian roulette (CLR_STATUS_ROULETTE)

EV_NAMES = [
    "interactions", "geometric", "wave", "coherent", "morphology",
    "particle_reflections", "entry_reflections", "internal_reflections", "absorptions",
    "cell_inner", "cell_outer", "cell_tir", "top", "top_tir",
    "bottom_inner", "bottom_outer", "bottom_tir",
    "source_bore_interactions", "source_bore_reflections", "entered_water",
    "water_steps", "null_collisions", "roulette_kills", "reserved",
]

f32, f64, i32, u32, i64, u64 = C.c_float, C.c_double, C.c_int32, C.c_uint32, C.c_int64, C.c_uint64
PD = C.POINTER(C.c_double)
PI32 = C.POINTER(C.c_int32)
PU8 = C.POINTER(C.c_uint8)


class SceneParams(C.Structure):
    _fields_ = [
        ("n_water", f32), ("n_acrylic", f32), ("n_air", f32), ("bore_n", f32), ("ring_face_n", f32),
        ("bottom_external_n", f32),
        ("rin", f32), ("rout", f32), ("zmin", f32), ("zmean", f32), ("zwall_top", f32),
        ("bottom_disc_thickness", f32),
        ("ring_in", f32), ("throat_out", f32), ("ring_out", f32), ("source_r", f32), ("throat_r", f32),
        ("counterbore_r", f32),
        ("beam_sigma", f32), ("alpha1", f32), ("alpha2", f32), ("legacy_accept_deg", f32),
        ("source_angular_model", i32), ("source_bore_model", i32), ("detector_bore_model", i32),
        ("ring_face_model", i32), ("photodiode_model", i32),
        ("max_bore_bounces", i32), ("max_ring_face_bounces", i32),
        ("free_surface_model", i32), ("vortex_delta_h", f32), ("vortex_core_radius", f32),
        ("wavelength", f32), ("rough_alpha", f32), ("spheroid_aspect", f32), ("orientation_kappa", f32),
        ("orientation_model", i32), ("max_particle_bounces", i32), ("max_cell_bounces", i32),
        ("max_axial_bounces", i32),
        ("max_iterations", f32),
        ("event_model", i32), ("conditional_retries", i32), ("sediment_model", i32),
        ("source_kind", i32), ("disc_radius", f32), ("disc_height", f32), ("water_absorption", f32),
        ("reserved", i32 * 3),
    ]


class ParticleSpec(C.Structure):
    _fields_ = [
        ("n_bins", i32), ("n_theta", i32), ("weight_mode", i32), ("moment_enabled", i32),
        ("diameter_m", PD), ("weight", PD), ("n_real", PD), ("k_imag", PD),
        ("moment_a", PD), ("moment_b", PD), ("moment_mode", PU8),
        ("concentration_kg_m3", f64), ("density_kg_m3", f64), ("n_medium", f64), ("wavelength_m", f64),
        ("wave_rms_height_m", f64), ("hybrid_wave_scale", f64), ("table_arithmetic", i32), ("reserved_spec", i32),
    ]


class SedimentSpec(C.Structure):
    _fields_ = [
        ("particle_density", f64), ("water_density", f64), ("water_viscosity", f64), ("gravity", f64),
        ("eddy_diffusivity", f64),
        ("n_quad", i32), ("n_radial", i32), ("grid_nr", i32), ("grid_nz", i32),
        ("grid", PD), ("grid_zmax", f64),
        ("rin", f64), ("zmin", f64), ("zmean", f64), ("vortex_delta_h", f64), ("vortex_core_radius", f64),
        ("meridional_nr", i32), ("meridional_nz", i32), ("solver_max_iterations", i32),
        ("solver_check_interval", i32), ("solver_tolerance", f64), ("solver_sor", f64),
        ("meridional_peak_speed", f64),
    ]


class RunParams(C.Structure):
    _fields_ = [
        ("n_rays", i64), ("ray_offset", u32), ("seed0", u32), ("seed1", u32), ("seed2", u32),
        ("detector_seed", u32), ("rng_mode", i32), ("philox_key", u64), ("scenario_id", u32),
        ("weight_mode", i32), ("roulette_threshold", f32), ("roulette_survival", f32),
        ("max_blocks", i32), ("rays_per_item", i32), ("flags", i32), ("reserved", i32 * 3),
    ]


class RayRecord(C.Structure):
    _fields_ = [(n, i32) for n in (
        "status", "interaction_count", "geometric", "wave", "coherent", "morphology",
        "particle_reflections", "entry_reflections", "internal_reflections", "absorptions",
        "cell_inner_reflections", "cell_outer_reflections", "cell_tir",
        "top_reflections", "top_tir", "bottom_inner_reflections", "bottom_outer_reflections", "bottom_tir",
        "source_bore_interactions", "source_bore_reflections", "entered_water",
        "failure_code", "failure_subcode", "native_id", "mirror_id", "native_bounces", "mirror_bounces",
    )] + [(n, f32) for n in ("air_x", "air_y", "air_z", "air_vx", "air_vy", "air_vz", "water_path",
                            "acrylic_path")]


RECORD_INT_FIELDS = [n for n, t in RayRecord._fields_ if t is i32]
RECORD_FLOAT_FIELDS = [n for n, t in RayRecord._fields_ if t is f32]


class Tallies(C.Structure):
    _fields_ = [
        ("n_rays", i64),
        ("hw_native", i64 * N_DETECTORS), ("hw_mirror", i64 * N_DETECTORS),
        ("hw_native_direct", i64 * N_DETECTORS), ("hw_mirror_direct", i64 * N_DETECTORS),
        ("hw_native_stray", i64 * N_DETECTORS), ("hw_mirror_stray", i64 * N_DETECTORS),
        ("hw_native_face", i64 * N_DETECTORS), ("hw_mirror_face", i64 * N_DETECTORS),
        ("legacy_native", i64 * N_DETECTORS), ("legacy_mirror", i64 * N_DETECTORS),
        ("photodiode_native", f64 * N_DETECTORS), ("photodiode_mirror", f64 * N_DETECTORS),
        ("incidence_native_sum", f64 * N_DETECTORS), ("incidence_mirror_sum", f64 * N_DETECTORS),
        ("weight_native", f64 * N_DETECTORS), ("weight_mirror", f64 * N_DETECTORS),
        ("weight_sq_native", f64 * N_DETECTORS), ("weight_sq_mirror", f64 * N_DETECTORS),
        ("status_counts", i64 * N_STATUS),
        ("failure_code_counts", i64 * N_FAILURE_CODES),
        ("event_counts", i64 * N_EVENT_COUNTERS),
        ("conditional_stats", u64 * N_CONDITIONAL_STATS),
        ("device_error", i32), ("reserved", i32 * 7),
        ("entered_sums", i64 * 16), ("ray_flags", i64 * 16),
        ("failure_subcode_counts", i64 * N_SUBCODES), ("ic_hist", i64 * IC_HIST),
        ("sched_stats", i64 * 16),
        ("order_hits", i64 * N_DETECTORS * 6 * 2), ("geometric_order_hits", i64 * N_DETECTORS * 6 * 2),
        ("path_sums", i64 * N_DETECTORS * 2 * N_PATH_SUMS),
        ("path_mask_hits", i64 * N_DETECTORS * N_PATH_MASKS * 2), ("acrylic_order_hits", i64 * N_DETECTORS * 5 * 2),
    ]

    def as_dict(self) -> dict:
        import numpy as np
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            if hasattr(v, "_length_"):
                out[name] = np.ctypeslib.as_array(v).copy()
            else:
                out[name] = v
        return out


class ParticlePhysics(C.Structure):
    _fields_ = [(n, PD) for n in (
        "size_parameter", "qext", "qsca", "qabs", "qback", "asym_g", "albedo")] + [("nstop", PI32)] + [
        (n, PD) for n in (
            "radius", "number_density", "mu_geom_bin", "mu_sca_bin", "mu_ext_bin", "mu_wave_bin", "mu_event_bin",
            "trace_geom_bin", "trace_wave_bin", "geometric_cdf", "wave_cdf", "particle_event_cdf",
            "mu_scalars", "sed_majorants", "theta", "phase_cdf")]


PHYSICS_BIN_FIELDS = [
    "size_parameter", "qext", "qsca", "qabs", "qback", "asym_g", "albedo", "radius", "number_density",
    "mu_geom_bin", "mu_sca_bin", "mu_ext_bin", "mu_wave_bin", "mu_event_bin", "trace_geom_bin",
    "trace_wave_bin", "geometric_cdf", "wave_cdf", "particle_event_cdf",
]


def alloc_physics(n_bins: int, n_theta: int):
    """Allocate numpy outputs for clr_read_particle_physics and a struct pointing at them."""
    import numpy as np
    arrays = {k: np.zeros(n_bins, dtype=np.float64) for k in PHYSICS_BIN_FIELDS}
    arrays["nstop"] = np.zeros(n_bins, dtype=np.int32)
    arrays["mu_scalars"] = np.zeros(8, dtype=np.float64)
    arrays["sed_majorants"] = np.zeros(4, dtype=np.float64)
    arrays["theta"] = np.zeros(n_theta, dtype=np.float64)
    arrays["phase_cdf"] = np.zeros(n_bins * n_theta, dtype=np.float64)
    pp = ParticlePhysics()
    for k, a in arrays.items():
        setattr(pp, k, a.ctypes.data_as(PI32 if k == "nstop" else PD))
    return pp, arrays


def records_to_numpy(buf, n: int):
    """View a RayRecord buffer (ctypes array or bytes-like) as a structured numpy array."""
    import numpy as np
    dt = np.dtype([(nm, np.int32) for nm in RECORD_INT_FIELDS] + [(nm, np.float32) for nm in RECORD_FLOAT_FIELDS])
    assert dt.itemsize == C.sizeof(RayRecord)
    return np.frombuffer(buf, dtype=dt, count=n)


def record_dtype():
    import numpy as np
    return np.dtype([(nm, np.int32) for nm in RECORD_INT_FIELDS] + [(nm, np.float32) for nm in RECORD_FLOAT_FIELDS])


# clr_path_provenance: CLR_PB_* rows of bin_hits, CLR_WALL_* rows of wall_hits, event type codes
PROVENANCE_BIN_NAMES = ("first_particle_bin", "last_particle_bin", "first_geometric_bin", "last_geometric_bin",
                        "first_wave_bin", "last_wave_bin")
WALL_PATH_NAMES = ("zero_particle", "particle_no_acrylic_return", "particle_with_acrylic_return")
N_EVENT_TYPES = 8  # CLR_N_EVENT_TYPES
N_H170_ANGLE_BINS = 6  # CLR_N_H170_ANGLE_BINS
PARTICLE_EVENT_TYPE_NAMES = {1: "geometric_external_entry_reflection", 2: "geometric_surface_transmission_refraction",
                             3: "geometric_internal_reflection_path", 4: "coherent_mie_wave",
                             5: "morphology_wave_external_entry_reflection",
                             6: "morphology_wave_surface_transmission_refraction",
                             7: "morphology_wave_internal_reflection_path"}


class PathProvenance(C.Structure):
    _fields_ = [
        ("bin_hits", i64 * N_DETECTORS * MAX_BINS * 2 * len(PROVENANCE_BIN_NAMES)),
        ("first_type_hits", i64 * N_DETECTORS * N_EVENT_TYPES * 2),
        ("last_type_hits", i64 * N_DETECTORS * N_EVENT_TYPES * 2),
        ("wall_hits", i64 * N_DETECTORS * 3 * 2),
        ("after_return_hits", i64 * N_DETECTORS * 2),
        ("first_backscatter_hits", i64 * N_DETECTORS * 2),
        ("first_source_hemisphere_hits", i64 * N_DETECTORS * 2),
        ("first_angle_sum", f64 * N_DETECTORS * 2), ("first_angle_count", i64 * N_DETECTORS * 2),
        ("last_angle_sum", f64 * N_DETECTORS * 2), ("last_angle_count", i64 * N_DETECTORS * 2),
        ("last_type_angle_sum", f64 * N_DETECTORS * N_EVENT_TYPES * 2),
        ("last_type_angle_count", i64 * N_DETECTORS * N_EVENT_TYPES * 2),
        ("h170_last_angle_hits", i64 * N_H170_ANGLE_BINS * N_EVENT_TYPES * 2),
        ("h170_first_angle_hits", i64 * N_H170_ANGLE_BINS * 2),
    ]

    def as_dict(self) -> dict:
        import numpy as np
        return {name: np.ctypeslib.as_array(getattr(self, name)).copy() for name, _ in self._fields_}


TABLES_REFERENCE = 0  # CLR_TABLES_REFERENCE: the reference's order of operations (bit-identical tables)
TABLES_FAST = 1  # CLR_TABLES_FAST: FMA, two angles per Legendre recurrence (equal to rounding)

STAGE_NAMES = ("GEN", "ENTRY", "FLIGHT", "COND", "GEOM", "MORPH", "TOP", "BOTTOM", "SIDE", "ACRYL", "FIN")
ENGINE_DEFAULTS = {"flight_steps": 4, "tail_photons": 65536, "rare_batch": 8192, "pass_batch": 8, "acr_budget": 256}


class EngineConfig(C.Structure):
    """clr_engine_config: scheduling settings of the wavefront engine (zero = default)."""
    _fields_ = [("flight_steps", i32), ("tail_photons", i32), ("rare_batch", i32),
                ("stage_blocks", i32 * len(STAGE_NAMES)), ("pass_batch", i32), ("acr_budget", i32),
                ("reserved", i32 * 2)]

    @classmethod
    def from_dict(cls, d: dict | None) -> "EngineConfig":
        c = cls()
        for k, v in (d or {}).items():
            if k == "stage_blocks":
                for name, b in v.items():
                    c.stage_blocks[STAGE_NAMES.index(name)] = int(b)
            else:
                setattr(c, k, int(v))
        return c


class LightConfig(C.Structure):
    _fields_ = [("enabled", i32), ("nx", i32), ("ny", i32), ("nz", i32), ("max_rays", i32),
                ("representative_rays", i32), ("max_segments_per_ray", i32), ("heatmap_size", i32),
                ("zmax", f32), ("heat_zmax", f32)]


PF32 = C.POINTER(C.c_float)


class LightResult(C.Structure):
    _fields_ = [("track_length", PF32), ("post_scatter_track_length", PF32), ("scatter_event_weight", PF32),
                ("scatter_event_count", C.POINTER(C.c_uint32)), ("heatmap_xy", PF32), ("heatmap_zy", PF32),
                ("trajectory_x0", PF32), ("trajectory_y0", PF32), ("trajectory_z0", PF32),
                ("trajectory_x1", PF32), ("trajectory_y1", PF32), ("trajectory_z1", PF32),
                ("trajectory_order", PI32), ("trajectory_count", PI32), ("trajectory_overflow", PI32),
                ("segment_length_total", f64), ("deposited_length_total", f64),
                ("segment_count", i64), ("scatter_event_total", i64),
                ("error_count", i64), ("boundary_adjustment_count", i64), ("event_outside_count", i64),
                ("first_outside_xyz_tol", f32 * 4), ("first_outside_ray", u32), ("first_outside_set", u32)]

