"""Drop-in facade of the CLARITAS forward model on the GB300 library.

``ClaritasForwardModel(**kwargs)`` takes the reference constructor's keywords (CLARITAS/CLARITAS.py
:5577-5652) with the same defaults and validation (``scene.ModelConfig``); ``simulate`` keeps the
reference's signature (:7160-7179) and returns a ``ForwardResult`` with the reference's fields
(:5343-5515), computed from the library's tallies with the reference's formulas (:8882-8966,
:9600-9890). The photons of a call run in the reference's statistics batches
(``statistics_batch_rays`` rays each, global ray ids from ``ray_id_start``), traced together through
``clr_trace_batch``; the per-batch tallies give the batch-jackknife standard errors (:5244) and the
adaptive stopping rule (:8818-8880) exactly as the reference's batch loop does.

Two random streams are offered: ``rng="philox"`` (default; the fast production path) and
``rng="reference"`` (the reference's per-ray xorshift streams and seeds: per-ray outcomes equal the
reference kernels'). Features outside the photon-transport path raise ``NotImplementedError``:
population aggregation/fragmentation. Light-history diagnostics and heat maps run on the device (scatter-event
sites are the accepted particle collisions; absorption sites are not recorded). Named materials (the reference's
loess/kaolin PSD
tables) are not bundled: pass a ``scene.Particles`` as ``material`` or register one under a name.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np

from . import abi, materials as M, scene as S

DETECTOR_ANGLES_DEG = S.DETECTOR_ANGLES_DEG

# production failure codes and their names (the reference's table, CLARITAS/CLARITAS.py:424-444),
# kept identical so that failure dictionaries compare key by key
PRODUCTION_FAILURE_NAMES = {
    0: "PROD_OK", 1: "PARTICLE_MICROSURFACE_NUMERICAL", 2: "PARTICLE_MICROSURFACE_WATCHDOG",
    3: "PARTICLE_MACRO_GEOMETRY_FAILURE", 4: "PARTICLE_MACRO_BOUNCE_LIMIT", 5: "ACRYLIC_ANNULUS_NO_INTERSECTION",
    6: "ACRYLIC_ANNULUS_BOUNCE_LIMIT", 7: "BOTTOM_DISC_GEOMETRY_FAILURE", 8: "BOTTOM_DISC_BOUNCE_LIMIT",
    9: "WATER_BOUNDARY_NO_INTERSECTION", 10: "TRACE_ITERATION_LIMIT", 11: "NONFINITE_POSITION",
    12: "NONFINITE_DIRECTION", 13: "INVALID_MEDIUM_STATE", 14: "INVALID_EVENT_STATE", 15: "OTHER_EXPLICIT_FAILURE",
    16: "SPHEROID_GEOMETRY_FAILURE", 17: "HEADSPACE_BOUNDARY_NO_INTERSECTION", 18: "SPATIAL_MAJORANT_VIOLATION",
}
WATCHDOG_CODES = frozenset((2, 4, 6, 8, 10))           # :461
GEOMETRY_FAILURE_CODES = frozenset((3, 5, 7, 9, 13, 16, 17))  # :462
NONFINITE_CODES = frozenset((11, 12))                 # :463
SFH213_HALF_ANGLE_DEG = 10.0
SFH213_FIT_EXPONENT = 3.169925001442312

# status codes of a finished history (trace_kernel :5070-5103)
ST_AIR, ST_AXIAL, ST_SOURCE_REJECT, ST_FAILURE, ST_ABSORBED, ST_TOP, ST_BOTTOM, ST_TRAPPED = 1, 2, 3, 4, 5, 6, 7, 8


def jackknife_normalized_se(batch_scores) -> np.ndarray:
    """Batch-jackknife standard error of the normalized 18-channel response (CLARITAS.py:5244-5262)."""
    if len(batch_scores) < 3:
        return np.full(DETECTOR_ANGLES_DEG.size, np.nan)
    s = np.asarray(batch_scores, dtype=float)
    total = s.sum(axis=0)
    loo = [(total - row) / (total - row).sum() for row in s if (total - row).sum() > 0]
    if len(loo) < 3:
        return np.full(DETECTOR_ANGLES_DEG.size, np.nan)
    loo = np.asarray(loo)
    b = loo.shape[0]
    return np.sqrt((b - 1.0) / b * np.sum((loo - loo.mean(axis=0)) ** 2, axis=0))


def histogram_median(hist) -> float:
    """Median of an integer histogram (CLARITAS.py:5231-5241)."""
    hist = np.asarray(hist, dtype=np.int64)
    n = int(hist.sum())
    if n <= 0:
        return float("nan")
    cs = np.cumsum(hist)
    if n % 2:
        return float(np.searchsorted(cs, n // 2 + 1))
    return 0.5 * (int(np.searchsorted(cs, n // 2)) + int(np.searchsorted(cs, n // 2 + 1)))


def _norm(v: np.ndarray) -> np.ndarray:
    s = float(np.sum(v))
    return np.asarray(v, dtype=float) / s if s > 0 else np.zeros(DETECTOR_ANGLES_DEG.size)


def _div(a, b, fill=0.0):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return np.divide(a, b, out=np.full(a.shape, fill, dtype=float), where=b > 0)


@dataclass
class ForwardResult:
    """The reference's result record (CLARITAS.py:5343-5515), field for field."""
    detector_angles_deg: np.ndarray
    raw_hits: np.ndarray
    normalized_response: np.ndarray
    native_exact_hits: np.ndarray
    mirror_exact_hits: np.ndarray
    symmetry_exact_scores: np.ndarray
    normalized_native_exact_response: np.ndarray
    normalized_mirror_exact_response: np.ndarray
    normalized_symmetry_exact_response: np.ndarray
    normalized_response_jackknife_se: np.ndarray
    hardware_native_hits: np.ndarray
    hardware_mirror_hits: np.ndarray
    hardware_symmetry_scores: np.ndarray
    normalized_hardware_native_response: np.ndarray
    normalized_hardware_mirror_response: np.ndarray
    normalized_hardware_symmetry_response: np.ndarray
    hardware_normalized_jackknife_se: np.ndarray
    legacy_native_channel_counts: np.ndarray
    legacy_mirror_channel_counts: np.ndarray
    legacy_symmetry_channel_scores: np.ndarray
    normalized_legacy_native_response: np.ndarray
    normalized_legacy_mirror_response: np.ndarray
    normalized_legacy_symmetry_response: np.ndarray
    legacy_normalized_jackknife_se: np.ndarray
    legacy_acceptance_deg: float
    valid_exit_count: int
    numerical_failure_count: int
    numerical_failure_fraction: float
    production_failure_count: int
    production_failure_code_counts: dict
    production_failure_subcode_counts: dict
    production_watchdog_count: int
    production_geometry_failure_count: int
    production_nonfinite_count: int
    production_failure_diagnostics: dict
    n_rays: int
    requested_n_rays: int
    stopped_adaptively: bool
    stop_reason: str
    particle_event_model: str
    particle_surface_rms_slope_deg: float
    particle_surface_beckmann_alpha: float
    wave_surface_rms_height_nm: float
    wave_spheroid_aspect_ratio: float
    wave_spheroid_orientation_model: str
    wave_spheroid_orientation_kappa: float
    aggregation_model: str
    aggregation_collision_exposure: float
    aggregation_number_reduction_fraction: float
    aggregation_mass_conservation_error: float
    aggregation_projected_area_ratio: float
    aggregation_largest_bin_mass_fraction: float
    aggregation_overflow_event_fraction: float
    aggregation_steps: int
    population_number_reduction_fraction: float
    fragmentation_breakup_exposure: float
    fragmentation_reference_diameter_m: float
    fragmentation_size_exponent: float
    fragmentation_underflow_event_fraction: float
    aggregation_events_per_initial_particle: float
    fragmentation_events_per_initial_particle: float
    wave_coherent_fraction_nominal_cuda: float
    mean_coherent_wave_interactions: float
    mean_morphology_wave_interactions: float
    morphology_fraction_of_wave_interactions: float
    mu_geom_per_m: float
    mu_wave_per_m: float
    mu_event_per_m: float
    mu_sca_per_m: float
    mu_ext_per_m: float
    geometric_optical_depth_diameter: float
    optical_depth_diameter: float
    mean_interactions: float
    mean_geometric_interactions: float
    mean_wave_interactions: float
    median_interactions: float
    ballistic_fraction: float
    mean_fresnel_reflections: float
    entry_reflection_fraction: float
    internal_reflection_fraction: float
    particle_absorption_fraction: float
    particle_absorbed_ray_count: int
    mean_cell_inner_reflections: float
    mean_cell_outer_reflections: float
    cell_tir_fraction: float
    mean_top_surface_reflections: float
    top_surface_tir_fraction: float
    mean_top_surface_interactions: float
    free_surface_model: str
    vortex_wall_center_height_difference_mm: float
    vortex_core_radius_mm: float
    vortex_asymptotic_height_parameter_mm: float
    vortex_area_mean_uncorrected_rise_mm: float
    vortex_equivalent_core_rpm: float
    vortex_equivalent_rigid_body_rpm: float
    vortex_center_surface_z_mm: float
    vortex_wall_surface_z_mm: float
    sediment_transport_model: str
    sediment_eddy_diffusivity_m2_s: float
    sediment_majorant_geom_per_m: float
    sediment_majorant_wave_per_m: float
    sediment_majorant_total_per_m: float
    sediment_max_bin_density_scale: float
    meridional_circulation_ratio: float
    meridional_peak_speed_m_s: float
    meridional_grid_nr: int
    meridional_grid_nz: int
    meridional_solver_iterations: int
    meridional_solver_max_residual: float
    mean_bottom_inner_reflections: float
    mean_bottom_outer_reflections: float
    bottom_tir_fraction: float
    top_exit_fraction: float
    bottom_exit_fraction: float
    source_bore_surface_model: str
    detector_bore_surface_model: str
    bore_refractive_index: float
    ring_inner_face_surface_model: str
    ring_inner_face_refractive_index: float
    max_ring_face_bounces: int
    source_collimator_acceptance_fraction: float
    source_direct_acceptance_fraction: float
    source_reflected_acceptance_fraction: float
    source_bore_interactions_per_ray: float
    source_bore_reflections_per_ray: float
    hardware_native_direct_hits: np.ndarray
    hardware_mirror_direct_hits: np.ndarray
    hardware_symmetry_direct_scores: np.ndarray
    hardware_native_stray_hits: np.ndarray
    hardware_mirror_stray_hits: np.ndarray
    hardware_symmetry_stray_scores: np.ndarray
    detector_stray_fraction_by_channel: np.ndarray
    detector_stray_detection_fraction: float
    hardware_native_ring_face_stray_hits: np.ndarray
    hardware_mirror_ring_face_stray_hits: np.ndarray
    hardware_symmetry_ring_face_stray_scores: np.ndarray
    detector_ring_face_stray_fraction_by_channel: np.ndarray
    detector_ring_face_stray_detection_fraction: float
    photodiode_response_model: str
    sfh213_half_angle_deg: float
    sfh213_directional_fit_exponent: float
    photodiode_native_weighted_scores: np.ndarray
    photodiode_mirror_weighted_scores: np.ndarray
    photodiode_symmetry_weighted_scores: np.ndarray
    normalized_photodiode_native_response: np.ndarray
    normalized_photodiode_mirror_response: np.ndarray
    normalized_photodiode_symmetry_response: np.ndarray
    photodiode_relative_response_by_channel: np.ndarray
    detector_mean_incidence_angle_deg_by_channel: np.ndarray
    hardware_candidate_detection_fraction: float
    entered_water_fraction: float
    air_exit_fraction: float
    axial_loss_fraction: float
    detector_detection_fraction: float
    native_detector_detection_fraction: float
    mirror_detector_detection_fraction: float
    legacy_channel_score_per_ray: float
    symmetry_variance_reduction: bool
    batch_diagnostics: Optional[list] = None
    particle_diagnostics: Optional[Dict[str, np.ndarray]] = None
    detector_particle_path_diagnostics: Optional[Dict[str, np.ndarray]] = None
    ray_data: Optional[Dict[str, np.ndarray]] = None
    heatmap_xy: Optional[np.ndarray] = None
    heatmap_zy: Optional[np.ndarray] = None
    light_transport_diagnostics: Optional[dict] = None

    def to_dict(self) -> dict:
        d = dataclasses.asdict(self)
        for k, v in list(d.items()):
            if isinstance(v, np.ndarray):
                d[k] = v.tolist()
            elif isinstance(v, np.generic):
                d[k] = v.item()
        return d


class ClaritasForwardModel:
    """The reference's forward-model object over the GB300 library (one context per model)."""

    def __init__(self, rng: str = "philox", device: int = 0, **kwargs):
        self.config = S.ModelConfig(**kwargs)
        self.config.validate()
        if rng not in ("philox", "reference"):
            raise ValueError("rng must be 'philox' or 'reference'")
        self.rng_mode = abi.RNG_PHILOX if rng == "philox" else abi.RNG_REFERENCE_XORSHIFT
        self.device = int(device)
        self._ctx = None
        self._materials: dict = {}
        self._prepared_key = None
        self._physics = None
        for f in dataclasses.fields(self.config):  # the reference exposes its keywords as attributes
            setattr(self, f.name, getattr(self.config, f.name))

    # ---- materials and particle physics -------------------------------------------------------
    def register_material(self, name: str, particles: S.Particles) -> None:
        """Name a particle population (diameters, weights, n, k) for ``simulate(material=name, ...)``."""
        if not isinstance(particles, S.Particles):
            raise TypeError("particles must be a scene.Particles")
        self._materials[str(name)] = particles

    def _particles(self, material, concentration_g_per_L, weights, weight_mode) -> S.Particles:
        if isinstance(material, S.Particles):
            base = material
        elif material in self._materials:
            base = self._materials[material]
        else:
            # the reference's named materials: raw PSD weights and per-bin n/k, with the constructor's
            # optical-constants override, at the constructor's particle density (:6036-6052)
            d, w_raw = M.get_material_psd_raw(material)
            n, k = M.get_material_optical_constants(material, self.config.particle_optical_constants_by_material,
                                                    self.config.n_particle)
            base = S.Particles(d, w_raw, n, k, 0.0, float(self.config.density_kg_per_m3))
            if weights is not None and np.asarray(weights).shape != d.shape:
                raise ValueError(f"{material} requires {d.size} PSD weights")
        c = float(concentration_g_per_L)
        if not math.isfinite(c) or c < 0.0:
            raise ValueError("concentration must be finite and >=0")
        w = base.weight if weights is None else np.asarray(weights, dtype=np.float64)
        if w.shape != base.weight.shape:
            raise ValueError(f"weights must have {base.weight.size} entries (the material's diameter grid)")
        return S.Particles(base.diameter_m, w, base.n_real, base.k_imag, c, base.density_kg_m3, weight_mode)

    def _context(self):
        if self._ctx is None:
            from . import lib
            self._ctx = lib.Context(self.device)
            self._ctx.set_scene(self.config.to_scene_params())
        return self._ctx

    def _prepare(self, material, concentration_g_per_L, weights=None, weight_mode="mass_fraction"):
        parts = self._particles(material, concentration_g_per_L, weights, weight_mode)
        key = (id(material) if not isinstance(material, str) else material, float(concentration_g_per_L),
               None if weights is None else tuple(np.asarray(weights, dtype=float)), weight_mode)
        ctx = self._context()
        if key != self._prepared_key:
            # sediment model 3 without a supplied field: the library solves the meridional field on the device
            ss = self.config.sediment_spec()
            ctx.build_particles(parts.spec(self.config), ss)
            self._prepared_key = key
            self._physics = ctx.physics()
            self._meridional = {"peak_speed": float(ss.meridional_peak_speed), "nr": 2, "nz": 2, "iterations": 0,
                                "max_residual": 0.0}
            if self.config.sediment_transport_model == "schiller_naumann_meridional_advection_diffusion":
                f = ctx.sediment_field()
                self._meridional.update(nr=f["nr"], nz=f["nz"], iterations=f["iterations"],
                                        max_residual=f["max_residual"])
        return parts

    # the reference's diagnostic host keys (CLARITAS.py:6726-6767) that the library's tables provide
    _HOST_KEYS = {"size_parameter": "size_parameter", "qext": "qext", "qsca": "qsca", "qabs": "qabs",
                  "qback": "qback", "asymmetry_g": "asym_g", "single_scattering_albedo": "albedo",
                  "radius_m": "radius", "number_density_by_bin": "number_density", "mu_geom_by_bin": "mu_geom_bin",
                  "mu_sca_by_bin": "mu_sca_bin", "mu_ext_by_bin": "mu_ext_bin", "mu_wave_by_bin": "mu_wave_bin",
                  "mu_event_by_bin": "mu_event_bin"}
    # and its device tables (:6931-6965), here host copies
    _DEVICE_KEYS = {"radius": "radius", "gcdf": "geometric_cdf", "wcdf": "wave_cdf", "phase_cdf": "phase_cdf",
                    "theta": "theta", "qsca": "qsca", "qext": "qext", "mu_channels": "mu_scalars",
                    "trace_geom_bin": "trace_geom_bin", "trace_wave_bin": "trace_wave_bin",
                    "sed_majorants": "sed_majorants"}

    def _prepare_gpu_particle_physics(self, material, concentration_g_per_L, weights=None,
                                      weight_mode="mass_fraction") -> dict:
        """The reference's physics preparation (CLARITAS.py:6036-6965) and its return value (:6931-6965):
        the population's per-bin arrays (``d``, ``w``, ``nidx``, ``kidx``), ``n``, ``ntheta``, the tables
        under the reference's ``device`` keys (host copies: this library keeps its device tables inside the
        context) and the diagnostics under its ``host`` keys, as far as the library computes them (the
        population-balance and per-point sediment diagnostics are not part of it)."""
        parts = self._prepare(material, concentration_g_per_L, weights, weight_mode)
        ph = self._physics
        n = int(parts.diameter_m.size)
        device = {ref: np.asarray(ph[mine]).copy() for ref, mine in self._DEVICE_KEYS.items()}
        device["phase_cdf"] = device["phase_cdf"].reshape(n, -1)
        device["n"], device["k"] = parts.n_real.copy(), parts.k_imag.copy()
        if self.config.sediment_transport_model == "schiller_naumann_meridional_advection_diffusion":
            f = self._context().sediment_field()
            device.update(sed_grid=f["grid"], sed_grid_nr=int(f["nr"]), sed_grid_nz=int(f["nz"]),
                          sed_grid_zmax=float(self.config.sediment_spec().grid_zmax))
        host = {ref: np.asarray(ph[mine]).copy() for ref, mine in self._HOST_KEYS.items()}
        sg = math.pi * host["radius_m"] ** 2
        host.update(diameter_m=parts.diameter_m.copy(), n_real=parts.n_real.copy(), k_imag=parts.k_imag.copy(),
                    geometric_cross_section_m2=sg, scattering_cross_section_m2=host["qsca"] * sg,
                    extinction_cross_section_m2=host["qext"] * sg)
        theta, cdf = device["theta"], device["phase_cdf"]
        for lo, hi in ((165.0, 175.0), (169.0, 171.0)):  # near-backscatter band probabilities (:6780-6799)
            key = f"mie_phase_probability_{int(lo)}_{int(hi)}_by_bin"
            if self.config.particle_event_model == "hybrid_mie_excess" and theta.size > 2:
                at = lambda deg: np.array([np.interp(math.radians(deg), theta, row) for row in cdf])  # noqa: E731
                host[key] = np.maximum(at(hi) - at(lo), 0.0)
            else:
                host[key] = np.zeros(n)
        if self.config.sediment_transport_model == "schiller_naumann_meridional_advection_diffusion":
            host.update(meridional_solver_iterations=int(self._meridional["iterations"]),
                        meridional_solver_max_residual=float(self._meridional["max_residual"]),
                        meridional_solver_tolerance=float(self.config.meridional_solver_tolerance))
        return dict(d=parts.diameter_m.copy(), w=parts.weight.copy(), nidx=parts.n_real.copy(),
                    kidx=parts.k_imag.copy(), n=n, device=device, host=host, ntheta=int(theta.size))

    def phase_table_diagnostics(self, material, concentration_g_per_L, weights=None, weight_mode="mass_fraction"):
        """(theta [n_theta], cdf [n_bins, n_theta]) of the Mie phase tables (CLARITAS.py:7146)."""
        self._prepare(material, concentration_g_per_L, weights, weight_mode)
        return self._physics["theta"].copy(), self._physics["phase_cdf"].copy()

    # ---- the forward simulation ---------------------------------------------------------------
    def simulate(self, material, concentration_g_per_L, weights=None, n_rays=100000, seed=12345,
                 weight_mode="mass_fraction", collect_rays=False, heatmap_size=0, light_transport_config=None,
                 target_detector_score=None, min_rays=None, max_rays=None, min_rear_channel_score=None,
                 min_h170_score=None, stability_l1_tolerance=None, stability_window=3,
                 ray_id_start=0, path_provenance=True) -> ForwardResult:
        """The reference's simulate (CLARITAS.py:7160-7179). path_provenance (not a reference keyword): count
        the particle-event provenance partitions of the path diagnostics (first/last bin, event type and
        deflection, acrylic returns), which the reference always derives; off saves their device work."""
        light = self._light_setup(light_transport_config, heatmap_size)
        if collect_rays:
            raise NotImplementedError("collect_rays: use lib.Context.trace(run, records=True) for per-ray records")
        cfg = self.config
        requested = int(n_rays)
        ray_id_start = int(ray_id_start)
        if ray_id_start < 0 or ray_id_start + requested > 2 ** 32:
            raise ValueError("ray_id_start range exceeds uint32 global IDs")
        adaptive = target_detector_score is not None
        target = rear_target = h170_target = None
        if adaptive:  # request sizing of CLARITAS.py:7193-7219
            target = float(target_detector_score)
            if target <= 0:
                raise ValueError("target_detector_score must be >0")
            rear_target = None if min_rear_channel_score is None else float(min_rear_channel_score)
            h170_target = None if min_h170_score is None else float(min_h170_score)
            if rear_target is not None and rear_target <= 0:
                raise ValueError("min_rear_channel_score must be >0")
            if h170_target is not None and h170_target <= 0:
                raise ValueError("min_h170_score must be >0")
            max_n = int(max_rays if max_rays is not None else max(requested, cfg.statistics_batch_rays))
            min_n = int(min_rays if min_rays is not None else min(cfg.statistics_batch_rays, max_n))
            if min_n < 0 or max_n < min_n:
                raise ValueError("invalid min_rays/max_rays")
        else:
            max_n = min_n = requested
        if max_n < 1:
            raise ValueError("number of rays must be positive")
        self._prepare(material, concentration_g_per_L, weights, weight_mode)
        ctx = self._context()
        prov = bool(path_provenance)
        ctx.set_provenance(prov)
        try:
            batch = int(cfg.statistics_batch_rays)
            sizes = []
            left = max_n
            while left > 0:
                sizes.append(min(batch, left))
                left -= sizes[-1]
            # Batches are traced in groups through one clr_trace_batch call; a fixed-count run is one group.
            group = len(sizes) if not adaptive else max(1, min(len(sizes), 64))
            if adaptive and (light is not None or prov):
                group = 1  # diagnostics accumulate over traced batches: trace no batch past the stopping one
            tallies = []
            prov_parts = []
            stop_at = None
            state = _StopState()
            start = 0
            while start < len(sizes) and stop_at is None:
                runs = []
                off = ray_id_start + sum(sizes[:start])
                for k in range(start, min(start + group, len(sizes))):
                    runs.append(S.run_params(sizes[k], seed=seed, ray_offset=off, rng_mode=self.rng_mode))
                    off += sizes[k]
                got = ctx.trace_batch(runs)
                if prov:
                    prov_parts.append(ctx.read_provenance())
                for t in got:
                    tallies.append(t)
                    if adaptive and state.after_batch(self, t, min_n, target, rear_target, h170_target,
                                                      stability_l1_tolerance, stability_window):
                        stop_at = len(tallies)
                        break
                start += group
            if stop_at is not None:
                tallies = tallies[:stop_at]
                stop_reason = state.reason
            else:
                stop_reason = state.final_reason(adaptive, target, rear_target, h170_target, stability_l1_tolerance)
        finally:
            ctx.set_provenance(False)
        prov_total = None
        if prov_parts:
            prov_total = {k: np.sum([q[k] for q in prov_parts], axis=0) for k in prov_parts[0]}
        res = self._result(tallies, requested, adaptive, max_n, stop_reason, prov_total)
        if light is not None:
            res.heatmap_xy, res.heatmap_zy, res.light_transport_diagnostics = self._light_results(
                light, ray_id_start, res.n_rays)
        return res

    # ---- light-history diagnostics and heat maps (simulate's light_transport_config / heatmap_size,
    # CLARITAS.py:7229-7300 and :9453-9580) ------------------------------------------------------------
    def _light_setup(self, light_transport_config, heatmap_size):
        vis = int(heatmap_size)
        if vis < 0:
            raise ValueError("heatmap_size must be >= 0")
        ldc = dict(light_transport_config or {})
        enabled = bool(ldc.get("enabled", False))
        if not enabled and vis == 0:
            prev = getattr(self._ctx, "_light", None) if self._ctx is not None else None
            if prev is not None and (prev.enabled or prev.heatmap_size):
                self._ctx.set_light()
            return None
        max_rays = int(ldc.get("max_rays", 0)) if enabled else 0
        nx, ny, nz = ((int(ldc.get("nx", 1)), int(ldc.get("ny", 1)), int(ldc.get("nz", 1))) if enabled
                      else (1, 1, 1))
        rep = min(int(ldc.get("representative_rays", 0)), max_rays) if enabled else 0
        max_seg = int(ldc.get("max_segments_per_ray", 0)) if enabled else 0
        if enabled:
            if max_rays < 1:
                raise ValueError("light diagnostic max_rays must be >=1")
            if min(nx, ny, nz) < 4:
                raise ValueError("light diagnostic grid dimensions must each be >=4")
            if rep < 0 or max_seg < 1:
                raise ValueError("invalid representative-ray diagnostic configuration")
        cfg = self.config
        vg = S.vortex_surface_geometry(cfg.free_surface_model, cfg.zmean, cfg.tube_inner_radius_m,
                                       cfg.vortex_wall_center_height_difference_m, cfg.vortex_core_radius_m,
                                       cfg.gravity_m_s2)
        zmax = max(float(vg["center_z"]), float(vg["wall_z"])) if enabled else cfg.zmean
        voxels = nx * ny * nz if enabled else 1
        nbytes = voxels * 20 + max(rep * max_seg, 1) * 32 + max(rep, 1) * 8 + 8
        if enabled and nbytes > 1_000_000_000:
            raise ValueError(f"light diagnostic allocation is too large ({nbytes / 1e9:.3g} GB); reduce grid "
                             "dimensions, representative rays, or segments per ray")
        self._context().set_light(enabled, nx, ny, nz, max_rays, rep, max_seg, vis, zmax, float(vg["wall_z"]))
        return {"enabled": enabled, "vis": vis, "nx": nx, "ny": ny, "nz": nz, "max_rays": max_rays, "rep": rep,
                "max_seg": max_seg, "zmax": zmax, "bytes": nbytes, "t0": __import__("time").perf_counter()}

    def _light_results(self, light, ray_id_start: int, total_rays: int):
        import time
        a = self._context().read_light()
        hm = (a["heatmap_xy"], a["heatmap_zy"]) if light["vis"] > 0 else (None, None)
        if not light["enabled"]:
            return hm[0], hm[1], None
        cfg = self.config
        total, post, ew = a["track_length"], a["post_scatter_track_length"], a["scatter_event_weight"]
        ec = a["scatter_event_count"]
        seg, dep = float(a["segment_length_total"]), float(a["deposited_length_total"])
        ev_grid = int(np.sum(ec, dtype=np.uint64))
        outside = None
        if a["first_outside_set"]:
            x, y, z, tol = a["first_outside_xyz_tol"]
            outside = {"global_ray_id": int(a["first_outside_ray"]), "x_m": float(x), "y_m": float(y), "z_m": float(z),
                       "coordinate_tolerance_m": float(tol),
                       "x_bounds_m": [-cfg.tube_inner_radius_m, cfg.tube_inner_radius_m],
                       "y_bounds_m": [-cfg.tube_inner_radius_m, cfg.tube_inner_radius_m],
                       "z_bounds_m": [cfg.zmin, light["zmax"]]}
        zeros = np.zeros_like(ec)
        diag = {
            "track_length_m": total, "post_scatter_track_length_m": post,
            "absorption_event_count": zeros, "absorption_event_total": 0, "deposited_absorption_event_total": 0,
            "absorption_event_closure_error": 0,
            "absorption_grid_basis": "accepted extinction encounter site; not recorded by this library",
            "scatter_event_weight": ew, "scatter_event_count": ec,
            "nx": light["nx"], "ny": light["ny"], "nz": light["nz"],
            "x_min_m": -cfg.tube_inner_radius_m, "x_max_m": cfg.tube_inner_radius_m,
            "y_min_m": -cfg.tube_inner_radius_m, "y_max_m": cfg.tube_inner_radius_m,
            "z_min_m": cfg.zmin, "z_max_m": light["zmax"],
            "diagnostic_ray_limit": light["max_rays"],
            "diagnostic_rays_processed": max(0, min(total_rays, light["max_rays"] - ray_id_start)),
            "representative_ray_limit": light["rep"], "max_segments_per_ray": light["max_seg"],
            "segment_count": int(a["segment_count"]), "scatter_event_total": int(a["scatter_event_total"]),
            "deposited_scatter_event_total": ev_grid,
            "scatter_event_closure_error": ev_grid - int(a["scatter_event_total"]),
            "error_count": int(a["error_count"]), "hard_error_count": int(a["error_count"]),
            "boundary_adjustment_count": int(a["boundary_adjustment_count"]),
            "event_outside_count": int(a["event_outside_count"]), "first_outside_event": outside,
            "nonfinite_count": sum(int(np.count_nonzero(~np.isfinite(v))) for v in (total, post, ew)),
            "negative_value_count": sum(int(np.count_nonzero(v < 0)) for v in (total, post, ew)),
            "diagnostic_memory_bytes": int(light["bytes"]),
            "diagnostic_active_wall_time_s": float(time.perf_counter() - light["t0"]),
            "segment_length_total_m": seg, "deposited_length_total_m": dep,
            "deposition_closure_relative_error": abs(dep - seg) / max(abs(seg), 1e-30),
            "grid_closure_relative_error": abs(float(np.sum(total, dtype=np.float64)) - seg) / max(abs(seg), 1e-30),
            "trajectory_count": a["trajectory_count"], "trajectory_overflow": a["trajectory_overflow"],
        }
        for k in ("x0", "y0", "z0", "x1", "y1", "z1"):
            diag[f"trajectory_{k}_m"] = a["trajectory_" + k]
        diag["trajectory_particle_order"] = a["trajectory_order"]
        # the event code of each kept segment's end is not recorded by this library: -1 throughout
        diag["trajectory_event_code"] = np.full(np.shape(a["trajectory_order"]), -1, dtype=np.int32)
        return hm[0], hm[1], diag

    # ---- result assembly (formulas of CLARITAS.py:8882-8966 and :9600-9890) --------------------
    def _batch_scores(self, t):
        cfg = self.config
        nat, mir = t["hw_native"].astype(float), t["hw_mirror"].astype(float)
        hw = 0.5 * (nat + mir) if cfg.symmetry_average_exact else nat
        pd = 0.5 * (t["photodiode_native"] + t["photodiode_mirror"]) if cfg.symmetry_average_exact \
            else t["photodiode_native"].copy()
        sel = hw if cfg.photodiode_response_model == "ideal_hard_aperture" else pd
        lnat, lmir = t["legacy_native"].astype(float), t["legacy_mirror"].astype(float)
        leg = 0.5 * (lnat + lmir) if cfg.symmetry_average_exact else lnat
        return sel, hw, pd, leg

    def _result(self, tallies, requested, adaptive, max_n, stop_reason, prov=None) -> ForwardResult:
        cfg = self.config
        sym = avg = cfg.symmetry_average_exact
        tot = {k: np.sum([np.asarray(t[k]) for t in tallies], axis=0) for k in tallies[0]
               if isinstance(tallies[0][k], np.ndarray)}
        n = int(sum(t["n_rays"] for t in tallies))
        scores = [self._batch_scores(t) for t in tallies]
        sym_total = np.sum([s[0] for s in scores], axis=0)
        legacy_sym_total = np.sum([s[3] for s in scores], axis=0)
        native, mirror = tot["hw_native"].astype(np.int64), tot["hw_mirror"].astype(np.int64)
        hw_sym = 0.5 * (native + mirror) if avg else native.astype(float)
        pd_nat, pd_mir = tot["photodiode_native"], tot["photodiode_mirror"]
        pd_sym = 0.5 * (pd_nat + pd_mir) if avg else pd_nat.copy()
        ideal = cfg.photodiode_response_model == "ideal_hard_aperture"

        def sym2(a, b):
            return 0.5 * (a.astype(float) + b.astype(float)) if avg else a.astype(float)

        direct_sym = sym2(tot["hw_native_direct"], tot["hw_mirror_direct"])
        stray_sym = sym2(tot["hw_native_stray"], tot["hw_mirror_stray"])
        face_sym = sym2(tot["hw_native_face"], tot["hw_mirror_face"])
        inc_sym = 0.5 * (tot["incidence_native_sum"] + tot["incidence_mirror_sum"]) if avg \
            else tot["incidence_native_sum"].copy()
        lnat, lmir = tot["legacy_native"].astype(np.int64), tot["legacy_mirror"].astype(np.int64)
        nrays = max(n, 1)
        fc = tot["failure_code_counts"].astype(np.int64)
        fail_total = int(fc[1:].sum())
        pf_counts = {PRODUCTION_FAILURE_NAMES.get(i, f"CODE_{i}"): int(v) for i, v in enumerate(fc) if i and v}
        sub = {}
        for i, v in enumerate(tot["failure_subcode_counts"]):
            if v:
                sub[str(abi.subcode_of_index(i))] = int(v)
        es = dict(zip(abi.ES_NAMES, tot["entered_sums"][:len(abi.ES_NAMES)].astype(float)))
        rf = dict(zip(abi.RF_NAMES, tot["ray_flags"][:len(abi.RF_NAMES)].astype(np.int64)))
        st = tot["status_counts"].astype(np.int64)
        ev = dict(zip(abi.EV_NAMES, tot["event_counts"].astype(np.int64)))
        entered = int(rf["entered"])
        den = max(entered, 1)

        def per_entered(v):
            return float(v) / den if entered else float("nan")

        ph = self._physics
        mu = ph["mu_scalars"]  # trace geom, trace wave, geom, sca, ext, wave, event, coherent fraction (:6864-6868)
        vg = S.vortex_surface_geometry(cfg.free_surface_model, cfg.zmean, cfg.tube_inner_radius_m,
                                       cfg.vortex_wall_center_height_difference_m, cfg.vortex_core_radius_m,
                                       cfg.gravity_m_s2)
        ns = _norm(sym_total)
        nn, nm, nh = _norm(native), _norm(mirror), _norm(hw_sym)
        rows = []
        cum = np.zeros(18)
        cum_leg = 0.0
        total_rays = 0
        prev = None
        for t, (sel, hw, pd, leg) in zip(tallies, scores):
            total_rays += int(t["n_rays"])
            cum = cum + sel
            cum_leg += float(leg.sum())
            c = _norm(cum)
            l1 = float(np.sum(np.abs(c - prev))) if prev is not None else float("nan")
            prev = c
            rows.append({"batch": len(rows) + 1, "batch_rays": int(t["n_rays"]), "cumulative_rays": total_rays,
                         "batch_native_hits": int(t["hw_native"].sum()), "batch_mirror_hits": int(t["hw_mirror"].sum()),
                         "batch_hardware_candidate_score": float(hw.sum()),
                         "batch_photodiode_weighted_score": float(pd.sum()), "batch_selected_score": float(sel.sum()),
                         "cumulative_selected_score": float(cum.sum()), "cumulative_H150_score": float(cum[15]),
                         "cumulative_H160_score": float(cum[16]), "cumulative_H170_score": float(cum[17]),
                         "cumulative_min_rear_score_H150_H170": float(np.min(cum[15:18])),
                         "batch_legacy_channel_score": float(leg.sum()), "cumulative_legacy_channel_score": cum_leg,
                         "cumulative_l1_change": l1})
        sed = ph["sed_majorants"]
        ag_zero = dict(aggregation_model="none", aggregation_collision_exposure=0.0,
                       aggregation_number_reduction_fraction=0.0, aggregation_mass_conservation_error=0.0,
                       aggregation_projected_area_ratio=1.0, aggregation_largest_bin_mass_fraction=0.0,
                       aggregation_overflow_event_fraction=0.0, aggregation_steps=0,
                       population_number_reduction_fraction=0.0, fragmentation_breakup_exposure=0.0,
                       fragmentation_reference_diameter_m=float("nan"), fragmentation_size_exponent=float("nan"),
                       fragmentation_underflow_event_fraction=0.0, aggregation_events_per_initial_particle=0.0,
                       fragmentation_events_per_initial_particle=0.0)
        return ForwardResult(
            detector_angles_deg=DETECTOR_ANGLES_DEG.copy(), raw_hits=native.copy(), normalized_response=ns,
            native_exact_hits=native.copy(), mirror_exact_hits=mirror.copy(), symmetry_exact_scores=sym_total.copy(),
            normalized_native_exact_response=nn, normalized_mirror_exact_response=nm,
            normalized_symmetry_exact_response=ns,
            normalized_response_jackknife_se=jackknife_normalized_se([s[0] for s in scores]),
            hardware_native_hits=native.copy(), hardware_mirror_hits=mirror.copy(), hardware_symmetry_scores=hw_sym,
            normalized_hardware_native_response=nn, normalized_hardware_mirror_response=nm,
            normalized_hardware_symmetry_response=nh,
            hardware_normalized_jackknife_se=jackknife_normalized_se([s[1] for s in scores]),
            legacy_native_channel_counts=lnat.copy(), legacy_mirror_channel_counts=lmir.copy(),
            legacy_symmetry_channel_scores=legacy_sym_total.copy(),
            normalized_legacy_native_response=_norm(lnat), normalized_legacy_mirror_response=_norm(lmir),
            normalized_legacy_symmetry_response=_norm(legacy_sym_total),
            legacy_normalized_jackknife_se=jackknife_normalized_se([s[3] for s in scores]),
            legacy_acceptance_deg=cfg.legacy_detector_acceptance_deg,
            valid_exit_count=int(rf["valid_air"]), numerical_failure_count=fail_total,
            numerical_failure_fraction=fail_total / nrays, production_failure_count=fail_total,
            production_failure_code_counts=pf_counts, production_failure_subcode_counts=sub,
            production_watchdog_count=int(sum(fc[i] for i in WATCHDOG_CODES if i < fc.size)),
            production_geometry_failure_count=int(sum(fc[i] for i in GEOMETRY_FAILURE_CODES if i < fc.size)),
            production_nonfinite_count=int(sum(fc[i] for i in NONFINITE_CODES if i < fc.size)),
            production_failure_diagnostics={"code_counts": pf_counts, "subcode_counts": sub,
                                            "count_closure_ok": int(fc[1:].sum()) == int(st[ST_FAILURE]),
                                            "acrylic_trapped_tir_count": int(st[ST_TRAPPED]),
                                            "acrylic_trapped_tir_fraction": float(st[ST_TRAPPED]) / nrays},
            n_rays=n, requested_n_rays=requested, stopped_adaptively=bool(adaptive and n < max_n),
            stop_reason=stop_reason, particle_event_model=cfg.particle_event_model,
            particle_surface_rms_slope_deg=cfg.particle_surface_rms_slope_deg,
            particle_surface_beckmann_alpha=cfg.rough_alpha,
            wave_surface_rms_height_nm=cfg.wave_surface_rms_height_m * 1e9,
            wave_spheroid_aspect_ratio=cfg.wave_spheroid_aspect_ratio,
            wave_spheroid_orientation_model=cfg.wave_spheroid_orientation_model,
            wave_spheroid_orientation_kappa=cfg.wave_spheroid_orientation_kappa,
            **ag_zero,
            wave_coherent_fraction_nominal_cuda=float(mu[7]),
            mean_coherent_wave_interactions=per_entered(es["wcoh"]),
            mean_morphology_wave_interactions=per_entered(es["wmorph"]),
            morphology_fraction_of_wave_interactions=float(es["wmorph"] / es["wic"]) if es["wic"] > 0 else 0.0,
            mu_geom_per_m=float(mu[2]), mu_wave_per_m=float(mu[5]), mu_event_per_m=float(mu[6]),
            mu_sca_per_m=float(mu[3]), mu_ext_per_m=float(mu[4]),
            geometric_optical_depth_diameter=float(mu[2]) * 2 * cfg.tube_inner_radius_m,
            optical_depth_diameter=float(mu[6]) * 2 * cfg.tube_inner_radius_m,
            mean_interactions=per_entered(es["ic"]), mean_geometric_interactions=per_entered(es["gic"]),
            mean_wave_interactions=per_entered(es["wic"]), median_interactions=histogram_median(tot["ic_hist"]),
            ballistic_fraction=per_entered(rf["ballistic"]), mean_fresnel_reflections=per_entered(es["pr"]),
            entry_reflection_fraction=per_entered(rf["entry_reflected"]),
            internal_reflection_fraction=per_entered(rf["internal_reflected"]),
            particle_absorption_fraction=per_entered(rf["absorbed"]), particle_absorbed_ray_count=int(rf["absorbed"]),
            mean_cell_inner_reflections=per_entered(es["cir"]), mean_cell_outer_reflections=per_entered(es["cor"]),
            cell_tir_fraction=per_entered(rf["cell_tir"]), mean_top_surface_reflections=per_entered(es["top"]),
            top_surface_tir_fraction=per_entered(rf["top_tir"]),
            mean_top_surface_interactions=per_entered(es["top"] + st[ST_TOP]),
            free_surface_model=cfg.free_surface_model,
            vortex_wall_center_height_difference_mm=cfg.vortex_wall_center_height_difference_m * 1e3,
            vortex_core_radius_mm=(cfg.vortex_core_radius_m * 1e3
                                   if cfg.free_surface_model == "localized_scully_vortex" else float("nan")),
            vortex_asymptotic_height_parameter_mm=vg["h_inf"] * 1e3,
            vortex_area_mean_uncorrected_rise_mm=vg["h_bar"] * 1e3,
            vortex_equivalent_core_rpm=vg["equivalent_core_rpm"],
            vortex_equivalent_rigid_body_rpm=vg["equivalent_rigid_body_rpm"],
            vortex_center_surface_z_mm=vg["center_z"] * 1e3, vortex_wall_surface_z_mm=vg["wall_z"] * 1e3,
            sediment_transport_model=cfg.sediment_transport_model,
            sediment_eddy_diffusivity_m2_s=cfg.sediment_eddy_diffusivity_m2_s,
            sediment_majorant_geom_per_m=float(sed[0]), sediment_majorant_wave_per_m=float(sed[1]),
            sediment_majorant_total_per_m=float(sed[2]), sediment_max_bin_density_scale=float("nan"),
            meridional_circulation_ratio=cfg.meridional_circulation_ratio,
            meridional_peak_speed_m_s=self._meridional["peak_speed"], meridional_grid_nr=self._meridional["nr"],
            meridional_grid_nz=self._meridional["nz"], meridional_solver_iterations=self._meridional["iterations"],
            meridional_solver_max_residual=self._meridional["max_residual"],
            mean_bottom_inner_reflections=per_entered(es["bir"]), mean_bottom_outer_reflections=per_entered(es["bor"]),
            bottom_tir_fraction=per_entered(rf["bottom_tir"]),
            top_exit_fraction=float(st[ST_TOP]) / nrays, bottom_exit_fraction=float(st[ST_BOTTOM]) / nrays,
            source_bore_surface_model=cfg.source_bore_surface_model,
            detector_bore_surface_model=cfg.detector_bore_surface_model,
            bore_refractive_index=cfg.bore_refractive_index,
            ring_inner_face_surface_model=cfg.ring_inner_face_surface_model,
            ring_inner_face_refractive_index=cfg.ring_inner_face_refractive_index,
            max_ring_face_bounces=cfg.max_ring_face_bounces,
            source_collimator_acceptance_fraction=float(rf["source_accepted"]) / nrays,
            source_direct_acceptance_fraction=float(rf["source_direct"]) / nrays,
            source_reflected_acceptance_fraction=float(rf["source_reflected"]) / nrays,
            source_bore_interactions_per_ray=float(ev["source_bore_interactions"]) / nrays,
            source_bore_reflections_per_ray=float(ev["source_bore_reflections"]) / nrays,
            hardware_native_direct_hits=tot["hw_native_direct"].astype(np.int64),
            hardware_mirror_direct_hits=tot["hw_mirror_direct"].astype(np.int64),
            hardware_symmetry_direct_scores=direct_sym,
            hardware_native_stray_hits=tot["hw_native_stray"].astype(np.int64),
            hardware_mirror_stray_hits=tot["hw_mirror_stray"].astype(np.int64),
            hardware_symmetry_stray_scores=stray_sym, detector_stray_fraction_by_channel=_div(stray_sym, hw_sym),
            detector_stray_detection_fraction=float(stray_sym.sum()) / nrays,
            hardware_native_ring_face_stray_hits=tot["hw_native_face"].astype(np.int64),
            hardware_mirror_ring_face_stray_hits=tot["hw_mirror_face"].astype(np.int64),
            hardware_symmetry_ring_face_stray_scores=face_sym,
            detector_ring_face_stray_fraction_by_channel=_div(face_sym, hw_sym),
            detector_ring_face_stray_detection_fraction=float(face_sym.sum()) / nrays,
            photodiode_response_model=cfg.photodiode_response_model, sfh213_half_angle_deg=SFH213_HALF_ANGLE_DEG,
            sfh213_directional_fit_exponent=SFH213_FIT_EXPONENT,
            photodiode_native_weighted_scores=pd_nat.copy(), photodiode_mirror_weighted_scores=pd_mir.copy(),
            photodiode_symmetry_weighted_scores=pd_sym.copy(),
            normalized_photodiode_native_response=_norm(pd_nat), normalized_photodiode_mirror_response=_norm(pd_mir),
            normalized_photodiode_symmetry_response=_norm(pd_sym),
            photodiode_relative_response_by_channel=_div(pd_sym, hw_sym),
            detector_mean_incidence_angle_deg_by_channel=_div(inc_sym, hw_sym, fill=float("nan")),
            hardware_candidate_detection_fraction=float(hw_sym.sum()) / nrays,
            entered_water_fraction=entered / nrays, air_exit_fraction=float(rf["valid_air"]) / nrays,
            axial_loss_fraction=float(st[ST_AXIAL]) / nrays,
            detector_detection_fraction=float(sym_total.sum()) / nrays,
            native_detector_detection_fraction=float(native.sum() if ideal else pd_nat.sum()) / nrays,
            mirror_detector_detection_fraction=float(mirror.sum() if ideal else pd_mir.sum()) / nrays,
            legacy_channel_score_per_ray=float(legacy_sym_total.sum()) / nrays,
            symmetry_variance_reduction=bool(sym), batch_diagnostics=rows, particle_diagnostics=dict(ph),
            detector_particle_path_diagnostics=self._path_diagnostics(tot, hw_sym, avg, prov))

    # The reference's detector particle-path diagnostics (simulate, CLARITAS.py:8019-8110 and :8972-9140) from
    # the device partitions of the detected rays; partitions that need per-ray provenance the device does not
    # keep (first/last bin, deflection angles, causal sequences) are not produced.
    _ORDER_LABELS = ["0", "1", "2", "3", "4", "5+"]
    _MEAN_KEYS = ["mean_particle_interactions_by_channel", "mean_geometric_interactions_by_channel",
                  "mean_wave_interactions_by_channel", "mean_coherent_wave_interactions_by_channel",
                  "mean_morphology_wave_interactions_by_channel", "mean_entry_reflections_by_channel",
                  "mean_internal_reflections_by_channel"]
    _CSTAT_NAMES = ["candidate_trials", "outcome_rejections", "inaccessible_trials", "accepted_geometric",
                    "accepted_coherent", "accepted_morphology", "accepted_absorptions", "accepted_scatterings",
                    "numerical_failures", "retry_exhaustions"]

    def _path_diagnostics(self, tot: dict, denp: np.ndarray, avg: bool, prov: Optional[dict] = None) -> dict:
        def sym(native, mirror):
            return 0.5 * (native + mirror) if avg else native.copy()
        oh = np.asarray(tot["order_hits"], dtype=np.float64)            # [side][order][channel]
        gh = np.asarray(tot["geometric_order_hits"], dtype=np.float64)  # [side][order][channel]
        ps = np.asarray(tot["path_sums"], dtype=np.float64)             # [sum][side][channel]
        order, gorder = sym(oh[0], oh[1]), sym(gh[0], gh[1])            # [6][18]
        sums = sym(ps[:, 0, :], ps[:, 1, :])                            # [7][18]
        denp = np.asarray(denp, dtype=np.float64)
        mh = np.asarray(tot["path_mask_hits"], dtype=np.float64)        # [side][mask][channel]
        ah = np.asarray(tot["acrylic_order_hits"], dtype=np.float64)    # [side][order][channel]
        masks, acr = sym(mh[0], mh[1]), sym(ah[0], ah[1])
        # event-history mask scores and their fractions of the hard-aperture score (:8968-8977)
        out = {"hardware_symmetry_scores": denp.copy()}
        path = {}
        for k, name in enumerate(abi.PATH_MASK_NAMES):
            path[name] = masks[k]
            out[name + "_scores"] = masks[k].copy()
            out[name + "_fraction"] = np.divide(masks[k], denp, out=np.zeros_like(denp), where=denp > 0)
        out["interaction_order_partition_closure_error_scores"] = path["any_particle"] - (
            path["single_interaction"] + path["interaction_order_2"] + path["interaction_order_3"]
            + path["interaction_order_4plus"])
        out["multiple_branch_partition_closure_error_scores"] = path["multiple_interaction"] - (
            path["mixed_geometric_wave"] + path["geometric_only_multiple"] + path["wave_only_multiple"])
        out["single_branch_partition_closure_error_scores"] = path["single_interaction"] - (
            path["single_external_entry_reflection_escape"] + path["single_internal_reflection_escape"]
            + path["single_surface_transmission_escape"] + path["single_coherent_wave_escape"])
        out["acrylic_reflection_order_labels"] = ["0", "1", "2", "3", "4+"]
        out["acrylic_reflection_order_scores"] = acr
        out["acrylic_reflection_order_partition_closure_error_scores"] = denp - acr.sum(axis=0)
        out.update({"exact_particle_order_labels": list(self._ORDER_LABELS), "exact_particle_order_scores": order,
               "exact_geometric_order_labels": list(self._ORDER_LABELS), "exact_geometric_order_scores": gorder,
               "exact_particle_order_partition_closure_error_scores": denp - order.sum(axis=0),
               "exact_geometric_order_partition_closure_error_scores": denp - gorder.sum(axis=0)})
        for k, key in enumerate(self._MEAN_KEYS):
            out[key] = np.divide(sums[k], denp, out=np.full(denp.shape, np.nan), where=denp > 0)
        cond = self.config.particle_event_model in ("hybrid_mie_exact_rate", "hybrid_mie_exact_rate_moment_constrained")
        out["conditional_sampler_counts"] = dict(zip(self._CSTAT_NAMES, [int(v) for v in tot["conditional_stats"]]))
        out["closure"] = ("Mie extinction and terminal outcomes; conditional finite-particle angular/path law"
                          if cond else self.config.particle_event_model + "; configured unconditional event law")
        out["conditional_max_trials"] = 16384
        if prov is not None:
            out.update(self._provenance_diagnostics(prov, denp, path["any_particle"], sym))
        return out

    def _provenance_diagnostics(self, pv: dict, denp: np.ndarray, any_particle: np.ndarray, sym) -> dict:
        """The reference's causal outputs of the path diagnostics (CLARITAS.py:9008-9091, :9135-9150)."""
        npart = int(np.asarray(self._physics["radius"]).size)

        def nan_div(a, b):
            return np.divide(a, b, out=np.full(np.shape(a), np.nan), where=b > 0)

        def frac(a):
            return np.divide(a, denp, out=np.zeros_like(a, dtype=np.float64), where=denp > 0)
        out = {}
        bh = np.asarray(pv["bin_hits"], dtype=np.float64)                 # [kind][side][bin][channel]
        for k, name in enumerate(abi.PROVENANCE_BIN_NAMES):
            out[name + "_scores"] = sym(bh[k, 0], bh[k, 1])[:npart]
        for name in ("first_particle_bin", "last_particle_bin"):
            out[name + "_partition_closure_error_scores"] = any_particle - out[name + "_scores"].sum(axis=0)
        ft = np.asarray(pv["first_type_hits"], dtype=np.float64)
        lt = np.asarray(pv["last_type_hits"], dtype=np.float64)
        las = np.asarray(pv["last_type_angle_sum"], dtype=np.float64)
        lac = np.asarray(pv["last_type_angle_count"], dtype=np.float64)
        first_all, last_all = np.zeros_like(denp), np.zeros_like(denp)
        for code, name in abi.PARTICLE_EVENT_TYPE_NAMES.items():
            last, first = sym(lt[0, code], lt[1, code]), sym(ft[0, code], ft[1, code])
            out[f"last_event_{name}_scores"], out[f"last_event_{name}_fraction"] = last, frac(last)
            out[f"first_event_{name}_scores"], out[f"first_event_{name}_fraction"] = first, frac(first)
            out[f"last_event_{name}_mean_deflection_deg_by_channel"] = nan_div(
                sym(las[0, code], las[1, code]), sym(lac[0, code], lac[1, code]))
            first_all, last_all = first_all + first, last_all + last
        for key, field in (("first_event_backscatter", "first_backscatter_hits"),
                           ("first_event_source_hemisphere", "first_source_hemisphere_hits")):
            a = np.asarray(pv[field], dtype=np.float64)
            out[key + "_scores"] = sym(a[0], a[1])
            out[key + "_fraction"] = frac(out[key + "_scores"])
        for which in ("first", "last"):
            a = np.asarray(pv[which + "_angle_sum"], dtype=np.float64)
            c = np.asarray(pv[which + "_angle_count"], dtype=np.float64)
            out[f"mean_{which}_particle_deflection_deg_by_channel"] = nan_div(sym(a[0], a[1]), sym(c[0], c[1]))
        out["causal_last_event_partition_closure_error_scores"] = any_particle - last_all
        out["causal_first_event_partition_closure_error_scores"] = any_particle - first_all
        out["H170_last_event_angle_bin_edges_deg"] = np.asarray([0.0, 30.0, 60.0, 90.0, 120.0, 150.0, 180.0001])
        h = np.asarray(pv["h170_last_angle_hits"], dtype=np.float64)
        out["H170_last_event_angle_histogram_scores_by_event_code"] = sym(h[0], h[1])
        h = np.asarray(pv["h170_first_angle_hits"], dtype=np.float64)
        out["H170_first_event_angle_histogram_scores"] = sym(h[0], h[1])
        w = np.asarray(pv["wall_hits"], dtype=np.float64)
        out["wall_path_scores"] = {name: sym(w[0, k], w[1, k]) for k, name in enumerate(abi.WALL_PATH_NAMES)}
        out["wall_path_partition_closure_error_scores"] = denp - sum(out["wall_path_scores"].values())
        a = np.asarray(pv["after_return_hits"], dtype=np.float64)
        out["particle_after_acrylic_return_scores"] = sym(a[0], a[1])
        return out

    def close(self):
        if self._ctx is not None:
            self._ctx.close()
            self._ctx = None


class _StopState:
    """The reference's adaptive stopping rule, evaluated after each statistics batch (CLARITAS.py:8818-8880)."""

    def __init__(self):
        self.sym = np.zeros(18)
        self.rays = 0
        self.prev = None
        self.recent = []
        self.reason = "fixed_n_rays"

    def after_batch(self, model, t, min_n, target, rear_target, h170_target, l1_tol, window) -> bool:
        sel = model._batch_scores(t)[0]
        self.sym = self.sym + sel
        self.rays += int(t["n_rays"])
        cum = _norm(self.sym)
        if self.prev is not None:
            self.recent.append(float(np.sum(np.abs(cum - self.prev))))
        self.prev = cum
        if self.rays >= min_n and self.sym.sum() >= target:
            rear_ok = rear_target is None or float(np.min(self.sym[15:18])) >= rear_target
            h170_ok = h170_target is None or float(self.sym[17]) >= h170_target
            stable = True
            if l1_tol is not None:
                w = max(1, int(window))
                stable = len(self.recent) >= w and all(q <= float(l1_tol) for q in self.recent[-w:])
            if rear_ok and h170_ok and stable:
                bits = ["target_detector_score"]
                if rear_target is not None:
                    bits.append("rear_channels")
                if h170_target is not None:
                    bits.append("H170")
                if l1_tol is not None:
                    bits.append("stability")
                self.reason = "_and_".join(bits)
                return True
        return False

    def final_reason(self, adaptive, target, rear_target, h170_target, l1_tol) -> str:
        if not adaptive:
            return "fixed_n_rays"
        if self.sym.sum() < target:
            return "max_rays_before_target"
        if rear_target is not None and float(np.min(self.sym[15:18])) < rear_target:
            return "max_rays_before_rear_channel_target"
        if h170_target is not None and float(self.sym[17]) < h170_target:
            return "max_rays_before_H170_target"
        if l1_tol is not None:
            return "max_rays_before_stability"
        return "max_rays"
