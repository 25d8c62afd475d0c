"""Scene, particle and run descriptions for the photon-transport path.

``ModelConfig`` holds the keyword arguments of the reference's
``ClaritasForwardModel.__init__`` (CLARITAS/CLARITAS.py:5577-5652) with the same
names and defaults, and derives the launch-time scalars exactly as that
constructor does (:5660-5760): z = 0 is the sensor plane, ``zmin =
-sensor_height``, ``zmean = water_height - sensor_height``, ``zwall_top =
tube_length - sensor_height``, ``throat_out = ring_out - counterbore_depth``,
``rough_alpha = tan(rms_slope)``. ``to_scene_params`` packs them into the
C ABI struct (include/claritas_gb.h).

The workload builders at the bottom describe the synthetic scenes the tests
and the benchmark use (no dataset is involved: the reference publishes none).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field, fields, replace
from typing import Optional

import numpy as np

from . import abi

EVENT_MODEL_CODES = {
    "geometric": 0, "mie_qsca": 1, "mie_qext": 2, "hybrid_mie_excess": 3,
    "hybrid_mie_exact_rate": 4, "hybrid_mie_exact_rate_moment_constrained": 5,
}
WEIGHT_MODE_CODES = {"mass_fraction": 0, "number_fraction": 1}
SOURCE_ANGULAR_MODEL_CODES = {"legacy_polar_pdf": 0, "beta_radiance_3d": 1, "thesis_planar_beta": 2}
BORE_SURFACE_MODEL_CODES = {"absorbing": 0, "smooth_fresnel_nylon": 1}
RING_FACE_SURFACE_MODEL_CODES = {"absorbing": 0, "smooth_fresnel_nylon": 1}
PHOTODIODE_RESPONSE_MODEL_CODES = {"ideal_hard_aperture": 0, "sfh213_datasheet_fit": 1}
SPHEROID_ORIENTATION_MODEL_CODES = {"isotropic": 0, "local_tangential_axial_vmf": 1}
# "rankine_vortex" is this library's (no reference counterpart): see rankine_surface_coefficients
FREE_SURFACE_MODEL_CODES = {"flat": 0, "parabolic_vortex": 1, "localized_scully_vortex": 2, "rankine_vortex": 3}
SEDIMENT_TRANSPORT_MODEL_CODES = {
    "uniform": 0, "stokes_drift_diffusion": 1, "schiller_naumann_drift_diffusion": 2,
    "schiller_naumann_meridional_advection_diffusion": 3,
}
CONDITIONAL_MAX_TRIALS = 16384  # CLARITAS/CLARITAS.py:1117
DEFAULT_PARTICLE_WAVELENGTH_M = 622e-9  # CLARITAS/CLARITAS.py:705
DETECTOR_ANGLES_DEG = np.arange(0, 180, 10, dtype=np.float64)


@dataclass
class ModelConfig:
    """ClaritasForwardModel keyword arguments (same names and defaults)."""
    n_water: float = 1.33
    n_particle: float = 1.59
    n_acrylic: float = 1.4906
    n_air: float = 1.0
    tube_inner_radius_m: float = 0.0465
    tube_outer_radius_m: float = 0.0500
    tube_length_m: float = 0.491
    water_height_m: float = 0.142
    sensor_height_above_bottom_m: float = 0.093
    sensor_ring_inner_radius_m: float = 0.0505
    sensor_ring_outer_radius_m: float = 0.0655
    counterbore_depth_m: float = 0.008
    through_bore_diameter_m: float = 0.004
    counterbore_diameter_m: float = 0.0087
    source_launch_radius_m: float = 0.0655
    legacy_detector_acceptance_deg: float = 6.5
    source_beam_sigma_m: float = 1.0e-5
    source_bore_surface_model: str = "absorbing"
    detector_bore_surface_model: str = "absorbing"
    bore_refractive_index: float = 1.53
    max_bore_bounces: int = 16
    ring_inner_face_surface_model: str = "absorbing"
    ring_inner_face_refractive_index: float = 1.53
    max_ring_face_bounces: int = 16
    photodiode_response_model: str = "ideal_hard_aperture"
    particle_wavelength_m: float = DEFAULT_PARTICLE_WAVELENGTH_M
    particle_optical_constants_by_material: Optional[dict] = None
    particle_event_model: str = "geometric"
    hybrid_wave_scale: float = 1.0
    mie_phase_grid_size: int = 2049
    moment_constraint_by_material: Optional[dict] = None
    particle_surface_rms_slope_deg: float = 25.0
    wave_surface_rms_height_m: float = 100e-9
    wave_spheroid_aspect_ratio: float = 1.5
    wave_spheroid_orientation_model: str = "isotropic"
    wave_spheroid_orientation_kappa: float = 0.0
    free_surface_model: str = "localized_scully_vortex"
    vortex_wall_center_height_difference_m: float = 0.050
    vortex_core_radius_m: float = 0.020
    sediment_transport_model: str = "schiller_naumann_drift_diffusion"
    sediment_eddy_diffusivity_m2_s: float = 1.0e-3
    water_density_kg_per_m3: float = 997.0
    water_dynamic_viscosity_pa_s: float = 8.9e-4
    gravity_m_s2: float = 9.81
    sediment_transport_quadrature_points: int = 4096
    sediment_radial_lookup_points: int = 2049
    meridional_circulation_ratio: float = 0.10
    meridional_grid_nr: int = 48
    meridional_grid_nz: int = 96
    meridional_solver_max_iterations: int = 8000
    meridional_solver_check_interval: int = 250
    meridional_solver_tolerance: float = 1.0e-6
    meridional_solver_sor: float = 1.75
    aggregation_model: str = "none"
    aggregation_collision_exposure: float = 0.0
    fragmentation_breakup_exposure: float = 0.0
    fragmentation_reference_diameter_m: float = 100e-6
    fragmentation_size_exponent: float = 1.0
    aggregation_step_safety: float = 0.2
    aggregation_max_steps: int = 200000
    alpha1: float = 0.45
    alpha2: float = 5.0
    source_angular_model: str = "beta_radiance_3d"
    density_kg_per_m3: float = 2600.0
    bottom_disc_thickness_m: float = 0.003
    bottom_external_refractive_index: float = 1.0
    max_axial_bounces: int = 64
    max_iterations: int = int(1e6)
    max_internal_bounces: int = 64
    max_cell_bounces: int = 64
    chunk_size: int = 250000
    statistics_batch_rays: int = 250000
    symmetry_average_exact: bool = True
    # new capabilities (no reference counterpart); defaults keep reference behaviour
    source_kind: str = "reference_led"
    disc_beam_radius_m: float = 1.0e-3
    water_absorption_per_m: float = 0.0

    # ---- derived quantities (CLARITAS/CLARITAS.py:5660-5700) ----
    @property
    def zmin(self) -> float:
        return -float(self.sensor_height_above_bottom_m)

    @property
    def zmean(self) -> float:
        return float(self.water_height_m) - float(self.sensor_height_above_bottom_m)

    @property
    def zwall_top(self) -> float:
        return float(self.tube_length_m) - float(self.sensor_height_above_bottom_m)

    @property
    def throat_out(self) -> float:
        return float(self.sensor_ring_outer_radius_m) - float(self.counterbore_depth_m)

    @property
    def rough_alpha(self) -> float:
        return float(np.tan(np.deg2rad(float(self.particle_surface_rms_slope_deg))))

    def validate(self) -> None:
        """Configuration checks of the reference constructor (CLARITAS/CLARITAS.py:5754-5999) on the hot path."""
        rin, rout = self.tube_inner_radius_m, self.tube_outer_radius_m
        ring_in, ring_out = self.sensor_ring_inner_radius_m, self.sensor_ring_outer_radius_m
        if not (0 < rin < rout < ring_in < self.throat_out <= self.source_launch_radius_m <= ring_out):
            raise ValueError("TARDIIS radial/source geometry is inconsistent")
        if not (self.tube_length_m > 0.0 and np.isfinite(self.tube_length_m)):
            raise ValueError("tube_length_m must be finite and positive")
        if not (self.zwall_top > self.zmean > self.zmin):
            raise ValueError("physical wall top must lie above the complete water/free-surface domain and bottom")
        for name, table in (
            ("photodiode_response_model", PHOTODIODE_RESPONSE_MODEL_CODES),
            ("particle_event_model", EVENT_MODEL_CODES),
            ("wave_spheroid_orientation_model", SPHEROID_ORIENTATION_MODEL_CODES),
            ("free_surface_model", FREE_SURFACE_MODEL_CODES),
            ("sediment_transport_model", SEDIMENT_TRANSPORT_MODEL_CODES),
            ("source_angular_model", SOURCE_ANGULAR_MODEL_CODES),
            ("source_bore_surface_model", BORE_SURFACE_MODEL_CODES),
            ("detector_bore_surface_model", BORE_SURFACE_MODEL_CODES),
            ("ring_inner_face_surface_model", RING_FACE_SURFACE_MODEL_CODES),
        ):
            if str(getattr(self, name)).strip().lower() not in table:
                raise ValueError(f"invalid {name} {getattr(self, name)!r}")
        if self.photodiode_response_model != "ideal_hard_aperture" and (
            self.detector_bore_surface_model != "absorbing" or self.ring_inner_face_surface_model != "absorbing"
        ):
            raise ValueError("SFH213 package-response audit requires absorbing detector bores and absorbing ring inner face")
        if not (0 < 0.5 * self.through_bore_diameter_m < 0.5 * self.counterbore_diameter_m):
            raise ValueError("through-bore must be narrower than counterbore")
        if not (0.0 < self.legacy_detector_acceptance_deg < 90.0):
            raise ValueError("legacy detector acceptance must be between 0 and 90 degrees")
        if self.particle_wavelength_m <= 0:
            raise ValueError("particle_wavelength_m must be positive")
        if self.hybrid_wave_scale < 0 or not np.isfinite(self.hybrid_wave_scale):
            raise ValueError("hybrid_wave_scale must be finite and >=0")
        if self.mie_phase_grid_size < 257:
            raise ValueError("mie_phase_grid_size must be >=257")
        if not np.isfinite(self.particle_surface_rms_slope_deg) or not (0.0 <= self.particle_surface_rms_slope_deg < 80.0):
            raise ValueError("particle_surface_rms_slope_deg must be finite and in [0,80) degrees")
        if not np.isfinite(self.wave_surface_rms_height_m) or self.wave_surface_rms_height_m < 0.0:
            raise ValueError("wave_surface_rms_height_m must be finite and >=0")
        if not np.isfinite(self.wave_spheroid_aspect_ratio) or not (0.2 <= self.wave_spheroid_aspect_ratio <= 5.0):
            raise ValueError("wave_spheroid_aspect_ratio must be finite and in [0.2,5.0]")
        if not np.isfinite(self.wave_spheroid_orientation_kappa) or not (0.0 <= self.wave_spheroid_orientation_kappa <= 100.0):
            raise ValueError("wave_spheroid_orientation_kappa must be finite and in [0,100]")
        if not np.isfinite(self.vortex_wall_center_height_difference_m) or self.vortex_wall_center_height_difference_m < 0.0:
            raise ValueError("vortex_wall_center_height_difference_m must be finite and >=0")
        if self.free_surface_model == "localized_scully_vortex" and not (
            np.isfinite(self.vortex_core_radius_m) and self.vortex_core_radius_m > 0.0
        ):
            raise ValueError("vortex_core_radius_m must be finite and >0 for localized_scully_vortex")
        if self.free_surface_model == "rankine_vortex":
            if not (np.isfinite(self.vortex_core_radius_m) and self.vortex_core_radius_m > 0.0):
                raise ValueError("vortex_core_radius_m must be finite and >0 for rankine_vortex")
            if self.sediment_transport_model in ("stokes_drift_diffusion", "schiller_naumann_drift_diffusion"):
                raise ValueError("the analytic drift-diffusion sediment fields follow the reference's free surfaces; "
                                 "with rankine_vortex use 'uniform' or a supplied meridional field")
        if not np.isfinite(self.sediment_eddy_diffusivity_m2_s) or self.sediment_eddy_diffusivity_m2_s <= 0.0:
            raise ValueError("sediment_eddy_diffusivity_m2_s must be finite and >0")
        if not (np.isfinite(self.water_density_kg_per_m3) and 0.0 < self.water_density_kg_per_m3 < self.density_kg_per_m3):
            raise ValueError("water_density_kg_per_m3 must be positive and below particle density")
        if not np.isfinite(self.water_dynamic_viscosity_pa_s) or self.water_dynamic_viscosity_pa_s <= 0.0:
            raise ValueError("water_dynamic_viscosity_pa_s must be finite and >0")
        if not np.isfinite(self.gravity_m_s2) or self.gravity_m_s2 <= 0.0:
            raise ValueError("gravity_m_s2 must be finite and >0")
        if self.sediment_transport_quadrature_points < 64:
            raise ValueError("sediment_transport_quadrature_points must be >=64")
        if self.sediment_radial_lookup_points < 65:
            raise ValueError("sediment_radial_lookup_points must be >=65")
        if not np.isfinite(self.meridional_circulation_ratio) or not (0.0 <= self.meridional_circulation_ratio <= 0.5):
            raise ValueError("meridional_circulation_ratio must be finite and in [0,0.5]")
        if self.meridional_grid_nr < 16 or self.meridional_grid_nz < 32:
            raise ValueError("meridional solver grid must be at least 16 x 32")
        if self.meridional_solver_max_iterations < 250 or self.meridional_solver_check_interval < 10:
            raise ValueError("invalid meridional solver iteration controls")
        if not np.isfinite(self.meridional_solver_tolerance) or not (0.0 < self.meridional_solver_tolerance < 1e-2):
            raise ValueError("meridional_solver_tolerance must be in (0,1e-2)")
        if not np.isfinite(self.meridional_solver_sor) or not (1.0 <= self.meridional_solver_sor < 1.95):
            raise ValueError("meridional_solver_sor must be in [1,1.95)")
        vg = vortex_surface_geometry(self.free_surface_model, self.zmean, self.tube_inner_radius_m,
                                     self.vortex_wall_center_height_difference_m, self.vortex_core_radius_m,
                                     self.gravity_m_s2)
        if not (vg["wall_z"] < self.zwall_top):
            raise ValueError("free surface reaches or exceeds the physical acrylic wall top")
        if vg["center_z"] <= self.zmin:
            raise ValueError("vortex depression reaches or passes the acrylic bottom")
        if not (self.alpha1 > 0.0 and self.alpha2 > 0.0):
            raise ValueError("source Beta alpha1/alpha2 must be positive")
        if not (self.bore_refractive_index > 1.0):
            raise ValueError("bore_refractive_index must be >1")
        if self.max_bore_bounces < 0:
            raise ValueError("max_bore_bounces must be >=0")
        if self.max_ring_face_bounces < 1:
            raise ValueError("max_ring_face_bounces must be >=1")
        if not (self.zmin < 0 < self.zmean):
            raise ValueError("sensor plane must lie within water column")
        if self.bottom_disc_thickness_m <= 0.0:
            raise ValueError("bottom_disc_thickness_m must be positive")
        if self.bottom_external_refractive_index <= 0.0:
            raise ValueError("bottom_external_refractive_index must be positive")
        if self.max_axial_bounces < 1:
            raise ValueError("max_axial_bounces must be >=1")
        if self.chunk_size < 1 or self.statistics_batch_rays < 1:
            raise ValueError("chunk/batch sizes must be positive")
        if self.source_kind not in ("reference_led", "collimated_disc"):
            raise ValueError("source_kind must be 'reference_led' or 'collimated_disc'")
        if not (np.isfinite(self.water_absorption_per_m) and self.water_absorption_per_m >= 0.0):
            raise ValueError("water_absorption_per_m must be finite and nonnegative")
        if self.aggregation_model not in ("none", "orthokinetic_compact", "orthokinetic_compact_fragmentation"):
            raise ValueError("aggregation_model must be 'none', 'orthokinetic_compact', or "
                             "'orthokinetic_compact_fragmentation'")
        if not np.isfinite(self.aggregation_collision_exposure) or self.aggregation_collision_exposure < 0.0:
            raise ValueError("aggregation_collision_exposure must be finite and >=0")
        if not np.isfinite(self.fragmentation_breakup_exposure) or self.fragmentation_breakup_exposure < 0.0:
            raise ValueError("fragmentation_breakup_exposure must be finite and >=0")
        if not np.isfinite(self.fragmentation_reference_diameter_m) or self.fragmentation_reference_diameter_m <= 0.0:
            raise ValueError("fragmentation_reference_diameter_m must be finite and >0")
        if not np.isfinite(self.fragmentation_size_exponent) or not (0.0 <= self.fragmentation_size_exponent <= 6.0):
            raise ValueError("fragmentation_size_exponent must be finite and in [0,6]")
        if self.aggregation_model != "orthokinetic_compact_fragmentation" and self.fragmentation_breakup_exposure > 0.0:
            raise ValueError("fragmentation_breakup_exposure requires aggregation_model=orthokinetic_compact_fragmentation")
        if not (0.0 < self.aggregation_step_safety <= 0.25):
            raise ValueError("aggregation_step_safety must be in (0,0.25]")
        if self.aggregation_max_steps < 1:
            raise ValueError("aggregation_max_steps must be >=1")
        if self.aggregation_model != "none":
            raise NotImplementedError("aggregation/fragmentation population balance is not part of this library")

    def to_scene_params(self) -> abi.SceneParams:
        s = abi.SceneParams()
        s.n_water, s.n_acrylic, s.n_air = self.n_water, self.n_acrylic, self.n_air
        s.bore_n, s.ring_face_n = self.bore_refractive_index, self.ring_inner_face_refractive_index
        s.bottom_external_n = self.bottom_external_refractive_index
        s.rin, s.rout = self.tube_inner_radius_m, self.tube_outer_radius_m
        s.zmin, s.zmean, s.zwall_top = self.zmin, self.zmean, self.zwall_top
        s.bottom_disc_thickness = self.bottom_disc_thickness_m
        s.ring_in, s.throat_out, s.ring_out = self.sensor_ring_inner_radius_m, self.throat_out, self.sensor_ring_outer_radius_m
        s.source_r = self.source_launch_radius_m
        s.throat_r = 0.5 * self.through_bore_diameter_m
        s.counterbore_r = 0.5 * self.counterbore_diameter_m
        s.beam_sigma, s.alpha1, s.alpha2 = self.source_beam_sigma_m, self.alpha1, self.alpha2
        s.legacy_accept_deg = self.legacy_detector_acceptance_deg
        s.source_angular_model = SOURCE_ANGULAR_MODEL_CODES[self.source_angular_model]
        s.source_bore_model = BORE_SURFACE_MODEL_CODES[self.source_bore_surface_model]
        s.detector_bore_model = BORE_SURFACE_MODEL_CODES[self.detector_bore_surface_model]
        s.ring_face_model = RING_FACE_SURFACE_MODEL_CODES[self.ring_inner_face_surface_model]
        s.photodiode_model = PHOTODIODE_RESPONSE_MODEL_CODES[self.photodiode_response_model]
        s.max_bore_bounces, s.max_ring_face_bounces = self.max_bore_bounces, self.max_ring_face_bounces
        s.free_surface_model = FREE_SURFACE_MODEL_CODES[self.free_surface_model]
        s.vortex_delta_h, s.vortex_core_radius = self.vortex_wall_center_height_difference_m, self.vortex_core_radius_m
        s.wavelength = self.particle_wavelength_m
        s.rough_alpha = self.rough_alpha
        s.spheroid_aspect = self.wave_spheroid_aspect_ratio
        s.orientation_kappa = self.wave_spheroid_orientation_kappa
        s.orientation_model = SPHEROID_ORIENTATION_MODEL_CODES[self.wave_spheroid_orientation_model]
        s.max_particle_bounces = self.max_internal_bounces
        s.max_cell_bounces, s.max_axial_bounces = self.max_cell_bounces, self.max_axial_bounces
        s.max_iterations = float(self.max_iterations)
        s.event_model = EVENT_MODEL_CODES[self.particle_event_model]
        s.conditional_retries = CONDITIONAL_MAX_TRIALS
        s.sediment_model = SEDIMENT_TRANSPORT_MODEL_CODES[self.sediment_transport_model]
        s.source_kind = abi.SOURCE_COLLIMATED_DISC if self.source_kind == "collimated_disc" else abi.SOURCE_REFERENCE_LED
        s.disc_radius = self.disc_beam_radius_m
        s.disc_height = 0.0
        s.water_absorption = float(self.water_absorption_per_m)
        return s

    def sediment_spec(self, grid: Optional[np.ndarray] = None, grid_zmax: Optional[float] = None):
        """Sediment precompute inputs; keeps numpy buffers alive on the returned object."""
        sp = abi.SedimentSpec()
        sp.particle_density = self.density_kg_per_m3
        sp.water_density = self.water_density_kg_per_m3
        sp.water_viscosity = self.water_dynamic_viscosity_pa_s
        sp.gravity = self.gravity_m_s2
        sp.eddy_diffusivity = self.sediment_eddy_diffusivity_m2_s
        sp.n_quad = self.sediment_transport_quadrature_points
        sp.n_radial = self.sediment_radial_lookup_points
        vg = vortex_surface_geometry(self.free_surface_model, self.zmean, self.tube_inner_radius_m,
                                     self.vortex_wall_center_height_difference_m, self.vortex_core_radius_m,
                                     self.gravity_m_s2)
        sp.grid_zmax = float(vg["wall_z"]) if grid_zmax is None else float(grid_zmax)
        # FP64 geometry as the reference passes it to its sediment kernels (CLARITAS/CLARITAS.py:6413-6418)
        sp.rin, sp.zmin, sp.zmean = float(self.tube_inner_radius_m), self.zmin, self.zmean
        sp.vortex_delta_h = float(self.vortex_wall_center_height_difference_m)
        sp.vortex_core_radius = float(self.vortex_core_radius_m)
        # meridional solver settings (used for sediment model 3 without a supplied grid, :6451-6725); the peak
        # speed is chi x the vortex's peak azimuthal speed for a stirred surface, else 0 (:5901-5907)
        sp.meridional_nr, sp.meridional_nz = int(self.meridional_grid_nr), int(self.meridional_grid_nz)
        sp.solver_max_iterations = int(self.meridional_solver_max_iterations)
        sp.solver_check_interval = int(self.meridional_solver_check_interval)
        sp.solver_tolerance = float(self.meridional_solver_tolerance)
        sp.solver_sor = float(self.meridional_solver_sor)
        stirred = (self.free_surface_model in ("localized_scully_vortex", "parabolic_vortex")
                   and self.vortex_wall_center_height_difference_m > 0.0)
        sp.meridional_peak_speed = (float(self.meridional_circulation_ratio) * float(vg["vtheta_peak_m_s"])
                                    if stirred else 0.0)
        keep = []
        if grid is not None:
            g = np.ascontiguousarray(grid, dtype=np.float64)
            if g.ndim != 3:
                raise ValueError("sediment grid must be [bins, nr, nz]")
            sp.grid_nr, sp.grid_nz = int(g.shape[1]), int(g.shape[2])
            sp.grid = g.ctypes.data_as(abi.PD)
            keep.append(g)
        else:
            sp.grid_nr = sp.grid_nz = 2
        sp._keep = keep  # type: ignore[attr-defined]
        return sp


def rankine_surface_coefficients(zmean: float, R: float, delta_h: float, core_r: float):
    """(k, a, z0) of the Rankine free surface z0 + k r^2 (r <= a), z0 + k a^2 (2 - a^2/r^2) (r > a).

    The stirrer turns the core r <= a as a solid body at angular speed W and the liquid outside as a free
    vortex (v = W a^2 / r); the radial pressure balance gives k = W^2 / (2 g), continuous with its slope at
    r = a. k is set by the wall-centre height difference delta_h = k a^2 (2 - a^2/R^2), and z0 = zmean - hbar
    by volume conservation, hbar = (k/R^2) (a^4/2 + 2 a^2 (R^2 - a^2) - 2 a^4 ln(R/a)). A core wider than the
    tube is clamped to it (solid-body rotation, the parabolic surface). No reference counterpart.
    """
    R, a = float(R), min(float(core_r), float(R))
    a2, R2 = a * a, R * R
    k = float(delta_h) / (a2 * (2.0 - a2 / R2))
    hbar = (k / R2) * (0.5 * a2 * a2 + 2.0 * a2 * (R2 - a2) - 2.0 * a2 * a2 * math.log(R / a))
    return k, a, float(zmean) - hbar


def rankine_surface(r, zmean: float, R: float, delta_h: float, core_r: float):
    """Height of the Rankine free surface at radius r (array or scalar)."""
    k, a, z0 = rankine_surface_coefficients(zmean, R, delta_h, core_r)
    r = np.asarray(r, dtype=float)
    q = r * r
    return np.where(q <= a * a, z0 + k * q, z0 + k * a * a * (2.0 - a * a / np.maximum(q, 1e-300)))


def stirrer_rankine_delta_h(rpm: float, core_radius_m: float, R: float, gravity: float = 9.81) -> float:
    """Wall-minus-centre height of the Rankine surface of a stirrer whose core (radius a) turns at `rpm`:
    k = W^2 / (2 g) with W = 2 pi rpm / 60, and delta_h = k a^2 (2 - a^2/R^2). No reference counterpart."""
    w = float(rpm) * 2.0 * math.pi / 60.0
    a = min(float(core_radius_m), float(R))
    k = w * w / (2.0 * gravity)
    return k * a * a * (2.0 - a * a / (float(R) * float(R)))


def vortex_surface_geometry(model, zmean, R, delta_h, core_r, gravity=9.81):
    """Free-surface centre/wall heights and swirl of the selected surface model.

    Same arithmetic as the reference host helper (CLARITAS/CLARITAS.py:708-792), because the wall
    height sets the sediment grid's upper edge and the constructor's geometry checks. The Rankine
    vortex (this library's model) reports its core angular speed.
    """
    model = str(model).strip().lower()
    zmean, R, D, a, g = float(zmean), float(R), float(delta_h), float(core_r), float(gravity)
    if not (R > 0.0 and np.isfinite(R)):
        raise ValueError("vessel radius must be finite and positive")
    if not (D >= 0.0 and np.isfinite(D)):
        raise ValueError("vortex wall-centre height difference must be finite and nonnegative")
    if not (g > 0.0 and np.isfinite(g)):
        raise ValueError("gravity must be finite and positive")
    R2 = R * R
    if not (R2 > 0.0 and np.isfinite(R2)):
        raise ValueError("vessel radius squared is outside the finite numerical range")
    if model == "flat" or D == 0.0:
        return dict(center_z=zmean, wall_z=zmean, h_inf=0.0, h_bar=0.0, angular_velocity_rad_s=0.0,
                    vtheta_peak_m_s=0.0, equivalent_rigid_body_rpm=0.0, equivalent_core_rpm=0.0)
    if model == "parabolic_vortex":
        omega = math.sqrt(2.0 * g * D / R2)
        if not (np.isfinite(omega) and np.isfinite(omega * 60.0 / (2.0 * math.pi))):
            raise ValueError("parabolic vortex derived angular velocity is non-finite")
        return dict(center_z=zmean - 0.5 * D, wall_z=zmean + 0.5 * D, h_inf=D, h_bar=0.5 * D,
                    angular_velocity_rad_s=omega, vtheta_peak_m_s=omega * R,
                    equivalent_rigid_body_rpm=omega * 60.0 / (2.0 * math.pi), equivalent_core_rpm=float("nan"))
    if model == "rankine_vortex":
        if not (a > 0.0):
            raise ValueError("Rankine vortex requires a positive core radius")
        k, ae, z0 = rankine_surface_coefficients(zmean, R, D, a)
        omega = math.sqrt(2.0 * g * k)
        return dict(center_z=z0, wall_z=z0 + D, h_inf=k * ae * ae * 2.0, h_bar=zmean - z0,
                    angular_velocity_rad_s=omega, vtheta_peak_m_s=omega * ae,
                    equivalent_rigid_body_rpm=float("nan"), equivalent_core_rpm=omega * 60.0 / (2.0 * math.pi))
    if model != "localized_scully_vortex":
        raise ValueError(f"unknown free-surface model {model!r}")
    if not (a > 0.0):
        raise ValueError("localized Scully vortex requires positive core and vessel radii")
    a2 = a * a
    if not (a2 > 0.0 and np.isfinite(a2)):
        raise ValueError("localized Scully core radius squared is outside the finite numerical range")
    h_inf = D * (a2 + R2) / R2
    h_bar = h_inf * (1.0 - (a2 / R2) * math.log1p(R2 / a2))
    omega_c = math.sqrt(2.0 * g * h_inf / a2)
    if not all(np.isfinite(q) for q in (h_inf, h_bar, omega_c)):
        raise ValueError("localized Scully derived geometry or angular velocity is non-finite")
    return dict(center_z=zmean - h_bar, wall_z=zmean - h_bar + D, h_inf=h_inf, h_bar=h_bar,
                angular_velocity_rad_s=omega_c, vtheta_peak_m_s=0.5 * omega_c * a,
                equivalent_rigid_body_rpm=float("nan"), equivalent_core_rpm=omega_c * 60.0 / (2.0 * math.pi))


@dataclass
class Particles:
    """A particle population in size bins: diameters, weights and complex index per bin."""
    diameter_m: np.ndarray
    weight: np.ndarray
    n_real: np.ndarray
    k_imag: np.ndarray
    concentration_kg_m3: float
    density_kg_m3: float = 2650.0
    weight_mode: str = "mass_fraction"

    def __post_init__(self):
        for name in ("diameter_m", "weight", "n_real", "k_imag"):
            setattr(self, name, np.ascontiguousarray(np.asarray(getattr(self, name), dtype=np.float64)))
        n = self.diameter_m.size
        if not (1 <= n <= abi.MAX_BINS):
            raise ValueError(f"1..{abi.MAX_BINS} size bins are supported, got {n}")
        for name in ("weight", "n_real", "k_imag"):
            if getattr(self, name).shape != (n,):
                raise ValueError(f"{name} must have {n} entries")
        w = self.weight
        if np.any(~np.isfinite(w)) or np.any(w < 0.0) or not np.any(w > 0.0):
            raise ValueError("invalid PSD weights")
        if np.any(~np.isfinite(self.n_real)) or np.any(self.n_real <= 0) or np.any(self.k_imag < 0):
            raise ValueError("invalid n/k values")
        if self.weight_mode not in WEIGHT_MODE_CODES:
            raise ValueError("weight_mode must be 'mass_fraction' or 'number_fraction'")
        c = float(self.concentration_kg_m3)
        if not np.isfinite(c) or c < 0.0:
            raise ValueError("concentration must be finite and >=0")

    def spec(self, cfg: ModelConfig, moments: Optional[dict] = None,
             table_arithmetic: int = abi.TABLES_REFERENCE) -> abi.ParticleSpec:
        ps = abi.ParticleSpec()
        ps.table_arithmetic = int(table_arithmetic)
        ps.n_bins = int(self.diameter_m.size)
        hybrid = cfg.particle_event_model in ("hybrid_mie_excess", "hybrid_mie_exact_rate",
                                              "hybrid_mie_exact_rate_moment_constrained")
        ps.n_theta = int(cfg.mie_phase_grid_size) if hybrid else 2
        ps.weight_mode = WEIGHT_MODE_CODES[self.weight_mode]
        keep = [self.diameter_m, self.weight, self.n_real, self.k_imag]
        ps.diameter_m = self.diameter_m.ctypes.data_as(abi.PD)
        ps.weight = self.weight.ctypes.data_as(abi.PD)
        ps.n_real = self.n_real.ctypes.data_as(abi.PD)
        ps.k_imag = self.k_imag.ctypes.data_as(abi.PD)
        if moments is not None:
            a = np.ascontiguousarray(moments["a"], dtype=np.float64)
            b = np.ascontiguousarray(moments["b"], dtype=np.float64)
            m = np.ascontiguousarray(moments["mode"], dtype=np.uint8)
            keep += [a, b, m]
            ps.moment_enabled = 1
            ps.moment_a = a.ctypes.data_as(abi.PD)
            ps.moment_b = b.ctypes.data_as(abi.PD)
            ps.moment_mode = m.ctypes.data_as(abi.PU8)
        ps.concentration_kg_m3 = float(self.concentration_kg_m3)
        ps.density_kg_m3 = float(self.density_kg_m3)
        ps.n_medium = float(cfg.n_water)
        ps.wavelength_m = float(cfg.particle_wavelength_m)
        ps.wave_rms_height_m = float(cfg.wave_surface_rms_height_m)
        ps.hybrid_wave_scale = float(cfg.hybrid_wave_scale)
        ps._keep = keep  # type: ignore[attr-defined]
        return ps


def reference_seeds(seed: int) -> tuple[int, int, int, int]:
    """The reference's derived per-run seeds (simulate, CLARITAS/CLARITAS.py:7304-7306 and :7780-7782)."""
    s = int(seed)
    seed0 = ((s * 1664525 + 1013904223) & 0x7FFFFFFF) or 1
    seed1 = ((s * 22695477 + 1) & 0x7FFFFFFF) or 7
    seed2 = ((s * 1103515245 + 12345) & 0x7FFFFFFF) or 11
    det = ((s * 2654435761 + 97531) & 0x7FFFFFFF) or 17
    return seed0, seed1, seed2, det


def run_params(n_rays: int, seed: int = 0, ray_offset: int = 0, rng_mode: int = abi.RNG_REFERENCE_XORSHIFT,
               weight_mode: int = abi.WEIGHT_ANALOG, roulette_threshold: float = 1e-4, roulette_survival: float = 1e-3,
               scenario_id: int = 0, max_blocks: int = 0, rays_per_item: int = 0, flags: int = 0) -> abi.RunParams:
    r = abi.RunParams()
    r.n_rays = int(n_rays)
    r.ray_offset = int(ray_offset) & 0xFFFFFFFF
    r.seed0, r.seed1, r.seed2, r.detector_seed = reference_seeds(seed)
    r.rng_mode = int(rng_mode)
    r.philox_key = (int(seed) * 0x9E3779B97F4A7C15 + 0x632BE59BD9B4E019) & 0xFFFFFFFFFFFFFFFF
    r.scenario_id = int(scenario_id)
    r.weight_mode = int(weight_mode)
    r.roulette_threshold = float(roulette_threshold)
    r.roulette_survival = float(roulette_survival)
    r.max_blocks = int(max_blocks)
    r.rays_per_item = int(rays_per_item)
    r.flags = int(flags)
    return r


# ----------------------------------------------------------------------------------------------
# Synthetic workloads (seeded; shapes and value ranges of the benchmark descriptions)
# ----------------------------------------------------------------------------------------------
def replica_ray_offset(rank: int, step: int, steps_per_rank: int, n_rays: int) -> int:
    """First global photon id of one replica step. Replicas (one per GPU) and their steps take
    disjoint, contiguous photon ranges; with per-ray random streams keyed by the global photon id the
    summed integer tallies of the shards equal those of one run over the union."""
    return ((int(rank) * int(steps_per_rank) + int(step)) * int(n_rays)) % (1 << 31)


def lognormal_mass_psd(n_bins: int, d_min: float, d_max: float, median: float, sigma_g: float):
    """Log-spaced diameters with lognormal mass weights (bin-centre density x log-width)."""
    d = np.geomspace(d_min, d_max, n_bins)
    z = (np.log(d) - math.log(median)) / math.log(sigma_g)
    w = np.exp(-0.5 * z * z)
    return d, w / w.sum()


def small_cell_config(**overrides) -> ModelConfig:
    """The small plain-MC cell: r = 12.5 mm, 50 mm tube, 40 mm water, beam plane 20 mm above the bottom.

    Wall, ring and bore dimensions keep the reference's engineering offsets (3.5 mm acrylic, 0.5 mm
    clearance, 15 mm ring, 8 mm counterbore), so the constructor's radial ordering holds.
    """
    base = dict(
        tube_inner_radius_m=0.0125, tube_outer_radius_m=0.0160, tube_length_m=0.050,
        water_height_m=0.040, sensor_height_above_bottom_m=0.020,
        sensor_ring_inner_radius_m=0.0165, sensor_ring_outer_radius_m=0.0315, source_launch_radius_m=0.0315,
        counterbore_depth_m=0.008, n_water=1.33,
        free_surface_model="flat", vortex_wall_center_height_difference_m=0.0,
        sediment_transport_model="uniform", particle_event_model="hybrid_mie_exact_rate",
        particle_wavelength_m=860e-9, mie_phase_grid_size=1801, density_kg_per_m3=2650.0,
    )
    base.update(overrides)
    return ModelConfig(**base)


def quartz_particles(concentration_mg_l: float = 100.0, n_bins: int = 64, median_um: float = 20.0,
                     sigma_g: float = 1.6, d_min_um: float = 1.0, d_max_um: float = 200.0, n: float = 1.54,
                     k: float = 0.0, density: float = 2650.0) -> Particles:
    d, w = lognormal_mass_psd(n_bins, d_min_um * 1e-6, d_max_um * 1e-6, median_um * 1e-6, sigma_g)
    return Particles(d, w, np.full(n_bins, n), np.full(n_bins, k), concentration_mg_l * 1e-3, density)


def kaolin_clay_particles(concentration_mg_l: float, n_bins: int = 16, median_um: float = 2.0, sigma_g: float = 1.5,
                          d_min_um: float = 0.5, d_max_um: float = 10.0, density: float = 2650.0) -> Particles:
    """Lognormal clay whose per-bin n and k follow the reference's kaolin optical-constant table (bundled in
    materials.npz), interpolated in log diameter and held constant beyond the table's ends."""
    from . import materials as M
    d, w = lognormal_mass_psd(n_bins, d_min_um * 1e-6, d_max_um * 1e-6, median_um * 1e-6, sigma_g)
    td, _ = M.get_material_psd_raw("kaolin")
    tn, tk = M.get_material_optical_constants("kaolin")
    order = np.argsort(td)
    x, xs = np.log(d), np.log(td[order])
    return Particles(d, w, np.interp(x, xs, tn[order]), np.interp(x, xs, tk[order]), concentration_mg_l * 1e-3,
                     density)


def three_component_particles(concentration_mg_l: float = 500.0, bins_per_component: int = 21,
                              medians_um=(2.0, 20.0, 100.0), fractions=(0.3, 0.5, 0.2), sigma_g: float = 1.4,
                              n: float = 1.54, k: float = 0.0, density: float = 2650.0) -> Particles:
    """Clay/silt/sand mixture: three lognormal components on separate log grids, mass fractions summed."""
    ds, ws = [], []
    for med, frac in zip(medians_um, fractions):
        lo, hi = med * 1e-6 / sigma_g ** 3, med * 1e-6 * sigma_g ** 3
        d, w = lognormal_mass_psd(bins_per_component, lo, hi, med * 1e-6, sigma_g)
        ds.append(d)
        ws.append(w * frac)
    d = np.concatenate(ds)
    w = np.concatenate(ws)
    order = np.argsort(d)
    d, w = d[order], w[order]
    m = d.size
    return Particles(d, w / w.sum(), np.full(m, n), np.full(m, k), concentration_mg_l * 1e-3, density)


def stirrer_scully_delta_h(rpm: float, core_radius_m: float, R: float, gravity: float = 9.81) -> float:
    """Wall-minus-centre height of the localized Scully surface whose core turns at `rpm`.

    Inverts the reference's relation omega_c = sqrt(2 g H_inf)/a with H_inf = dH (a^2+R^2)/R^2
    (vortex_surface_geometry, CLARITAS/CLARITAS.py:772-779) for dH.
    """
    omega = float(rpm) * 2.0 * math.pi / 60.0
    a, R2 = float(core_radius_m), float(R) * float(R)
    h_inf = (omega * a) ** 2 / (2.0 * gravity)
    return h_inf * R2 / (a * a + R2)


def rouse_radial_grid(cfg: ModelConfig, n_bins: int, nr: int = 64, nz: int = 64, rouse: float = 0.3,
                      ref_height_frac: float = 0.05, radial_kappa: float = 0.5) -> tuple[np.ndarray, float]:
    """Concentration-scale field on the reference's cell-centred (r, z) grid, volume mean 1 over the water.

    Vertical: Rouse profile c/c_a = [((h - s)/s) (a/(h - a))]^P, s the height above the bottom, h the local
    water depth, a = ref_height_frac*h (clamped below a). Radial: centrifugal depletion exp(kappa (r^2/R^2 - 1)).
    Cells above the local free surface take the value of the highest liquid cell in their column, as the
    reference's grid extension does (CLARITAS/CLARITAS.py:4195-4201), so bilinear lookups near the surface
    stay inside the field. Returns (grid [bins][nr][nz], grid_zmax).
    """
    R, zmin = float(cfg.tube_inner_radius_m), cfg.zmin
    vg = vortex_surface_geometry(cfg.free_surface_model, cfg.zmean, R, cfg.vortex_wall_center_height_difference_m,
                                 cfg.vortex_core_radius_m, cfg.gravity_m_s2)
    zmax = float(vg["wall_z"])
    dr, dz = R / nr, (zmax - zmin) / nz
    rc = (np.arange(nr) + 0.5) * dr
    zc = zmin + (np.arange(nz) + 0.5) * dz

    def surface(r):
        if cfg.free_surface_model == "flat" or cfg.vortex_wall_center_height_difference_m <= 0:
            return np.full_like(r, cfg.zmean)
        dh = cfg.vortex_wall_center_height_difference_m
        if cfg.free_surface_model == "parabolic_vortex":
            return cfg.zmean + dh * (r * r / (R * R) - 0.5)
        if cfg.free_surface_model == "rankine_vortex":
            return rankine_surface(r, cfg.zmean, R, dh, cfg.vortex_core_radius_m)
        a2, R2 = cfg.vortex_core_radius_m ** 2, R * R
        return cfg.zmean - vg["h_bar"] + vg["h_inf"] * r * r / (a2 + r * r)

    zs = surface(rc)
    g = np.zeros((nr, nz))
    active = np.zeros((nr, nz), bool)
    for i in range(nr):
        h = zs[i] - zmin
        a = ref_height_frac * h
        s = np.clip(zc - zmin, 1e-9, None)
        live = zc < zs[i]
        prof = np.where(s > a, (((h - s) / s) * (a / (h - a))).clip(min=0.0) ** rouse, 1.0)
        g[i] = prof * math.exp(radial_kappa * (rc[i] ** 2 / (R * R) - 1.0))
        active[i] = live
        top = np.nonzero(live)[0]
        if top.size:
            g[i, top[-1] + 1:] = g[i, top[-1]]
    w = (rc[:, None] * dr * dz) * active
    g /= (g * w).sum() / w.sum()
    return np.ascontiguousarray(np.broadcast_to(g, (n_bins, nr, nz))), zmax


def full_scene_workload(n_photons: int = 100_000_000, surface: str = "localized_scully_vortex", rpm: float = 600.0):
    """The full scene: three-component mixture at 500 mg/L in a (r, z) Rouse x radial-depletion field with a
    stirred (600 rpm, 5 mm core) free surface, small cell. `surface` is the stirred surface: the Rankine
    vortex ("rankine_vortex", this library's model of a stirrer) or the reference's localized Scully vortex
    with the same core angular speed (the reference-supported stand-in). Returns (config, particles, grid,
    grid_zmax)."""
    base = small_cell_config(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0)
    if surface == "rankine_vortex":
        dh = stirrer_rankine_delta_h(rpm, 0.005, base.tube_inner_radius_m)
    elif surface == "localized_scully_vortex":
        dh = stirrer_scully_delta_h(rpm, 0.005, base.tube_inner_radius_m)
    else:
        raise ValueError(f"unknown stirred surface {surface!r}")
    cfg = small_cell_config(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0,
                            free_surface_model=surface, vortex_wall_center_height_difference_m=dh,
                            vortex_core_radius_m=0.005,
                            sediment_transport_model="schiller_naumann_meridional_advection_diffusion")
    cfg.validate()
    parts = three_component_particles(500.0)
    grid, zmax = rouse_radial_grid(cfg, parts.diameter_m.size)
    return cfg, parts, grid, zmax


def small_plain_workload():
    """The small plain-MC case: 64 lognormal bins (median 20 um, sigma_g 1.6) of quartz at 100 mg/L, uniform,
    lit by a 2 mm collimated disc beam through the 180-degree port at the sensor plane (20 mm above the
    bottom; this library's source option, the reference has only its LED)."""
    cfg = small_cell_config(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0,
                            source_kind="collimated_disc", disc_beam_radius_m=1.0e-3)
    cfg.validate()
    return cfg, quartz_particles(100.0), None, None


@dataclass
class SweepScenario:
    """One scenario of a batched sweep: its configuration, particles, photon count and seed."""
    cfg: ModelConfig
    particles: Particles
    n_photons: int
    seed: int
    params: dict


def sweep_workload(n_scenarios: int = 512, sampler_seed: int = 0, n_bins: int = 64,
                   photons: tuple = (1e5, 1e7), scale_photons: float = 1.0) -> list:
    """The batched sweep: n_scenarios scenarios in the small cell, drawn with numpy's PCG64 from
    `sampler_seed`. Per scenario: photon count log-uniform over `photons` (times scale_photons),
    concentration log-uniform 1-1e4 mg/L, median diameter log-uniform 2-200 um, sigma_g uniform 1.2-2.0,
    stirrer rpm uniform 0-1200 (localized-vortex surface with a 5 mm core), particle index uniform
    1.50-1.60 (k = 0); 860 nm; 64 lognormal mass bins over 1-200 um; uniform sediment; scenario i uses
    seed i."""
    rng = np.random.Generator(np.random.PCG64(int(sampler_seed)))
    n = int(n_scenarios)
    lo, hi = math.log(photons[0]), math.log(photons[1])
    n_ph = np.exp(rng.uniform(lo, hi, n))
    conc = np.exp(rng.uniform(math.log(1.0), math.log(1e4), n))
    d50 = np.exp(rng.uniform(math.log(2.0), math.log(200.0), n))
    sig = rng.uniform(1.2, 2.0, n)
    rpm = rng.uniform(0.0, 1200.0, n)
    nidx = rng.uniform(1.50, 1.60, n)
    base = small_cell_config(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0)
    out = []
    for i in range(n):
        dh = stirrer_scully_delta_h(float(rpm[i]), 0.005, base.tube_inner_radius_m)
        if dh > 0.0:
            cfg = small_cell_config(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0,
                                    free_surface_model="localized_scully_vortex",
                                    vortex_wall_center_height_difference_m=dh, vortex_core_radius_m=0.005)
        else:
            cfg = small_cell_config(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0)
        cfg.validate()
        parts = quartz_particles(float(conc[i]), n_bins=n_bins, median_um=float(d50[i]), sigma_g=float(sig[i]),
                                 n=float(nidx[i]))
        out.append(SweepScenario(cfg, parts, max(1, int(round(float(n_ph[i]) * scale_photons))), i,
                                 dict(concentration_mg_l=float(conc[i]), median_um=float(d50[i]),
                                      sigma_g=float(sig[i]), rpm=float(rpm[i]), n_particle=float(nidx[i]))))
    return out


def sweep_specs(scenarios: list, table_arithmetic: int = abi.TABLES_REFERENCE) -> tuple[list, list, list]:
    """ABI inputs of a sweep: (scene params, particle specs, sediment specs), one each per scenario."""
    scenes = [sc.cfg.to_scene_params() for sc in scenarios]
    parts = [sc.particles.spec(sc.cfg, table_arithmetic=table_arithmetic) for sc in scenarios]
    seds = [sc.cfg.sediment_spec() for sc in scenarios]
    return scenes, parts, seds

