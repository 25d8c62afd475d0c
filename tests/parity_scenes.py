"""Parity scenes shared by the golden-fixture generators and the parity tests.

Every scene is the small cell (r = 12.5 mm) with one physics option switched
on, so that together they exercise every branch of the transport path:
rough/smooth particle surfaces, spheroid morphology, coherent Mie sampling,
absorbing bins (conditional closure), the three free surfaces, the four
sediment transport models, reflective bores and ring face, photodiode
response and the source angular laws, and the meridional field solver.
"""
from __future__ import annotations

import hashlib

import numpy as np

from tardiis_and_claritas_gb300 import scene as S


def _grid(n_bins: int) -> np.ndarray:
    rng = np.random.default_rng(20261203)
    return rng.uniform(0.5, 1.5, (n_bins, 32, 48))


PARABOLIC = dict(free_surface_model="parabolic_vortex", vortex_wall_center_height_difference_m=0.01)
SCULLY = dict(free_surface_model="localized_scully_vortex", vortex_wall_center_height_difference_m=0.008,
              vortex_core_radius_m=0.005)

# name -> (config overrides, particle kwargs, needs grid)
SCENES = {
    "c1_smooth_coherent": (dict(particle_surface_rms_slope_deg=0.0, wave_surface_rms_height_m=0.0),
                           dict(concentration_mg_l=100.0), False),
    "rough_spheroid": (dict(), dict(concentration_mg_l=2000.0), False),
    "smooth_spheroid": (dict(particle_surface_rms_slope_deg=0.0), dict(concentration_mg_l=2000.0), False),
    "geometric_law": (dict(particle_event_model="geometric"), dict(concentration_mg_l=2000.0), False),
    "mie_qsca_law": (dict(particle_event_model="mie_qsca"), dict(concentration_mg_l=2000.0), False),
    "hybrid_excess": (dict(particle_event_model="hybrid_mie_excess"), dict(concentration_mg_l=2000.0), False),
    "absorbing_conditional": (dict(), dict(concentration_mg_l=2000.0, k=1e-3), False),
    "parabolic_surface": (PARABOLIC, dict(concentration_mg_l=2000.0), False),
    "scully_surface": (SCULLY, dict(concentration_mg_l=2000.0), False),
    "stokes_sediment": (dict(PARABOLIC, sediment_transport_model="stokes_drift_diffusion"),
                        dict(concentration_mg_l=2000.0), False),
    "schiller_sediment": (dict(SCULLY, sediment_transport_model="schiller_naumann_drift_diffusion"),
                          dict(concentration_mg_l=2000.0), False),
    "grid_sediment": (dict(PARABOLIC, sediment_transport_model="schiller_naumann_meridional_advection_diffusion"),
                      dict(concentration_mg_l=2000.0), True),
    # model 3 without a supplied field: the meridional advection-diffusion solver makes it
    "meridional_solver": (dict(SCULLY, sediment_transport_model="schiller_naumann_meridional_advection_diffusion"),
                          dict(concentration_mg_l=2000.0), False),
    "reflective_bores": (dict(source_bore_surface_model="smooth_fresnel_nylon",
                              detector_bore_surface_model="smooth_fresnel_nylon",
                              ring_inner_face_surface_model="smooth_fresnel_nylon"),
                         dict(concentration_mg_l=2000.0), False),
    "sfh213_photodiode": (dict(photodiode_response_model="sfh213_datasheet_fit"), dict(concentration_mg_l=2000.0), False),
    "legacy_source": (dict(source_angular_model="legacy_polar_pdf"), dict(concentration_mg_l=500.0), False),
    "vmf_orientation": (dict(wave_spheroid_orientation_model="local_tangential_axial_vmf",
                             wave_spheroid_orientation_kappa=3.0), dict(concentration_mg_l=2000.0), False),
}


# The dense stress regime (the 20 g/L, 2 um clay case in the small cell, localized-vortex surface: optical
# depth ~100, tens of thousands of events on the longest histories): CPU oracle only.
CPU_ONLY = {
    "dense_clay": (SCULLY, dict(concentration_mg_l=20000.0, n_bins=16, median_um=2.0, sigma_g=1.5, d_min_um=0.5,
                                d_max_um=10.0), False),
}
# The moment-constrained event law (model 5: the Mie two-moment post-outcome map of the reference,
# apply_mie_moment_constraint, CLARITAS/CLARITAS.py:4459-4476) with per-bin moment coefficients; its GPU
# golden fixture is a file of its own (gpu_ref_moment_fixtures.npz).
MOMENT_SCENES = {
    "moment_constrained": (dict(particle_event_model="hybrid_mie_exact_rate_moment_constrained"),
                           dict(concentration_mg_l=2000.0), False),
}
# Every scene runs in the CPU oracle as well (the meridional field solver included).
CPU_SCENES = list(SCENES) + list(CPU_ONLY)
# Scenes whose sediment field the meridional solver makes (no supplied grid).
SOLVED_FIELD = {"meridional_solver"}


def moments(name: str, n_bins: int):
    """Per-bin moment coefficients (a, b, mode) of a moment-constrained scene, else None: a fixed,
    non-trivial map (a in [0.7, 1.3], |b| <= 0.15, the map off in every third bin)."""
    if name not in MOMENT_SCENES:
        return None
    i = np.arange(n_bins, dtype=np.float64)
    return {"a": 0.7 + 0.6 * (i / max(n_bins - 1, 1)), "b": 0.15 * np.sin(i),
            "mode": (np.arange(n_bins) % 3 != 0).astype(np.uint8)}


def build(name: str):
    """(config, particles, grid-or-None) of a parity scene."""
    table = SCENES if name in SCENES else MOMENT_SCENES if name in MOMENT_SCENES else CPU_ONLY
    over, pk, needs_grid = table[name]
    cfg = S.small_cell_config(**over)
    cfg.validate()
    parts = S.quartz_particles(**pk)
    grid = _grid(parts.diameter_m.size) if needs_grid else None
    return cfg, parts, grid


def seed_of(name: str) -> int:
    return int(hashlib.sha256(name.encode()).hexdigest()[:6], 16)


def records_digest(rec: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(rec).tobytes()).hexdigest()


COMPACT_FIELDS = ("status", "interaction_count", "native_id", "mirror_id", "failure_code", "cell_inner_reflections",
                  "top_reflections")


def compact(rec: np.ndarray, n: int) -> np.ndarray:
    """Small integer summary of the first n records, stored in fixtures for diagnosis."""
    return np.stack([rec[f][:n].astype(np.int32) for f in COMPACT_FIELDS], axis=1)


TALLY_KEYS = ("hw_native", "hw_mirror", "hw_native_direct", "hw_mirror_direct", "hw_native_stray",
              "hw_mirror_stray", "hw_native_face", "hw_mirror_face", "legacy_native", "legacy_mirror",
              "status_counts", "failure_code_counts", "entered_sums", "ray_flags", "failure_subcode_counts",
              "ic_hist")
EVENT_KEYS = 20  # event_counts[0:20] are the reference's per-ray counter sums


def physics_digests(ph: dict) -> dict:
    out = {}
    for k, v in ph.items():
        out[k] = hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
    return out
