"""The reference's per-case output files, written from a ForwardResult.

* ``detector_response.csv`` — one row per detector angle with the reference's columns and integrity checks
  (`_write_detector_outputs`, CLARITAS/CLARITAS.py:12653-12696): absolute and normalised symmetric scores,
  native/mirror counts, the particle-uninteracted / interacted split from the exact interaction-order
  partition, sqrt(N) and batch-jackknife standard errors.
* ``run_summary.json`` — the case summary under the reference's key names (`_summary_dict`, :12849-12971),
  filled from the result and the model configuration; keys that describe the reference's own script
  environment (source digest, comparison baselines) carry this library's equivalents or None.

JSON and CSV values go through the reference's sanitiser rules (`_json_safe`, :11362-11375): arrays become
lists, NumPy scalars Python scalars, non-finite floats None; JSON is written sorted with indent 2.

The case-integrity policy (`resolved_failure_policy`, `production_integrity`, `diagnostic_integrity`,
`enforce_case_integrity`; :11876-12070) judges a case by its failed-ray fraction (failed rays stay in the
launched denominator) and, with light diagnostics, by their event reconciliation and track-length closure.
"""
from __future__ import annotations

import csv
import json
import math
from pathlib import Path

import numpy as np

from .scene import DETECTOR_ANGLES_DEG, vortex_surface_geometry


class CaseIntegrityError(RuntimeError):
    """A result field failed the reference's output integrity checks."""


# The reference's case-integrity policy (CLARITAS/CLARITAS.py:46-51): "report" keeps going and reports,
# "strict" stops on any diagnostic issue; a case whose failed-ray fraction exceeds the limit is fatal after
# its results are exported. None disables a limit.
DIAGNOSTIC_POLICY = "report"
MAX_FAILED_RAY_FRACTION = 0.001
MAX_UNEXPLAINED_EVENT_FRACTION = 0.001
MAX_DIAGNOSTIC_CLOSURE_ERROR = 0.001
ABORT_ON_SYSTEMIC_DIAGNOSTICS = False
STRICT_DIAGNOSTIC_CLOSURE_ERROR = 2e-6


def resolved_failure_policy(mode=None, **limits) -> dict:
    """The policy in force (`_resolved_failure_policy`, :11876-11892); keywords override the module values."""
    mode = DIAGNOSTIC_POLICY if mode is None else mode
    if mode not in ("report", "strict"):
        raise ValueError("DIAGNOSTIC_POLICY must be report or strict")
    lim = {"max_failed_ray_fraction": MAX_FAILED_RAY_FRACTION,
           "max_unexplained_event_fraction": MAX_UNEXPLAINED_EVENT_FRACTION,
           "max_diagnostic_closure_error": MAX_DIAGNOSTIC_CLOSURE_ERROR,
           "strict_closure_error": STRICT_DIAGNOSTIC_CLOSURE_ERROR}
    lim.update(limits)
    for key, value in lim.items():
        if value is not None and (not np.isfinite(value) or value < 0):
            raise ValueError(f"{key} must be finite and nonnegative, or None")
    return dict(lim, mode=mode, abort_on_systemic_diagnostics=bool(ABORT_ON_SYSTEMIC_DIAGNOSTICS))


def production_integrity(launched: int, failed: int, diagnostics: dict, policy: dict) -> dict:
    """Failed-ray accounting of a case (`_production_integrity`, :11895-11920): failed rays stay in the
    launched denominator (no renormalisation over successful rays); fatal beyond the policy's fraction."""
    if launched <= 0 or failed < 0 or failed > launched:
        raise ValueError("corrupted production ray counts")
    if not diagnostics.get("count_closure_ok", True):
        raise ValueError("production failure categories do not reconcile")
    fraction = failed / launched
    limit = policy["max_failed_ray_fraction"]
    fatal = limit is not None and fraction > limit
    return {
        "launched_rays": int(launched), "failed_rays": int(failed), "failed_ray_fraction": fraction,
        "normalization_rays": int(launched),
        "failure_categories": diagnostics.get("code_counts", {}),
        "failure_subcategories": diagnostics.get("subcode_counts", {}),
        "failure_samples": diagnostics.get("samples", []),
        "limitations": (["failed rays terminate without completion; valid histories and prefixes remain; "
                         "no successful-ray renormalization"] if failed else []),
        "fatal": bool(fatal),
        "status": "systemic_failure" if fatal else ("limited" if failed else "ok"),
    }


def case_integrity(res, policy=None):
    """The production and light-diagnostic integrity reports of a ForwardResult (the reference's case flow,
    :13031-13036 and :12066-12068); the light report is the disabled one without light diagnostics."""
    policy = resolved_failure_policy() if policy is None else policy
    prod = production_integrity(int(res.n_rays), int(res.production_failure_count),
                                res.production_failure_diagnostics, policy)
    light = getattr(res, "light_transport_diagnostics", None)
    diag = (diagnostic_integrity(light, policy) if light
            else {"diagnostic_status": "disabled", "fatal": False, "skipped_outputs": []})
    return prod, diag


def write_case_integrity(out, res, policy=None):
    """production_integrity_report.json (and light_transport_integrity_report.json with light diagnostics)
    of one case; returns both reports. The caller exports the case first and then calls
    enforce_case_integrity, as the reference does (:13204)."""
    out = Path(out)
    out.mkdir(parents=True, exist_ok=True)
    prod, diag = case_integrity(res, policy)
    write_json(out / "production_integrity_report.json", prod)
    if diag.get("diagnostic_status") != "disabled":
        write_json(out / "light_transport_integrity_report.json", diag)
    return prod, diag


def enforce_case_integrity(production: dict, diagnostic: dict) -> None:
    """`_enforce_case_integrity` (:11923-11927): raise once either report is fatal."""
    if production["fatal"] or diagnostic.get("fatal", False):
        raise CaseIntegrityError("case exceeded configured integrity policy; inspect persisted integrity reports "
                                 "and run_summary.json")


def light_transport_cross_sections(diag: dict, cfg: dict) -> dict:
    """Source-axis (x slab) and sensor-plane (z slab) sections of the light-history grids
    (`_light_transport_cross_sections`, CLARITAS/CLARITAS.py:11645-11700): voxel centres, the slabs'
    voxel indices (the nearest voxel when a slab is thinner than one), summed track length, post-scatter
    track length and event counts, and the same as densities per diagnostic ray and unit volume."""
    nx, ny, nz = (int(diag[k]) for k in ("nx", "ny", "nz"))

    def centres(axis, n):
        lo, hi = float(diag[axis + "_min_m"]), float(diag[axis + "_max_m"])
        return np.linspace(lo, hi, n, endpoint=False) + (hi - lo) / (2 * n), (hi - lo) / n
    (x, dx), (y, dy), (z, dz) = centres("x", nx), centres("y", ny), centres("z", nz)
    rays = max(int(diag["diagnostic_rays_processed"]), 1)
    vol = dx * dy * dz
    xi = np.flatnonzero(np.abs(x) <= 0.5 * cfg["vertical_slice_thickness_m"])
    zi = np.flatnonzero(np.abs(z) <= 0.5 * cfg["sensor_slice_thickness_m"])
    if not len(xi):
        xi = np.array([int(np.argmin(np.abs(x)))])
    if not len(zi):
        zi = np.array([int(np.argmin(np.abs(z)))])
    total = np.asarray(diag["track_length_m"], dtype=float)        # [z][y][x]
    post = np.asarray(diag["post_scatter_track_length_m"], dtype=float)
    events = np.asarray(diag["scatter_event_count"], dtype=float)
    q = {"x": x, "y": y, "z": z, "xi": xi, "zi": zi, "dx": dx, "dy": dy, "dz": dz, "voxel_volume": vol,
         "vr": total[:, :, xi].sum(2), "vp": post[:, :, xi].sum(2), "ve": events[:, :, xi].sum(2),
         "hr": total[zi].sum(0), "hp": post[zi].sum(0), "he": events[zi].sum(0)}
    for k in ("vr", "vp", "ve"):
        q[{"vr": "vd", "vp": "vpd", "ve": "ved"}[k]] = q[k] / (rays * vol * len(xi))
    for k in ("hr", "hp", "he"):
        q[{"hr": "hd", "hp": "hpd", "he": "hed"}[k]] = q[k] / (rays * vol * len(zi))
    return q


_DIAG_FIELDS = ("track_length_m", "post_scatter_track_length_m", "scatter_event_weight", "scatter_event_count")
_TRAJ_FIELDS = ("trajectory_x0_m", "trajectory_y0_m", "trajectory_z0_m", "trajectory_x1_m", "trajectory_y1_m",
                "trajectory_z1_m", "trajectory_particle_order", "trajectory_event_code")


def diagnostic_integrity(diag: dict, policy: dict) -> dict:
    """Integrity report of the light-history diagnostics (`_diagnostic_integrity`, :11930-12070): shapes and
    bounds (corruption raises), field validity, event reconciliation (observed = deposited + rejected, grid
    counts = deposited), track-length closure; limited / systemic / fatal by the policy."""
    shape = (int(diag["nz"]), int(diag["ny"]), int(diag["nx"]))
    if min(shape) <= 0:
        raise ValueError("invalid diagnostic grid dimensions")
    for axis in ("x", "y", "z"):
        lo, hi = float(diag[axis + "_min_m"]), float(diag[axis + "_max_m"])
        if not np.isfinite(lo) or not np.isfinite(hi) or hi <= lo:
            raise ValueError("corrupted diagnostic grid bounds")
    if int(diag["diagnostic_rays_processed"]) <= 0:
        raise ValueError("invalid diagnostic launched-ray denominator")
    valid = {}
    for key in _DIAG_FIELDS:
        a = np.asarray(diag[key])
        if a.shape != shape:
            raise ValueError(f"corrupted diagnostic shape: {key}: {a.shape}, expected {shape}")
        valid[key] = bool(np.all(np.isfinite(a)) and np.all(a >= 0))
    counts = np.asarray(diag["trajectory_count"])
    nseg = int(diag["max_segments_per_ray"])
    if counts.ndim != 1 or np.any(counts < 0) or np.any(counts > nseg):
        raise ValueError("corrupted trajectory counts")
    if np.asarray(diag["trajectory_overflow"]).shape != counts.shape:
        raise ValueError("corrupted trajectory overflow shape")
    for key in _TRAJ_FIELDS:
        a = np.asarray(diag[key])
        if a.shape != (len(counts), nseg):
            raise ValueError(f"corrupted trajectory shape: {key}")
        valid[key] = all(np.all(np.isfinite(a[i, :int(n)])) for i, n in enumerate(counts))
    observed, deposited = int(diag["scatter_event_total"]), int(diag["deposited_scatter_event_total"])
    rejected = int(diag.get("event_outside_count", 0))
    if min(observed, deposited, rejected) < 0:
        raise ValueError("corrupted diagnostic event counts")
    discrepancy = deposited + rejected - observed
    grid_discrepancy = (int(np.sum(diag["scatter_event_count"], dtype=np.uint64)) - deposited
                        if valid["scatter_event_count"] else None)
    unexplained = max(abs(discrepancy), abs(grid_discrepancy or 0)) / max(observed, 1)
    closure, grid_closure = float(diag["deposition_closure_relative_error"]), float(diag["grid_closure_relative_error"])
    issues = []
    if rejected:
        issues.append("rejected diagnostic events explicitly accounted")
    if discrepancy or grid_discrepancy:
        issues.append("unexplained diagnostic event discrepancy")
    if int(diag.get("hard_error_count", diag.get("error_count", 0))):
        issues.append("diagnostic traversal errors")
    guard = int(diag.get("water_advance_guard_failure_count", 0))
    if guard:
        issues.append("water guard terminated rays")
    unsafe = (not all(valid.values()) or int(diag.get("nonfinite_count", 0)) > 0
              or int(diag.get("negative_value_count", 0)) > 0)
    if unsafe:
        issues.append("unsafe diagnostic fields; derived outputs skipped")
    strict_limit = policy["strict_closure_error"]
    if (not np.isfinite(closure) or not np.isfinite(grid_closure)
            or (strict_limit is not None and max(closure, grid_closure) > strict_limit)):
        issues.append("diagnostic track-length closure exceeds strict limit")
    systemic = unsafe or not np.isfinite(closure) or not np.isfinite(grid_closure)
    for value, limit in ((unexplained, policy["max_unexplained_event_fraction"]),
                         (max(closure, grid_closure), policy["max_diagnostic_closure_error"])):
        systemic = systemic or (limit is not None and value > limit)
    return {
        "policy": policy, "diagnostic_status": "limited" if issues else "ok",
        "limitations": (["failed-ray history prefixes remain in diagnostics; failed rays stay in launched "
                         "denominators"] if guard else []),
        "issues": issues, "field_validity": valid, "derived_outputs_safe": not unsafe,
        "observed_diagnostic_events": observed, "deposited_diagnostic_events": deposited,
        "rejected_diagnostic_events": rejected, "reconciled_event_discrepancy": discrepancy,
        "event_accounting_reconciled": discrepancy == 0 and grid_discrepancy == 0,
        "deposited_grid_event_discrepancy": grid_discrepancy,
        "deposited_only_event_discrepancy": deposited - observed,
        "unexplained_event_fraction": unexplained,
        "diagnostic_clipped_track_length_m": diag["segment_length_total_m"],
        "physical_full_path_length_m": None,
        "path_length_scope": "segment totals are clipped to diagnostic grid; full physical path is not collected",
        "systemic_diagnostic_issue": bool(systemic),
        "fatal": bool((policy["mode"] == "strict" and issues) or (policy["abort_on_systemic_diagnostics"] and systemic)),
        "skipped_outputs": ([] if not unsafe else ["diagnostic cross-section CSVs, volume product, trajectories and "
                                                  "diagnostic plots: unsafe fields"]),
        "first_outside_event": diag.get("first_outside_event"),
        "first_water_advance_guard_failure": diag.get("first_water_advance_guard_failure"),
    }


def json_safe(value):
    if isinstance(value, np.ndarray):
        return value.tolist()
    if isinstance(value, np.generic):
        return value.item()
    if isinstance(value, Path):
        return str(value)
    if isinstance(value, dict):
        return {str(k): json_safe(v) for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [json_safe(v) for v in value]
    if isinstance(value, float) and not np.isfinite(value):
        return None
    return value


def write_json(path, data) -> None:
    Path(path).write_text(json.dumps(json_safe(data), indent=2, sort_keys=True), encoding="utf-8")


def save_csv(path, fieldnames, rows) -> None:
    with Path(path).open("w", newline="", encoding="utf-8") as f:
        w = csv.DictWriter(f, fieldnames=list(fieldnames))
        w.writeheader()
        for row in rows:
            w.writerow({k: json_safe(row.get(k)) for k in fieldnames})


def write_detector_outputs(out, material: str, concentration: float, wavelength_nm: float, seed: int, res) -> list:
    """detector_response.csv of one case; returns its rows."""
    out = Path(out)
    score = np.asarray(res.hardware_symmetry_scores, dtype=float)
    norm = np.asarray(res.normalized_hardware_symmetry_response, dtype=float)
    jk = np.asarray(res.hardware_normalized_jackknife_se, dtype=float)
    native = np.asarray(res.hardware_native_hits, dtype=np.int64)
    mirror = np.asarray(res.hardware_mirror_hits, dtype=np.int64)
    expected = (len(DETECTOR_ANGLES_DEG),)
    if any(a.shape != expected for a in (score, norm, jk, native, mirror)):
        raise ValueError("corrupted production detector array shape")
    if any(not np.all(np.isfinite(a)) or np.any(a < 0) for a in (score, norm, native, mirror)):
        raise CaseIntegrityError("nonfinite or negative production detector field")
    order_scores = np.asarray(res.detector_particle_path_diagnostics["exact_particle_order_scores"])
    if order_scores.shape != (6, len(score)) or not np.allclose(order_scores.sum(axis=0), score, rtol=1e-12,
                                                                 atol=1e-8):
        raise CaseIntegrityError("particle interaction-order detector partition does not close")
    rows = []
    for i, angle in enumerate(DETECTOR_ANGLES_DEG):
        rows.append({
            "material": material,
            "concentration_g_L": concentration,
            "wavelength_nm": wavelength_nm,
            "seed": seed,
            "n_rays": int(res.n_rays),
            "angle_deg": float(angle),
            "absolute_score": float(score[i]),
            "particle_uninteracted_score": float(order_scores[0, i]),
            "particle_interacted_score": float(np.sum(order_scores[1:, i])),
            "absolute_score_per_launched_ray": float(score[i] / res.n_rays),
            "normalized_score": float(norm[i]),
            "native_hit_count": int(native[i]),
            "mirror_hit_count": int(mirror[i]),
            "absolute_score_sqrtN_se_approx": float(math.sqrt(max(score[i], 0.0))),
            "normalized_score_jackknife_se": float(jk[i]) if np.isfinite(jk[i]) else None,
        })
    out.mkdir(parents=True, exist_ok=True)
    save_csv(out / "detector_response.csv", rows[0].keys(), rows)
    return rows


def summary_dict(material: str, concentration: float, wavelength_nm: float, seed: int, gpu_name: str,
                 runtime_s: float, res, cfg, out, wavelength_assumptions=None) -> dict:
    """The case summary under the reference's keys (values from the result and the configuration)."""
    from . import lib
    ph = res.particle_diagnostics or {}
    total_nd = float(np.sum(np.asarray(ph.get("number_density_by_bin", []), dtype=float)))
    mu_sca, mu_ext = float(res.mu_sca_per_m), float(res.mu_ext_per_m)
    vg = vortex_surface_geometry(cfg.free_surface_model, cfg.zmean, cfg.tube_inner_radius_m,
                                 cfg.vortex_wall_center_height_difference_m, cfg.vortex_core_radius_m,
                                 cfg.gravity_m_s2)
    sensor_h = float(cfg.sensor_height_above_bottom_m)
    pd = res.detector_particle_path_diagnostics or {}
    return {
        "claritas_source_sha256": None,
        "library_version": lib.load().clr_version().decode(),
        "configuration_valid": True,
        "material": material,
        "concentration_g_L": float(concentration),
        "wavelength_nm": float(wavelength_nm),
        "n_rays": int(res.n_rays),
        "requested_n_rays": int(res.requested_n_rays),
        "seed": int(seed),
        "runtime_s": float(runtime_s),
        "gpu_device_index": 0,
        "gpu_name": gpu_name,
        "output_directory": str(out),
        "stop_reason": res.stop_reason,
        "production_failure_count": int(res.production_failure_count),
        "entered_water_fraction": float(res.entered_water_fraction),
        "air_exit_fraction": float(res.air_exit_fraction),
        "axial_loss_fraction": float(res.axial_loss_fraction),
        "detector_detection_fraction": float(res.detector_detection_fraction),
        "mean_particle_interactions": float(res.mean_interactions),
        "mean_geometric_interactions": float(res.mean_geometric_interactions),
        "mean_wave_interactions": float(res.mean_wave_interactions),
        "total_particle_number_density_m3": total_nd,
        "mu_geom_per_m": float(res.mu_geom_per_m),
        "mu_wave_per_m": float(res.mu_wave_per_m),
        "mu_event_per_m": float(res.mu_event_per_m),
        "mu_sca_per_m": mu_sca,
        "mu_ext_per_m": mu_ext,
        "mu_abs_per_m": max(mu_ext - mu_sca, 0.0),
        "single_scattering_albedo": mu_sca / mu_ext if mu_ext > 0 else None,
        "optical_depth_diameter": float(res.optical_depth_diameter),
        "geometric_optical_depth_diameter": float(res.geometric_optical_depth_diameter),
        # the reference's batch driver runs a steady-state transport model exactly when its sediment
        # distribution is "steady_state" (_resolved_sediment_config, :10080-10090)
        "sediment_distribution": "steady_state" if cfg.sediment_transport_model != "uniform" else "uniform",
        "sediment_transport_model": res.sediment_transport_model,
        "steady_state_sediment_enabled": cfg.sediment_transport_model != "uniform",
        "sediment_eddy_diffusivity_m2_s": float(res.sediment_eddy_diffusivity_m2_s),
        "sediment_particle_density_kg_m3": float(cfg.density_kg_per_m3),
        "water_density_kg_m3": float(cfg.water_density_kg_per_m3),
        "water_dynamic_viscosity_pa_s": float(cfg.water_dynamic_viscosity_pa_s),
        "gravity_m_s2": float(cfg.gravity_m_s2),
        "vortex_enabled": cfg.free_surface_model != "flat" and cfg.vortex_wall_center_height_difference_m > 0,
        "free_surface_model": cfg.free_surface_model,
        "vortex_wall_center_height_difference_m": float(cfg.vortex_wall_center_height_difference_m),
        "vortex_core_radius_m": (float(cfg.vortex_core_radius_m)
                                 if cfg.free_surface_model == "localized_scully_vortex" else None),
        "vortex_equivalent_core_rpm": (float(vg["equivalent_core_rpm"])
                                       if np.isfinite(vg["equivalent_core_rpm"]) else None),
        "vortex_equivalent_rigid_body_rpm": (float(vg["equivalent_rigid_body_rpm"])
                                             if np.isfinite(vg["equivalent_rigid_body_rpm"]) else None),
        "vortex_center_surface_height_above_bottom_m": float(vg["center_z"] + sensor_h),
        "vortex_wall_surface_height_above_bottom_m": float(vg["wall_z"] + sensor_h),
        "meridional_circulation_ratio": float(cfg.meridional_circulation_ratio),
        "sample_cell_diameter_m": 2.0 * float(cfg.tube_inner_radius_m),
        "sample_cell_height_m": float(cfg.tube_length_m),
        "water_level_m": float(cfg.water_height_m),
        "sensor_ring_height_m": sensor_h,
        "validated_geometry_baseline": None,
        "validated_sediment_baseline": None,
        "comparison_configuration_match": None,
        "parabolic_transport_validation_pass": (
            bool(int(res.production_failure_count) == 0 and np.isfinite(float(res.sediment_majorant_total_per_m)))
            if cfg.free_surface_model == "parabolic_vortex" else None),
        "particle_event_model": res.particle_event_model,
        "conditional_outcome_closure": pd.get("closure"),
        "conditional_sampler_counts": pd.get("conditional_sampler_counts"),
        "particle_surface_rms_slope_deg": float(res.particle_surface_rms_slope_deg),
        "wave_surface_rms_height_nm": float(res.wave_surface_rms_height_nm),
        "wavelength_assumptions": wavelength_assumptions,
    }


def write_run_summary(out, material: str, concentration: float, wavelength_nm: float, seed: int, gpu_name: str,
                      runtime_s: float, res, cfg, wavelength_assumptions=None) -> dict:
    """run_summary.json of one case; returns the dict written."""
    out = Path(out)
    out.mkdir(parents=True, exist_ok=True)
    d = summary_dict(material, concentration, wavelength_nm, seed, gpu_name, runtime_s, res, cfg, out,
                     wavelength_assumptions)
    if hasattr(res, "production_failure_diagnostics"):
        d["production_integrity"], d["light_transport_diagnostics"] = case_integrity(res)
    write_json(out / "run_summary.json", d)
    return d
