"""CPU: the per-case output writers (the reference's column set, integrity checks and JSON sanitiser)."""
from __future__ import annotations

import csv
import json
import types

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import outputs as O


def fake_result(n=1000):
    rng = np.random.default_rng(0)
    nat = rng.integers(0, 50, 18)
    mir = rng.integers(0, 50, 18)
    sym = 0.5 * (nat + mir)
    order = np.zeros((6, 18))
    order[0] = 0.25 * sym
    order[1] = 0.5 * sym
    order[5] = 0.25 * sym
    return types.SimpleNamespace(hardware_symmetry_scores=sym, normalized_hardware_symmetry_response=sym / sym.sum(),
                                 hardware_normalized_jackknife_se=np.full(18, np.nan), hardware_native_hits=nat,
                                 hardware_mirror_hits=mir, n_rays=n,
                                 detector_particle_path_diagnostics={"exact_particle_order_scores": order})


def test_detector_csv_columns_and_values(tmp_path):
    res = fake_result()
    rows = O.write_detector_outputs(tmp_path, "quartz", 0.5, 860.0, 7, res)
    with open(tmp_path / "detector_response.csv") as f:
        got = list(csv.DictReader(f))
    assert list(got[0].keys()) == ["material", "concentration_g_L", "wavelength_nm", "seed", "n_rays", "angle_deg",
                                   "absolute_score", "particle_uninteracted_score", "particle_interacted_score",
                                   "absolute_score_per_launched_ray", "normalized_score", "native_hit_count",
                                   "mirror_hit_count", "absolute_score_sqrtN_se_approx",
                                   "normalized_score_jackknife_se"]
    assert [float(r["angle_deg"]) for r in got] == [10.0 * i for i in range(18)]
    assert got[3]["normalized_score_jackknife_se"] == ""           # NaN -> None -> empty field
    assert float(got[3]["particle_uninteracted_score"]) == pytest.approx(rows[3]["absolute_score"] * 0.25)


def test_detector_csv_integrity_checks(tmp_path):
    res = fake_result()
    res.detector_particle_path_diagnostics["exact_particle_order_scores"][2, 4] += 1.0
    with pytest.raises(O.CaseIntegrityError, match="does not close"):
        O.write_detector_outputs(tmp_path, "quartz", 0.5, 860.0, 7, res)
    res = fake_result()
    res.hardware_native_hits = res.hardware_native_hits[:5]
    with pytest.raises(ValueError, match="shape"):
        O.write_detector_outputs(tmp_path, "quartz", 0.5, 860.0, 7, res)


def test_json_safe_rules(tmp_path):
    O.write_json(tmp_path / "x.json", {"a": np.arange(3), "b": np.float64(2.5), "c": float("nan"), "d": (1, 2),
                                       "z": {"k": np.int32(4)}})
    txt = (tmp_path / "x.json").read_text()
    assert json.loads(txt) == {"a": [0, 1, 2], "b": 2.5, "c": None, "d": [1, 2], "z": {"k": 4}}
    assert txt.index('"a"') < txt.index('"z"')  # sorted keys


# ---- case-integrity policy (the reference's PolicyTests, CLARITAS/test_diagnostics.py) ----

def _diag_fixture():
    """A light-diagnostic result of a 2x2x2 grid: 9 observed events, 8 deposited, 1 outside the grid."""
    a = np.ones((2, 2, 2), dtype=np.float32)
    d = dict(nx=2, ny=2, nz=2, track_length_m=a, post_scatter_track_length_m=a.copy(), scatter_event_weight=a.copy(),
             scatter_event_count=a.astype(np.uint32), scatter_event_total=9, deposited_scatter_event_total=8,
             event_outside_count=1, deposition_closure_relative_error=1e-12, grid_closure_relative_error=1e-12,
             segment_length_total_m=8.0, deposited_length_total_m=8.0, trajectory_count=np.zeros(0, dtype=int),
             trajectory_overflow=np.zeros(0, dtype=int), max_segments_per_ray=4, nonfinite_count=0,
             negative_value_count=0, hard_error_count=1, water_advance_guard_failure_count=1,
             diagnostic_rays_processed=100)
    for k in O._TRAJ_FIELDS:
        d[k] = np.zeros((0, 4))
    for k in ("x", "y", "z"):
        d[k + "_min_m"], d[k + "_max_m"] = -0.049, 0.049
    return d


def test_one_failure_keeps_launched_denominator():
    p = O.production_integrity(100_000_000, 1, {"count_closure_ok": True, "code_counts": {"water_guard": 1}},
                               O.resolved_failure_policy())
    O.enforce_case_integrity(p, O.diagnostic_integrity(_diag_fixture(), O.resolved_failure_policy()))
    assert not p["fatal"] and p["normalization_rays"] == 100_000_000 and p["failed_ray_fraction"] == 1e-8
    assert p["status"] == "limited"


def test_rejected_events_reconcile():
    r = O.diagnostic_integrity(_diag_fixture(), O.resolved_failure_policy())
    assert r["reconciled_event_discrepancy"] == 0 and r["deposited_only_event_discrepancy"] == -1
    assert not r["fatal"] and r["diagnostic_status"] == "limited"


def test_unexplained_discrepancy_visible():
    d = _diag_fixture()
    d["event_outside_count"] = 0
    r = O.diagnostic_integrity(d, O.resolved_failure_policy())
    assert r["reconciled_event_discrepancy"] == -1 and not r["event_accounting_reconciled"] and not r["fatal"]
    p = O.resolved_failure_policy()
    p["abort_on_systemic_diagnostics"] = True
    assert O.diagnostic_integrity(d, p)["fatal"]


def test_strict_reports_then_stops():
    p = O.resolved_failure_policy(mode="strict")
    assert O.diagnostic_integrity(_diag_fixture(), p)["fatal"]
    with pytest.raises(O.CaseIntegrityError):
        O.enforce_case_integrity({"fatal": False}, O.diagnostic_integrity(_diag_fixture(), p))
    d = _diag_fixture()
    d.update(scatter_event_total=8, event_outside_count=0, hard_error_count=0, water_advance_guard_failure_count=0)
    assert not O.diagnostic_integrity(d, p)["fatal"]
    d["grid_closure_relative_error"] = 0.01
    assert O.diagnostic_integrity(d, p)["fatal"]


def test_unsafe_fields_are_reported():
    d = _diag_fixture()
    d["track_length_m"][0, 0, 0] = np.nan
    r = O.diagnostic_integrity(d, O.resolved_failure_policy())
    assert not r["derived_outputs_safe"] and r["skipped_outputs"] and not r["fatal"]
    assert not r["field_validity"]["track_length_m"] and r["field_validity"]["scatter_event_count"]


def test_shapes_and_counts_unrecoverable():
    d = _diag_fixture()
    d["track_length_m"] = np.zeros((1,))
    with pytest.raises(ValueError):
        O.diagnostic_integrity(d, O.resolved_failure_policy())
    with pytest.raises(ValueError):
        O.production_integrity(10, 1, {"count_closure_ok": False}, O.resolved_failure_policy())
    with pytest.raises(ValueError):
        O.resolved_failure_policy(mode="invalid")
    with pytest.raises(ValueError):
        O.resolved_failure_policy(max_failed_ray_fraction=-1.0)


def test_systemic_ray_limit():
    p = O.resolved_failure_policy()
    assert O.production_integrity(100, 2, {}, p)["fatal"]
    p["max_failed_ray_fraction"] = None
    assert not O.production_integrity(100, 2, {}, p)["fatal"]


def test_case_integrity_reports(tmp_path):
    res = fake_result(n=200_000)
    res.production_failure_count = 3
    res.production_failure_diagnostics = {"code_counts": {"acrylic_bounce_limit": 3}, "subcode_counts": {}}
    res.light_transport_diagnostics = None
    prod, diag = O.write_case_integrity(tmp_path, res)
    assert prod["failed_ray_fraction"] == 1.5e-5 and prod["status"] == "limited" and not prod["fatal"]
    assert diag["diagnostic_status"] == "disabled"
    back = json.loads((tmp_path / "production_integrity_report.json").read_text())
    assert back["failure_categories"] == {"acrylic_bounce_limit": 3}
    assert not (tmp_path / "light_transport_integrity_report.json").exists()
    O.enforce_case_integrity(prod, diag)
    res.light_transport_diagnostics = _diag_fixture()
    res.production_failure_count = 1000  # 0.5 % > 0.1 %: the case is exported, then stops
    prod, diag = O.write_case_integrity(tmp_path, res)
    assert prod["fatal"] and diag["diagnostic_status"] == "limited"
    assert (tmp_path / "light_transport_integrity_report.json").exists()
    with pytest.raises(O.CaseIntegrityError):
        O.enforce_case_integrity(prod, diag)


def test_light_transport_cross_sections():
    """The sections use every launched diagnostic history as denominator (the reference's check in
    test_one_failure_keeps_launched_denominator) and pick the slabs around the axes."""
    d = _diag_fixture()
    rng = np.random.default_rng(3)
    d.update(nx=6, ny=4, nz=5)
    for k in O._DIAG_FIELDS:
        d[k] = rng.uniform(0, 1, (5, 4, 6)).astype(np.float32)
    q = O.light_transport_cross_sections(d, {"vertical_slice_thickness_m": 0.049, "sensor_slice_thickness_m": 0.049})
    np.testing.assert_allclose(q["vd"], q["vr"] / (100 * q["dx"] * q["dy"] * q["dz"] * len(q["xi"])))
    np.testing.assert_allclose(q["hed"], q["he"] / (100 * q["voxel_volume"] * len(q["zi"])))
    assert q["vr"].shape == (5, 4) and q["hr"].shape == (4, 6)
    np.testing.assert_array_equal(q["xi"], np.flatnonzero(np.abs(q["x"]) <= 0.0245))
    thin = O.light_transport_cross_sections(d, {"vertical_slice_thickness_m": 1e-9, "sensor_slice_thickness_m": 1e-9})
    assert len(thin["xi"]) == 1 and len(thin["zi"]) == 1
    np.testing.assert_allclose(q["x"][0], -0.049 + 0.098 / 12)
