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
