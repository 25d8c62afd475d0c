"""CPU: the per-case writers against the reference's own writers, on the golden results in output_fixtures.json.

``tests/golden/make_output_fixtures.py`` ran the reference's ``_write_detector_outputs``
(CLARITAS/CLARITAS.py:12653-12696) and ``_summary_dict`` (:12849-12971) on seeded synthetic results. Here
``outputs.write_detector_outputs`` must write the same detector_response.csv byte for byte and raise the
same errors on the corrupted results, and ``outputs.summary_dict``, given the model configuration the
reference's batch driver builds (``_resolve_model_kwargs``), must carry every key of the reference's
summary with the same value, except the keys that describe the reference script's own environment.
"""
from __future__ import annotations

import json
import math
import os
import sys

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import outputs as O, scene as S

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_output_fixtures as G  # noqa: E402

FIX = json.load(open(os.path.join(HERE, "golden", "output_fixtures.json")))["cases"]
# keys whose reference value describes its own script and machine, not the case: the digest of its source
# file, the output folder, its comparison-baseline flags (this library reports None for those)
ENVIRONMENT_KEYS = {"claritas_source_sha256", "output_directory", "validated_geometry_baseline",
                    "validated_sediment_baseline", "comparison_configuration_match"}


@pytest.mark.parametrize("case", range(len(FIX)))
def test_detector_csv_is_the_reference_csv(case, tmp_path):
    c = FIX[case]
    O.write_detector_outputs(tmp_path, *c["args"], G.as_result(c["result"]))
    assert (tmp_path / "detector_response.csv").read_text(encoding="utf-8") == c["csv"]


@pytest.mark.parametrize("case", range(len(FIX)))
def test_corrupted_results_raise_the_reference_errors(case, tmp_path):
    c = FIX[case]
    for name, corrupt in G.CORRUPTIONS.items():
        bad = json.loads(json.dumps(c["result"]))
        corrupt(bad)
        want = c["errors"][name]
        with pytest.raises(Exception) as ei:
            O.write_detector_outputs(tmp_path, *c["args"], G.as_result(bad))
        assert [type(ei.value).__name__, str(ei.value)] == want, name


def _same(a, b) -> bool:
    if isinstance(a, float) or isinstance(b, float):
        if a is None or b is None:
            return a is b
        return math.isclose(float(a), float(b), rel_tol=1e-12, abs_tol=1e-15)
    if isinstance(a, dict) and isinstance(b, dict):
        return a.keys() == b.keys() and all(_same(a[k], b[k]) for k in a)
    if isinstance(a, list) and isinstance(b, list):
        return len(a) == len(b) and all(_same(x, y) for x, y in zip(a, b))
    return a == b


@pytest.mark.parametrize("case", range(len(FIX)))
def test_summary_carries_the_reference_keys_and_values(case, tmp_path):
    c = FIX[case]
    material, conc, wl, seed = c["args"]
    cfg = S.ModelConfig(**c["model_kwargs"])
    ours = O.json_safe(O.summary_dict(material, conc, wl, seed, "GB300-test", 12.5, G.as_result(c["result"]), cfg,
                                      tmp_path, wavelength_assumptions={"assumed": "test"}))
    ref = c["summary"]
    missing = sorted(set(ref) - set(ours))
    assert not missing, f"keys of the reference's summary missing: {missing}"
    wrong = {k: (ours[k], ref[k]) for k in ref if k not in ENVIRONMENT_KEYS and not _same(ours[k], ref[k])}
    assert not wrong, wrong
    assert np.isfinite(ours["vortex_wall_surface_height_above_bottom_m"])
