"""CPU tests of the forward-model facade: restated reference helpers against golden vectors made
by the reference's own functions (tests/golden/make_forward_fixtures.py), configuration handling,
and explicit rejection of features outside the library."""
from __future__ import annotations

import os

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import forward as F, scene as S

GOLD = os.path.join(os.path.dirname(__file__), "golden", "forward_fixtures.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("case", range(5))
def test_jackknife_matches_reference(gold, case):
    got = F.jackknife_normalized_se(list(gold[f"jk_in_{case}"]))
    np.testing.assert_allclose(got, gold[f"jk_out_{case}"], rtol=1e-12, atol=0, equal_nan=True)


@pytest.mark.parametrize("case", range(6))
def test_histogram_median_matches_reference(gold, case):
    got = F.histogram_median(gold[f"med_in_{case}"])
    want = float(gold[f"med_out_{case}"])
    assert (np.isnan(got) and np.isnan(want)) or got == want


def test_model_takes_reference_keywords_and_validates():
    m = F.ClaritasForwardModel(particle_event_model="geometric", symmetry_average_exact=False)
    assert m.particle_event_model == "geometric" and m.symmetry_average_exact is False
    with pytest.raises(ValueError):
        F.ClaritasForwardModel(legacy_detector_acceptance_deg=95.0)
    with pytest.raises(ValueError):
        F.ClaritasForwardModel(rng="mersenne")


def test_unsupported_features_raise_explicitly():
    m = F.ClaritasForwardModel()
    parts = S.quartz_particles(100.0, n_bins=4)
    # light diagnostics are validated with the reference's rules before anything reaches the device
    with pytest.raises(ValueError, match="max_rays must be >=1"):
        m.simulate(parts, 0.1, n_rays=10, light_transport_config={"enabled": True, "nx": 8, "ny": 8, "nz": 8})
    with pytest.raises(ValueError, match="grid dimensions"):
        m.simulate(parts, 0.1, n_rays=10, light_transport_config={"enabled": True, "max_rays": 5, "nx": 3})
    with pytest.raises(ValueError, match="representative-ray"):
        m.simulate(parts, 0.1, n_rays=10, light_transport_config={"enabled": True, "max_rays": 5, "nx": 4, "ny": 4,
                                                                 "nz": 4})
    with pytest.raises(ValueError, match="heatmap_size"):
        m.simulate(parts, 0.1, n_rays=10, heatmap_size=-1)
    with pytest.raises(NotImplementedError):
        m.simulate(parts, 0.1, n_rays=10, collect_rays=True)
    with pytest.raises(NotImplementedError, match="named PSD tables"):
        m.simulate("loess", 0.1, n_rays=10)
    with pytest.raises(ValueError, match="ray_id_start"):
        m.simulate(parts, 0.1, n_rays=10, ray_id_start=2 ** 32)


def test_registered_material_takes_weights_on_its_grid():
    m = F.ClaritasForwardModel()
    parts = S.quartz_particles(100.0, n_bins=5)
    m.register_material("sand", parts)
    p = m._particles("sand", 0.5, [1, 2, 3, 4, 5], "number_fraction")
    assert p.concentration_kg_m3 == 0.5 and p.weight_mode == "number_fraction"
    np.testing.assert_array_equal(p.weight, [1, 2, 3, 4, 5])
    with pytest.raises(ValueError, match="weights must have 5 entries"):
        m._particles("sand", 0.5, [1, 2], "mass_fraction")
