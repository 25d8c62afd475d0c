"""GPU: the device partitions of detected rays (particle-path diagnostics) and the per-case output files.

The reference derives its particle-path diagnostics on the host from per-ray arrays
(CLARITAS/CLARITAS.py:8019-8110). The library counts the same partitions on the device; with the reference's
streams its per-ray records are the reference's, so the partitions recomputed from those records with the
reference's definitions must equal the device counts exactly.
"""
from __future__ import annotations

import csv
import json

import numpy as np
import pytest

import parity_scenes as PS
from path_partitions import partitions_from_records
from tardiis_and_claritas_gb300 import abi, forward as F, outputs as O, scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", ["rough_spheroid", "c1_smooth_coherent", "meridional_solver"])
def test_device_partitions_equal_record_partitions(ctx, name):
    cfg, parts, grid = PS.build(name)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid))
    tal, rec = ctx.trace(S.run_params(200_000, seed=PS.seed_of(name)), records=True)
    order, gorder, sums, masks, acr = partitions_from_records(rec)
    np.testing.assert_array_equal(tal["order_hits"], order)
    np.testing.assert_array_equal(tal["geometric_order_hits"], gorder)
    np.testing.assert_array_equal(tal["path_sums"], sums)
    np.testing.assert_array_equal(tal["path_mask_hits"], masks)
    np.testing.assert_array_equal(tal["acrylic_order_hits"], acr)
    assert tal["path_mask_hits"][:, abi.PATH_MASK_NAMES.index("any_particle")].sum() > 0
    # every detected ray is in exactly one order class
    np.testing.assert_array_equal(tal["order_hits"].sum(axis=1), np.stack([tal["hw_native"], tal["hw_mirror"]]))
    assert tal["order_hits"].sum() > 0


def test_case_outputs_from_a_forward_result(ctx, tmp_path):
    kw = {k: v for k, v in S.small_cell_config().__dict__.items() if k not in ("source_kind", "disc_beam_radius_m")}
    kw["statistics_batch_rays"] = 50_000
    m = F.ClaritasForwardModel(**kw)
    m.register_material("quartz", S.quartz_particles(1.0, n_bins=32))
    res = m.simulate("quartz", 1.0, n_rays=200_000, seed=3)
    pd = res.detector_particle_path_diagnostics
    np.testing.assert_allclose(pd["exact_particle_order_scores"].sum(axis=0), res.hardware_symmetry_scores)
    assert np.all(pd["exact_particle_order_partition_closure_error_scores"] == 0.0)
    # the reference's closure checks of the event-history and acrylic-order partitions
    for key in ("interaction_order", "multiple_branch", "acrylic_reflection_order"):
        assert np.all(pd[key + "_partition_closure_error_scores"] == 0.0), key
    np.testing.assert_allclose(pd["ballistic_scores"] + pd["any_particle_scores"], res.hardware_symmetry_scores)
    # the provenance partitions close too (first/last bin, first/last event type, wall paths)
    for key in ("first_particle_bin", "last_particle_bin", "causal_last_event", "causal_first_event", "wall_path"):
        assert np.all(pd[key + "_partition_closure_error_scores"] == 0.0), key
    assert pd["first_particle_bin_scores"].shape == (32, 18)
    rows = O.write_detector_outputs(tmp_path, "quartz", 1.0, 860.0, 3, res)
    with open(tmp_path / "detector_response.csv") as f:
        got = list(csv.DictReader(f))
    assert len(got) == 18 and list(got[0].keys()) == list(rows[0].keys())
    assert float(got[0]["absolute_score"]) == pytest.approx(res.hardware_symmetry_scores[0])
    d = O.write_run_summary(tmp_path, "quartz", 1.0, 860.0, 3, "GB300", 1.0, res, m.config)
    back = json.loads((tmp_path / "run_summary.json").read_text())
    assert back["n_rays"] == 200_000 and back["conditional_sampler_counts"] == d["conditional_sampler_counts"]
    m.close()
