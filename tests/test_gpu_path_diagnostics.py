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
from tardiis_and_claritas_gb300 import abi, forward as F, outputs as O, scene as S

pytestmark = pytest.mark.gpu

SUM_FIELDS = ("interaction_count", "geometric", "wave", "coherent", "morphology", "entry_reflections",
              "internal_reflections")


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.close()


def history_masks(rec):
    """The reference's event-history masks (CLARITAS/CLARITAS.py:5265-5321) over the per-ray records."""
    ic, g, w = rec["interaction_count"], rec["geometric"], rec["wave"]
    coh, mor = rec["coherent"], rec["morphology"]
    per, pir, pabs = rec["entry_reflections"], rec["internal_reflections"], rec["absorptions"]
    single, multiple, surface = ic == 1, ic >= 2, (g > 0) | (mor > 0)
    m = {
        "any_particle": ic > 0, "any_geometric": g > 0, "any_wave": w > 0, "any_coherent_wave": coh > 0,
        "any_morphology_wave": mor > 0, "any_entry_reflection": per > 0, "any_internal_reflection": pir > 0,
        "ballistic": ic == 0, "single_interaction": single, "single_entry_reflection": single & (per > 0),
        "multiple_interaction": multiple, "interaction_order_2": ic == 2, "interaction_order_3": ic == 3,
        "interaction_order_4plus": ic >= 4, "exactly_one_geometric": single & (g == 1) & (w == 0),
        "exactly_one_wave": single & (g == 0) & (w == 1), "single_coherent_wave_escape": single & (coh == 1),
        "single_external_entry_reflection_escape": single & (per > 0),
        "single_internal_reflection_escape": single & (pir > 0),
        "single_surface_transmission_escape": single & surface & (per == 0) & (pir == 0) & (pabs == 0),
        "mixed_geometric_wave": multiple & (g > 0) & (w > 0),
        "geometric_only_multiple": multiple & (g > 0) & (w == 0),
        "wave_only_multiple": multiple & (g == 0) & (w > 0),
        "multiple_with_entry_reflection": multiple & (per > 0),
        "multiple_with_internal_reflection": multiple & (pir > 0),
    }
    return [m[k] for k in abi.PATH_MASK_NAMES]


def partitions_from_records(rec):
    order = np.zeros((2, 6, 18), np.int64)
    gorder = np.zeros((2, 6, 18), np.int64)
    sums = np.zeros((len(SUM_FIELDS), 2, 18), np.int64)
    masks = np.zeros((2, abi.N_PATH_MASKS, 18), np.int64)
    acr = np.zeros((2, 5, 18), np.int64)
    oi = np.minimum(rec["interaction_count"], 5)
    gi = np.minimum(rec["geometric"], 5)
    ai = np.minimum(rec["cell_inner_reflections"] + rec["cell_outer_reflections"]
                    + rec["bottom_inner_reflections"] + rec["bottom_outer_reflections"], 4)
    hm = history_masks(rec)
    for side, key in ((0, "native_id"), (1, "mirror_id")):
        ids = rec[key]
        ok = (ids >= 0) & (ids < 18)
        np.add.at(order[side], (oi[ok], ids[ok]), 1)
        np.add.at(gorder[side], (gi[ok], ids[ok]), 1)
        np.add.at(acr[side], (ai[ok], ids[ok]), 1)
        for k, f in enumerate(SUM_FIELDS):
            np.add.at(sums[k, side], ids[ok], rec[f][ok].astype(np.int64))
        for k, mk in enumerate(hm):
            np.add.at(masks[side, k], ids[ok & mk], 1)
    return order, gorder, sums, masks, acr


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
