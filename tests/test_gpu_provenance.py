"""GPU: particle-event provenance of detected rays (first/last bin, event type and deflection, acrylic returns).

The reference keeps per ray the provenance of its particle events and its host partitions the detected rays
by it (CLARITAS/CLARITAS.py:4625-4647, :4966-4979, :8063-8160, :8470-8481). The library counts the same
partitions on the device. Three checks, on the reference's xorshift streams:
  * the device partitions equal the partitions of the device's own per-ray provenance and records (the
    counting is exact);
  * per ray, the provenance equals the reference's (its own code built for the host,
    tests/golden/provenance_fixtures.npz) on every ray whose path agrees -- the host build uses the host's
    libm, so a small fraction of paths differ from the device's;
  * the partitions of whole runs agree with the reference's within those few differing rays.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import parity_scenes as PS
import provenance_partitions as PP
from tardiis_and_claritas_gb300 import abi, scene as S

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "provenance_fixtures.npz")
INT_KEYS = ("bin_hits", "first_type_hits", "last_type_hits", "wall_hits", "after_return_hits",
            "first_backscatter_hits", "first_source_hemisphere_hits", "first_angle_count", "last_angle_count",
            "last_type_angle_count", "h170_last_angle_hits", "h170_first_angle_hits")


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def gold():
    z = np.load(GOLD)
    return z, json.loads(bytes(z["meta"]).decode())


def run(ctx, name, n):
    cfg, parts, grid = PS.build(name)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid))
    ctx.set_provenance(True)
    try:
        tal, rec = ctx.trace(S.run_params(n, seed=PS.seed_of(name)), records=True)
        part = ctx.read_provenance()
        prov, defl = ctx.read_provenance_records(n)
    finally:
        ctx.set_provenance(False)
    return tal, rec, part, prov, defl


@pytest.mark.parametrize("name", ["rough_spheroid", "c1_smooth_coherent", "hybrid_excess", "absorbing_conditional",
                                  "reflective_bores", "scully_surface"])
def test_provenance_partitions(ctx, gold, name):
    z, meta = gold
    n = meta["n_rays"]
    tal, rec, part, prov, defl = run(ctx, name, n)
    # 1. the device partitions are those of its own per-ray provenance
    mine = PP.partitions(rec["interaction_count"], rec["native_id"], rec["mirror_id"], prov, defl)
    for k in INT_KEYS:
        np.testing.assert_array_equal(part[k], mine[k], err_msg=f"{name}: {k}")
    for k in ("first_angle_sum", "last_angle_sum", "last_type_angle_sum"):
        np.testing.assert_allclose(part[k], mine[k], rtol=1e-9, atol=1e-9, err_msg=f"{name}: {k}")
    # closures of the reference's partitions: every detected ray with a particle event has one first and one
    # last bin and type; every detected ray one wall-path class
    det = np.stack([tal["hw_native"], tal["hw_mirror"]])
    anyp = tal["path_mask_hits"][:, abi.PATH_MASK_NAMES.index("any_particle")]
    np.testing.assert_array_equal(part["bin_hits"][0].sum(axis=1), anyp)
    np.testing.assert_array_equal(part["bin_hits"][1].sum(axis=1), anyp)
    np.testing.assert_array_equal(part["last_type_hits"].sum(axis=1), anyp)
    np.testing.assert_array_equal(part["wall_hits"].sum(axis=1), det)
    assert anyp.sum() > 0
    # 3. whole-run partitions against the reference's: the differences stay within the few rays whose path
    # differs between the host's libm and the device's math
    agree = np.array_equal(tal["hw_native"], z[f"{name}/hw_native"])
    n_det = int(det.sum())
    for k in INT_KEYS:
        d = np.abs(part[k] - z[f"{name}/{k}"]).sum()
        assert d <= 0.01 * max(int(z[f"{name}/{k}"].sum()), 1) + 20, (name, k, d, agree, n_det)


@pytest.mark.parametrize("name", ["rough_spheroid", "hybrid_excess", "absorbing_conditional"])
def test_provenance_per_ray_equals_reference(ctx, gold, name):
    """2. per ray: equal to the reference's on every ray whose path (status, counters, detector ids) agrees."""
    z, meta = gold
    n = meta["n_per_ray"]
    _, rec, _, prov, defl = run(ctx, name, n)
    keys = np.stack([rec[k] for k in meta["keys"]], axis=1).astype(np.int16)
    same = np.all(keys == z[f"{name}/ray_keys"], axis=1)
    assert same.mean() >= 0.99, same.mean()
    want = z[f"{name}/ray_prov"].astype(np.int32)
    got = prov.copy()
    cols = [c for c in range(13) if c != PP.LAST_ORDER]  # the device does not keep the last event's order
    np.testing.assert_array_equal(got[same][:, cols], want[same][:, cols], err_msg=name)
    # deflections: the directions agree to a few ulp between the host's libm and the device's math, and near
    # forward scattering acos turns one ulp of cos (6e-8) into ~0.02 deg
    wd = z[f"{name}/ray_defl"]
    np.testing.assert_allclose(defl[same], wd[same], rtol=1e-5, atol=0.05, err_msg=name)
    assert np.mean(np.abs(defl[same] - wd[same])) < 1e-3
    assert (want[same][:, PP.LAST_TYPE] > 0).sum() > 500  # enough rays with particle events


def test_provenance_needs_the_wavefront_engine(ctx):
    cfg, parts, grid = PS.build("rough_spheroid")
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid))
    ctx.set_provenance(True)
    try:
        with pytest.raises(RuntimeError, match="wavefront"):
            ctx.trace(S.run_params(1000, flags=abi.RUN_PERSISTENT_KERNEL))
    finally:
        ctx.set_provenance(False)
    with pytest.raises(RuntimeError, match="provenance is off"):
        ctx.read_provenance()
