"""CPU checks of the provenance path: the decoding of the device's per-ray provenance words, the partitions
restated from the reference's host code, and the golden fixture made by the reference's own code."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

import oracle_harness as H
import parity_scenes as PS
import provenance_partitions as PP
from tardiis_and_claritas_gb300 import lib as L, scene as S

GOLD = os.path.join(os.path.dirname(__file__), "golden", "provenance_fixtures.npz")


def test_decode_provenance_words():
    import struct
    f = lambda v: struct.unpack("<I", struct.pack("<f", v))[0]  # noqa: E731
    raw = np.array([
        [0xFFFFFFFF, 0x0000FFFF, f(-1.0), f(-1.0)],                                  # no event
        [0x03FF0503, (2 << 20) | (4 << 16) | 0x0503 | (1 << 24) | (1 << 26) | (1 << 27), f(12.5), f(170.0)],
    ], np.uint32)
    prov, defl = L.decode_provenance(raw)
    assert prov[0].tolist() == [0, 0, -1, 0, 0, -1, -1, -1, -1, -1, -1, 0, 0]
    #             first type, last type, order, back, hemi, first/last p, first/last g, first/last w, ret, after
    assert prov[1].tolist() == [4, 2, -1, 1, 0, 3, 5, -1, 3, 3, 5, 1, 1]
    np.testing.assert_array_equal(defl, np.array([[-1.0, -1.0], [12.5, 170.0]], np.float32))


def test_fixture_partitions_close():
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]).decode())
    for name in meta["scenes"]:
        det = np.stack([z[f"{name}/hw_native"], z[f"{name}/hw_mirror"]])
        np.testing.assert_array_equal(z[f"{name}/wall_hits"].sum(axis=1), det)
        anyp = det - z[f"{name}/wall_hits"][:, 0]
        for k in (0, 1):  # first and last particle bin
            np.testing.assert_array_equal(z[f"{name}/bin_hits"][k].sum(axis=1), anyp)
        np.testing.assert_array_equal(z[f"{name}/last_type_hits"].sum(axis=1), anyp)
        np.testing.assert_array_equal(z[f"{name}/first_type_hits"].sum(axis=1), anyp)
        # rays with a geometric event have one first and one last geometric bin (likewise wave)
        for first, last in ((2, 3), (4, 5)):
            np.testing.assert_array_equal(z[f"{name}/bin_hits"][first].sum(axis=1),
                                          z[f"{name}/bin_hits"][last].sum(axis=1))
        assert anyp.sum() > 0


@pytest.mark.skipif(not H.reference_available(), reason="host build of the reference not present (no checkout)")
def test_fixture_regenerates_from_the_reference():
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]).decode())
    name = "absorbing_conditional"
    cfg, parts, grid = PS.build(name)
    ref = H.OracleRun("reference", cfg, parts, grid=grid)
    tal, rec, prov, defl = ref.trace_provenance(S.run_params(meta["n_rays"], seed=PS.seed_of(name)))
    ref.close()
    part = PP.partitions(rec["interaction_count"], rec["native_id"], rec["mirror_id"], prov, defl)
    for k, v in part.items():
        np.testing.assert_allclose(v, z[f"{name}/{k}"], rtol=1e-12, err_msg=k)


@pytest.mark.parametrize("name", ["rough_spheroid", "absorbing_conditional", "reflective_bores"])
def test_oracle_provenance_matches_reference_fixture(name):
    """The C restatement's per-ray provenance (oracle/claritas_oracle.c, o_prov_mark and the event and
    return sites) partitions the detected rays as the reference's own code does: exactly on the platform
    the fixture was made on, per ray on the kept rays."""
    import platform
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]).decode())
    cfg, parts, grid = PS.build(name)
    orc = H.OracleRun("port", cfg, parts, grid=grid)
    tal, rec, prov, defl = orc.trace_provenance(S.run_params(meta["n_rays"], seed=PS.seed_of(name)))
    orc.close()
    part = PP.partitions(rec["interaction_count"], rec["native_id"], rec["mirror_id"], prov, defl)
    same_platform = platform.machine() == meta["machine"]
    for k, v in part.items():
        if same_platform:
            np.testing.assert_allclose(v, z[f"{name}/{k}"], rtol=1e-12, atol=0, err_msg=k)
        else:
            assert np.abs(v - z[f"{name}/{k}"]).sum() <= 0.01 * max(float(np.abs(z[f"{name}/{k}"]).sum()), 1.0) + 20
    if name in meta["per_ray"]:
        n = meta["n_per_ray"]
        keys = np.stack([rec[k][:n] for k in meta["keys"]], axis=1).astype(np.int16)
        same = np.all(keys == z[f"{name}/ray_keys"], axis=1)
        rp = prov[:n].copy()
        rp[:, PP.ACR_RETURN] = rp[:, PP.ACR_RETURN] > 0
        rp[:, PP.AFTER_RETURN] = rp[:, PP.AFTER_RETURN] > 0
        rp = np.clip(rp, -1, 127)
        np.testing.assert_array_equal(rp[same], z[f"{name}/ray_prov"][same].astype(np.int32))
        if same_platform:
            assert same.all()
            np.testing.assert_array_equal(defl[:n, :2], z[f"{name}/ray_defl"])
            np.testing.assert_array_equal(defl[:n, 2:], z[f"{name}/ray_paths"])


@pytest.mark.skipif(not H.reference_available(), reason="host build of the reference not present (no checkout)")
def test_oracle_provenance_matches_live_reference():
    cfg, parts, grid = PS.build("hybrid_excess")
    run = S.run_params(40000, seed=11, ray_offset=777)
    a = H.OracleRun("port", cfg, parts, grid=grid)
    b = H.OracleRun("reference", cfg, parts, grid=grid)
    _, ra, pa, da = a.trace_provenance(run)
    _, rb, pb, db = b.trace_provenance(run)
    assert PS.records_digest(ra) == PS.records_digest(rb)
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(da, db)
