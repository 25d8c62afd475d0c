"""CPU tests of the oracle (our C restatement) against the reference's own code.

The golden file tests/golden/cpu_ref_fixtures.npz was produced by the
reference's CUDA_SRC compiled for the host (tests/golden/make_cpu_fixtures.py).
The restatement must reproduce it bit for bit on the platform it was made on:
every per-ray record (digest), every physics table (digest) and every tally.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import platform

import numpy as np
import pytest

import oracle_harness as H
import parity_scenes as PS
from tardiis_and_claritas_gb300 import scene as S

GOLD = os.path.join(os.path.dirname(__file__), "golden", "cpu_ref_fixtures.npz")


@pytest.fixture(scope="module")
def gold():
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


def test_erfinv_matches_scipy():
    special = pytest.importorskip("scipy.special")
    lib, _ = H.load("port")
    ys = np.concatenate([np.linspace(-0.999999, 0.999999, 2001), [1e-300, -1e-12, 0.5, 0.9999999999, -0.9999999999]])
    got = np.array([lib.clo_erfinv(float(y)) for y in ys])
    want = special.erfinv(ys)
    assert np.allclose(got, want, rtol=4e-15, atol=1e-300)


def test_philox_known_answers():
    """Published Philox4x32-10 test vectors (Random123 distribution, kat_vectors)."""
    lib, _ = H.load("port")

    def kat(key, ctr):
        k = (C.c_uint32 * 2)(*key)
        c = (C.c_uint32 * 4)(*ctr)
        o = (C.c_uint32 * 4)()
        lib.clo_philox4x32_10(k, c, o)
        return list(o)

    assert kat([0, 0], [0, 0, 0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert kat([0xFFFFFFFF] * 2, [0xFFFFFFFF] * 4) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert kat([0xA4093822, 0x299F31D0], [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


@pytest.mark.parametrize("name", PS.CPU_SCENES)
def test_oracle_matches_reference_fixture(gold, name):
    z, meta = gold
    m = meta["scenes"][name]
    cfg, parts, grid = PS.build(name)
    orc = H.OracleRun("port", cfg, parts, grid=grid)
    ph = orc.physics()
    tal, rec = orc.trace(S.run_params(meta["n_rays"], seed=PS.seed_of(name)), records=True)
    orc.close()
    # integer outcomes: exact on any platform
    for k in PS.TALLY_KEYS:
        np.testing.assert_array_equal(tal[k], z[f"{name}/{k}"], err_msg=f"{name}: tally {k}")
    assert tal["event_counts"][:PS.EVENT_KEYS].tolist() == m["event_counts"]
    assert [int(v) for v in tal["conditional_stats"]] == m["conditional_stats"]
    np.testing.assert_array_equal(PS.compact(rec, meta["n_compact"]).astype(np.int16), z[f"{name}/compact"])
    # full bitwise record and table identity on the platform the fixture was generated on
    if platform.machine() == meta["machine"]:
        assert PS.records_digest(rec) == m["records_sha256"], f"{name}: per-ray records differ"
        assert PS.physics_digests(ph) == m["physics_sha256"], f"{name}: physics tables differ"


def test_oracle_meridional_field_matches_reference_fixture(gold):
    """Sediment model 3 without a supplied field: the restated red-black SOR solver stops at the reference's
    iteration with its residual, and gives the reference's field (bit for bit on the fixture's platform)."""
    import hashlib
    z, meta = gold
    m = meta["scenes"]["meridional_solver"]["field"]
    cfg, parts, grid = PS.build("meridional_solver")
    orc = H.OracleRun("port", cfg, parts, grid=grid)
    f = orc.sediment_field()
    orc.close()
    assert f["grid"].shape[1:] == (m["nr"], m["nz"])
    assert f["iterations"] == m["iterations"]
    np.testing.assert_allclose(f["grid"][0], z["meridional_solver/field_bin0"], rtol=1e-9, atol=0)
    assert f["max_residual"] == pytest.approx(m["max_residual"], rel=1e-6)
    if platform.machine() == meta["machine"]:
        assert f["max_residual"] == m["max_residual"]
        assert hashlib.sha256(f["grid"].tobytes()).hexdigest() == m["sha256"]
    # columns above the free surface carry their highest liquid value; the field is positive everywhere
    assert np.all(f["grid"] > 0.0) and np.all(np.isfinite(f["grid"]))


def test_oracle_meridional_solver_reports_non_convergence():
    """An iteration budget below the tolerance's need is an error, as in the reference's host."""
    cfg, parts, _ = PS.build("meridional_solver")
    cfg.meridional_solver_max_iterations = 250
    with pytest.raises(RuntimeError, match="did not converge"):
        H.OracleRun("port", cfg, parts)


@pytest.mark.skipif(not H.reference_available(), reason="host build of the reference not present (no checkout)")
@pytest.mark.parametrize("name", ["rough_spheroid", "absorbing_conditional", "scully_surface", "grid_sediment",
                                  "meridional_solver"])
def test_oracle_matches_live_reference(name):
    """Larger run against the live host build of the reference, when it could be built here."""
    cfg, parts, grid = PS.build(name)
    a = H.OracleRun("port", cfg, parts, grid=grid)
    b = H.OracleRun("reference", cfg, parts, grid=grid)
    pa, pb = a.physics(), b.physics()
    for k in pa:
        np.testing.assert_array_equal(pa[k], pb[k], err_msg=k)
    run = S.run_params(50000, seed=7, ray_offset=123456)
    ta, ra = a.trace(run, records=True)
    tb, rb = b.trace(run, records=True)
    assert PS.records_digest(ra) == PS.records_digest(rb)
    for k in PS.TALLY_KEYS:
        np.testing.assert_array_equal(ta[k], tb[k])


def test_oracle_rejects_unsupported_modes():
    cfg, parts, grid = PS.build("c1_smooth_coherent")
    orc = H.OracleRun("port", cfg, parts)
    with pytest.raises(RuntimeError):
        orc.trace(S.run_params(10, rng_mode=1))


def test_oracle_empty_run_and_precompute_errors():
    cfg, parts, _ = PS.build("c1_smooth_coherent")
    orc = H.OracleRun("port", cfg, parts)
    tal, rec = orc.trace(S.run_params(0), records=True)
    assert tal["n_rays"] == 0 and tal["status_counts"].sum() == 0 and rec.size == 0
    # a size parameter beyond the Mie order limit is a precompute error (reference error code 1, :3510)
    big = S.Particles([5e-3], [1.0], [1.5], [0.0], 1.0)
    with pytest.raises(RuntimeError, match="Mie"):
        H.OracleRun("port", cfg, big)


def test_failure_categories_close(gold):
    """Every failed history carries one failure code (the reference's closure check of its production failure
    categories, CLARITAS/CLARITAS.py:9640-9655), in every scene of the reference fixture."""
    z, meta = gold
    for name in meta["scenes"]:
        assert int(z[f"{name}/failure_code_counts"][1:].sum()) == int(z[f"{name}/status_counts"][4]), name


def test_oracle_meridional_solver_properties():
    """The reference's validation of its meridional solver (CLARITAS/validate_claritas.py:1405-1460) on the
    restated solver: at least 1000 iterations, converged, the normalised mass of every bin is the liquid
    volume's, and the field is finite and non-negative in the liquid."""
    cfg = S.ModelConfig(free_surface_model="parabolic_vortex", vortex_wall_center_height_difference_m=0.05,
                        vortex_core_radius_m=0.02,
                        sediment_transport_model="schiller_naumann_meridional_advection_diffusion",
                        meridional_circulation_ratio=0.05, meridional_grid_nr=16, meridional_grid_nz=32,
                        meridional_solver_max_iterations=3000, meridional_solver_check_interval=100,
                        meridional_solver_tolerance=1e-05, meridional_solver_sor=1.5, particle_event_model="geometric")
    parts = S.quartz_particles(500.0, n_bins=12)
    orc = H.OracleRun("port", cfg, parts)
    f = orc.sediment_field()
    orc.close()
    assert f["iterations"] >= 1000 and f["max_residual"] <= 1e-05
    grid = f["grid"]
    nr, nz = grid.shape[1:]
    assert (nr, nz) == (16, 32)
    rin, zmin, zmean, dh = (float(cfg.tube_inner_radius_m), float(cfg.zmin), float(cfg.zmean),
                            float(cfg.vortex_wall_center_height_difference_m))
    ztop = float(cfg.sediment_spec().grid_zmax)
    r = (np.arange(nr) + 0.5) * rin / nr
    z = zmin + (np.arange(nz) + 0.5) * (ztop - zmin) / nz
    active = z[None, :] < (zmean + dh * (r * r / rin ** 2 - 0.5))[:, None]
    dr, dz = rin / nr, (ztop - zmin) / nz
    rw = np.arange(nr) * dr
    vol = 0.5 * ((rw + dr) ** 2 - rw ** 2)[:, None] * dz
    mass = np.sum(grid * active[None] * vol[None], axis=(1, 2))
    np.testing.assert_allclose(mass, 0.5 * rin ** 2 * (zmean - zmin), rtol=4e-12, atol=2e-16)
    vals = grid[:, active]
    assert np.all(np.isfinite(vals)) and np.all(vals >= 0.0)


@pytest.mark.parametrize("vortex", ["parabolic_vortex", "localized_scully_vortex"])
def test_oracle_full_ray_without_failures(vortex):
    """The reference's full-ray validation case (CLARITAS/validate_claritas.py:1461-1540: stirred default cell,
    Schiller-Naumann sediment, conditional closure, 2048 rays, seed 24630001) ends every history without a
    production failure; absorbing bins exercise the closure."""
    cfg = S.ModelConfig(free_surface_model=vortex, vortex_wall_center_height_difference_m=0.05, vortex_core_radius_m=0.02,
                        sediment_transport_model="schiller_naumann_drift_diffusion", meridional_circulation_ratio=0.0,
                        particle_event_model="hybrid_mie_exact_rate", hybrid_wave_scale=1.0, max_internal_bounces=4095)
    orc = H.OracleRun("port", cfg, S.quartz_particles(500.0, n_bins=32, k=1e-4))
    tal, _ = orc.trace(S.run_params(2048, seed=24630001))
    orc.close()
    assert int(tal["failure_code_counts"][1:].sum()) == 0 and int(tal["status_counts"][4]) == 0
    assert int(tal["status_counts"][5]) > 0 and int(tal["conditional_stats"][0]) > 0
    assert int(tal["status_counts"].sum()) == 2048


@pytest.mark.skipif(not H.reference_available(), reason="host build of the reference not present (no checkout)")
def test_oracle_moment_constrained_law_matches_live_reference():
    """Event model 5 with per-bin moment coefficients (apply_mie_moment_constraint, CLARITAS.py:4459-4476):
    the restatement against the reference's host build, bit for bit."""
    cfg, parts, grid = PS.build("moment_constrained")
    mom = PS.moments("moment_constrained", parts.diameter_m.size)
    a = H.OracleRun("port", cfg, parts, grid=grid, moments=mom)
    b = H.OracleRun("reference", cfg, parts, grid=grid, moments=mom)
    run = S.run_params(50000, seed=PS.seed_of("moment_constrained"))
    ta, ra = a.trace(run, records=True)
    tb, rb = b.trace(run, records=True)
    assert PS.records_digest(ra) == PS.records_digest(rb)
    for k in PS.TALLY_KEYS:
        np.testing.assert_array_equal(ta[k], tb[k])
    # the map is active: the same run without the moments gives other records
    c = H.OracleRun("port", cfg, parts, grid=grid)
    tc, rc = c.trace(run, records=True)
    assert PS.records_digest(rc) != PS.records_digest(ra)
