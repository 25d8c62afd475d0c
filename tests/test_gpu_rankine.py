"""GPU: the Rankine vortex free surface (this library's surface model 3) against the CPU oracle.

The reference has no Rankine surface (its models are flat, parabolic and localized Scully,
CLARITAS/CLARITAS.py:1503-1527), so parity here is statistical: the GPU path (FP32 crossings on the
counter-based stream, FP64 crossings on the xorshift stream) and the oracle's FP64 restatement must give
the same tallies, end statuses and failure counts within binomial standard errors, on a stirred cell at
600 and 1200 rpm (the latter's air core reaches below the beam) and on the full scene with its
Rouse x radial-depletion field.
"""
from __future__ import annotations

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import abi, scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.close()


def _z_binomial(a, na, b, nb):
    pa, pb = a / na, b / nb
    se = np.maximum(np.sqrt(pa * (1 - pa) / na + pb * (1 - pb) / nb), 1.0 / max(na, nb))
    return np.abs(pa - pb) / se


def _assert_agree(a, na, b, nb, what):
    # failure code 0 counts the rays without a failure: it is the complement of the other codes, so it is
    # left out (it would repeat their deviation)
    for key, lo in (("hw_native", 0), ("hw_mirror", 0), ("status_counts", 0), ("failure_code_counts", 1)):
        z = _z_binomial(a[key][lo:].astype(float), na, b[key][lo:].astype(float), nb)
        assert np.max(z) < 4.5 and np.sum(z > 3.0) <= 1, f"{what} {key}: z={np.round(z, 2)}"


def _stirred(rpm):
    dh = S.stirrer_rankine_delta_h(rpm, 0.005, 0.0125)
    cfg = S.small_cell_config(free_surface_model="rankine_vortex", vortex_wall_center_height_difference_m=dh,
                              vortex_core_radius_m=0.005)
    cfg.validate()
    return cfg


@pytest.mark.parametrize("rpm", [600.0, 1200.0])
def test_rankine_gpu_matches_cpu_oracle(ctx, rpm):
    import oracle_harness as H
    cfg = _stirred(rpm)
    parts = S.quartz_particles(2000.0)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec())
    n_gpu = 2_000_000
    p, _ = ctx.trace(S.run_params(n_gpu, seed=51, rng_mode=abi.RNG_PHILOX))
    x, _ = ctx.trace(S.run_params(n_gpu, seed=52, rng_mode=abi.RNG_REFERENCE_XORSHIFT))
    assert p["device_error"] == 0 and x["device_error"] == 0
    orc = H.OracleRun("port", cfg, parts)
    n_cpu = 400_000
    c, _ = orc.trace(S.run_params(n_cpu, seed=53))
    orc.close()
    _assert_agree(p, n_gpu, c, n_cpu, f"rankine {rpm:.0f} rpm philox/oracle")
    _assert_agree(x, n_gpu, c, n_cpu, f"rankine {rpm:.0f} rpm xorshift/oracle")
    _assert_agree(p, n_gpu, x, n_gpu, f"rankine {rpm:.0f} rpm philox/xorshift")
    # photons do reach the free surface and the headspace in this scene
    assert p["event_counts"][abi.EV_NAMES.index("top")] > 0


def test_rankine_full_scene_matches_cpu_oracle(ctx):
    import oracle_harness as H
    cfg, parts, grid, zmax = S.full_scene_workload(surface="rankine_vortex")
    assert cfg.free_surface_model == "rankine_vortex"
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid, zmax))
    n_gpu = 2_000_000
    g, _ = ctx.trace(S.run_params(n_gpu, seed=61, rng_mode=abi.RNG_PHILOX))
    assert g["device_error"] == 0
    orc = H.OracleRun("port", cfg, parts, grid=grid, grid_zmax=zmax)
    n_cpu = 300_000
    c, _ = orc.trace(S.run_params(n_cpu, seed=62))
    orc.close()
    _assert_agree(g, n_gpu, c, n_cpu, "rankine full scene")


def test_rankine_rejects_the_meridional_solver(ctx):
    cfg = S.small_cell_config(free_surface_model="rankine_vortex",
                              vortex_wall_center_height_difference_m=S.stirrer_rankine_delta_h(600, 0.005, 0.0125),
                              vortex_core_radius_m=0.005,
                              sediment_transport_model="schiller_naumann_meridional_advection_diffusion")
    cfg.validate()
    parts = S.quartz_particles(500.0, n_bins=8)
    ctx.set_scene(cfg.to_scene_params())
    with pytest.raises(RuntimeError, match="supply the"):
        ctx.build_particles(parts.spec(cfg), cfg.sediment_spec())
