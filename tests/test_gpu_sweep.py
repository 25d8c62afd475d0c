"""GPU: the scenario sweep (clr_sweep_build + clr_sweep_trace) against single-scene builds and traces.

A sweep builds every scenario's tables with the Mie and phase kernels running over the bins of many
scenarios per launch, and traces all scenarios in one engine execution. Each scenario must come out
exactly as if it had been built and traced alone: bit-identical tables, and (per-ray random streams
keyed by the run's seeds and global ray ids) identical integer tallies.
"""
from __future__ import annotations

import numpy as np
import pytest

import parity_scenes as PS
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


def _mixed_scenarios():
    """Sweep scenarios plus parity scenes of other event and sediment models (a 64x64 grid included),
    so the sweep's Mie key and table shapes change along the way."""
    out = []
    for sc in S.sweep_workload(5, sampler_seed=11, photons=(2e4, 4e4)):
        out.append((sc.cfg, sc.particles, None, sc.n_photons, sc.seed))
    for k, name in enumerate(("geometric_law", "schiller_sediment", "grid_sediment", "c1_smooth_coherent")):
        cfg, parts, grid = PS.build(name)
        out.append((cfg, parts, grid, 20_000 + 1000 * k, PS.seed_of(name)))
    return out


def _specs(items):
    scenes = [cfg.to_scene_params() for cfg, _, _, _, _ in items]
    parts = [p.spec(cfg) for cfg, p, _, _, _ in items]
    seds = [cfg.sediment_spec(grid) for cfg, _, grid, _, _ in items]
    return scenes, parts, seds


def _build_single(ctx, cfg, parts, grid):
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid))


def test_sweep_tables_equal_single_builds(ctx):
    items = _mixed_scenarios()
    scenes, parts, seds = _specs(items)
    ctx.sweep_build(scenes, parts, seds)
    for i, (cfg, p, grid, _, _) in enumerate(items):
        nb, nt = ctx.sweep_shape[i]
        got = ctx.sweep_physics(i, nb, nt)
        _build_single(ctx, cfg, p, grid)
        want = ctx.physics()
        for k in want:
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"scenario {i}: {k}")


def test_sweep_tables_across_a_launch_chunk_boundary(ctx):
    """70 scenarios of 63 bins: the Mie launches split after 4096 bins, inside scenario 65."""
    scs = S.sweep_workload(70, sampler_seed=4, n_bins=63)
    scenes, parts, seds = S.sweep_specs(scs)
    ctx.sweep_build(scenes, parts, seds)
    for i in (0, 64, 65, 66, 69):
        got = ctx.sweep_physics(i, 63, 1801)
        _build_single(ctx, scs[i].cfg, scs[i].particles, None)
        want = ctx.physics()
        for k in want:
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"scenario {i}: {k}")


@pytest.mark.parametrize("rng", ["reference", "philox"])
def test_sweep_trace_equals_single_traces(ctx, rng):
    items = _mixed_scenarios()
    scenes, parts, seds = _specs(items)
    mode = abi.RNG_REFERENCE_XORSHIFT if rng == "reference" else abi.RNG_PHILOX
    runs = [S.run_params(n, seed=sd, ray_offset=1000 * i, rng_mode=mode, scenario_id=i)
            for i, (_, _, _, n, sd) in enumerate(items)]
    ctx.sweep_build(scenes, parts, seds)
    got = ctx.sweep_trace(runs)
    for i, (cfg, p, grid, _, _) in enumerate(items):
        _build_single(ctx, cfg, p, grid)
        want, _ = ctx.trace(runs[i])
        for k in PS.TALLY_KEYS:
            np.testing.assert_array_equal(got[i][k], want[k], err_msg=f"{rng} scenario {i}: {k}")
        assert got[i]["n_rays"] == runs[i].n_rays and got[i]["device_error"] == 0


def test_sweep_errors(ctx):
    scs = S.sweep_workload(3, sampler_seed=1, photons=(1e3, 2e3))
    scenes, parts, seds = S.sweep_specs(scs)
    bad = abi.ParticleSpec()  # null particle arrays
    bad.n_bins = 4
    bad.n_theta = 1801
    with pytest.raises(RuntimeError, match="scenario 1: particle arrays must not be null"):
        ctx.sweep_build(scenes, [parts[0], bad, parts[2]], seds)
    with pytest.raises(RuntimeError, match="clr_sweep_build must succeed"):
        ctx.sweep_trace([S.run_params(10)] * 3)
    ctx.sweep_build(scenes, parts, seds)
    with pytest.raises(RuntimeError, match="2 runs for 3 scenarios"):
        ctx.sweep_trace([S.run_params(10)] * 2)
