"""GPU: the wavefront engine's scheduling settings change the trace time, never the tallies.

clr_engine_config (flight steps per FLIGHT visit, pass graphs between flag reads, the tail-kernel
threshold, the rare-stage batch, the bounces per acrylic-traversal piece and the blocks per SM of each
stage kernel) decides only when and where a
photon's next stage runs; its draws come from its own counter (Philox) or its own state (the reference's
per-ray xorshift), so every integer tally must be identical under any setting. Floating-point sums
(photodiode, incidence, weights) are summed per warp in FP32 and then by atomics in launch order, so they
agree to FP32 rounding (relative 1e-5).
The reference has one thread per ray (CLARITAS/CLARITAS.py:7307, :7637-7640) and no such settings.
"""
from __future__ import annotations

import numpy as np
import pytest

import parity_scenes as PS
from tardiis_and_claritas_gb300 import abi, autotune as AT, scene as S

pytestmark = pytest.mark.gpu

EXTREMES = [
    {"flight_steps": 1, "pass_batch": 2, "tail_photons": 1024, "rare_batch": 64, "acr_budget": 64,
     "stage_blocks": {s: 1 for s in abi.STAGE_NAMES}},
    {"flight_steps": 16, "pass_batch": 32, "tail_photons": 1 << 20, "rare_batch": 1 << 18, "acr_budget": 1024,
     "stage_blocks": {"GEN": 2, "SIDE": 2, "BOTTOM": 4, "TOP": 4}},
    {"flight_steps": 3, "tail_photons": 1, "acr_budget": 192},
]
FLOAT_KEYS = ("photodiode_native", "photodiode_mirror", "incidence_native_sum", "incidence_mirror_sum",
              "weight_native", "weight_mirror")


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.set_engine_config(None)
    c.close()


def _assert_same(a: dict, b: dict, what: str):
    for key in PS.TALLY_KEYS + ("event_counts", "conditional_stats", "path_sums", "order_hits",
                                "geometric_order_hits", "acrylic_order_hits", "path_mask_hits"):
        assert np.array_equal(a[key], b[key]), f"{what}: {key} differs"
    assert a["n_rays"] == b["n_rays"] and a["device_error"] == b["device_error"] == 0
    for key in FLOAT_KEYS:
        np.testing.assert_allclose(a[key], b[key], rtol=1e-5, atol=1e-6, err_msg=f"{what}: {key}")


def _under_configs(ctx, run):
    ctx.set_engine_config(None)
    base, _ = ctx.trace(run)
    out = []
    for cfg in EXTREMES:
        ctx.set_engine_config(cfg)
        t, _ = ctx.trace(run)
        out.append((cfg, t, ctx.engine_stats()))
    ctx.set_engine_config(None)
    return base, out


@pytest.mark.parametrize("name", ["rough_spheroid", "scully_surface"])
def test_parity_stream_tallies_identical_under_any_setting(ctx, name):
    cfg, parts, grid = PS.build(name)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid))
    base, out = _under_configs(ctx, S.run_params(200_000, seed=PS.seed_of(name)))
    for cfg_, t, _ in out:
        _assert_same(base, t, f"{name} {cfg_}")


def _assert_nearly_same(a: dict, b: dict, n: int, what: str):
    """At most a few photons in a million routed differently (see the production-stream test): per-photon
    histograms move by a few counts, per-photon sums (entered_sums, ray_flags) by a few photons' worth."""
    for key in PS.TALLY_KEYS:
        x, y = a[key].astype(np.int64), b[key].astype(np.int64)
        d = np.abs(x - y).sum()
        if key in ("entered_sums", "ray_flags"):
            assert d <= max(400, 1e-4 * np.abs(x).sum()), f"{what}: {key} differs by {d}"
        else:
            assert d <= max(8, 4e-6 * n), f"{what}: {key} differs by {d} counts"


def test_production_stream_full_scene_identical_under_any_setting(ctx):
    """The production stream's kernels are compiled with multiply-add contraction, which the compiler
    applies per kernel, so a photon carried by the tail kernel can round differently from the same photon
    carried by the stage kernels, and a photon whose next random comparison falls within that rounding
    takes another path. Built without contraction (CLR_ALL_NOFMA=1) every integer tally is identical;
    with it, a few photons per million may differ."""
    import os
    cfg, parts, grid, zmax = S.full_scene_workload()
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid, zmax))
    n = 2_000_000
    base, out = _under_configs(ctx, S.run_params(n, seed=11, rng_mode=abi.RNG_PHILOX))
    for cfg_, t, es in out:
        if os.environ.get("CLR_ALL_NOFMA"):
            _assert_same(base, t, f"full scene {cfg_}")
        else:
            _assert_nearly_same(base, t, n, f"full scene {cfg_}")
    # the settings took effect: tail threshold 1 leaves (almost) nothing to the tail kernel, 2^20 a lot
    assert out[1][2]["tail_photons"] > out[2][2]["tail_photons"]


def test_invalid_settings_rejected(ctx):
    for bad in ({"flight_steps": 65}, {"flight_steps": -1}, {"pass_batch": 100}, {"tail_photons": -5},
                {"stage_blocks": {"FLIGHT": 33}}, {"rare_batch": 1 << 22}, {"acr_budget": 100},
                {"acr_budget": 32768}):
        with pytest.raises(RuntimeError, match="engine config"):
            ctx.set_engine_config(bad)
    ctx.set_engine_config(None)


def test_tuner_picks_a_setting_and_leaves_it_set(ctx, tmp_path):
    cfg, parts, grid, zmax = S.full_scene_workload()
    sp, ps, ss = cfg.to_scene_params(), parts.spec(cfg), cfg.sediment_spec(grid, zmax)
    ctx.set_scene(sp)
    ctx.build_particles(ps, ss)
    n = 4_000_000
    mk = lambda i: S.run_params(n, seed=5, ray_offset=i * n, rng_mode=abi.RNG_PHILOX)  # noqa: E731
    cache = str(tmp_path / "tune.json")
    res = AT.tune(ctx, mk, key=AT.scene_key(sp, ps, ss), photons=n, device="test", reps=1,
                  cache_file=cache)
    assert res["cached"] is False and res["trials"] > 10
    assert res["trace_s"] <= res["default_trace_s"] * 1.0001
    again = AT.tune(ctx, mk, key=AT.scene_key(sp, ps, ss), photons=n, device="test",
                    cache_file=cache)
    assert again["cached"] == "user" and again["config"] == res["config"]
    # the tuned context gives the default's tallies (up to contraction rounding, as above)
    run = S.run_params(500_000, seed=9, rng_mode=abi.RNG_PHILOX)
    tuned, _ = ctx.trace(run)
    ctx.set_engine_config(None)
    default, _ = ctx.trace(run)
    _assert_nearly_same(default, tuned, 500_000, f"tuned {res['config']}")
