"""GPU: the weighted estimator (implicit capture + Russian roulette) against the analog one.

The reference transports analog photons: absorption ends a history (CLARITAS/CLARITAS.py:4851, :4874,
:4931) and detector tallies are integer hit counts (:4416, :4424). The weighted mode is new: absorption
is never sampled, the photon's weight carries the survival probability, and Russian roulette cuts the
low-weight tail. Its detector weight sums must estimate the analog hit counts without bias: they agree
within combined standard errors on every absorbing configuration, and are identical when nothing absorbs.
"""
from __future__ import annotations

import numpy as np
import pytest

import parity_scenes as PS
from tardiis_and_claritas_gb300 import abi, scene as S

pytestmark = pytest.mark.gpu

HEADLINE = (0, 9, 17)  # transmitted, nephelometric (90 deg) and nearest-backscatter (170 deg) channels


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.close()


def _load(ctx, cfg, parts, grid=None, zmax=None):
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid, zmax))


def _weighted(n, seed, threshold=1e-4, survival=1e-3):
    return S.run_params(n, seed=seed, rng_mode=abi.RNG_PHILOX, weight_mode=abi.WEIGHT_IMPLICIT,
                        roulette_threshold=threshold, roulette_survival=survival)


def _z(analog, na, weighted, nw, side):
    """Per-detector z of (weighted mean weight per photon) - (analog hit fraction)."""
    hits = analog[f"hw_{side}"].astype(float)
    p = hits / na
    var_a = p * (1.0 - p) / na
    w = weighted[f"weight_{side}"] / nw
    w2 = weighted[f"weight_sq_{side}"] / nw
    var_w = np.maximum(w2 - w * w, 0.0) / nw
    se = np.sqrt(var_a + var_w)
    return np.where(se > 0, np.abs(w - p) / np.where(se > 0, se, 1.0), 0.0)


def _assert_unbiased(analog, na, weighted, nw, what):
    for side in ("native", "mirror"):
        z = _z(analog, na, weighted, nw, side)
        assert np.all(z[list(HEADLINE)] < 3.0), f"{what} {side}: headline z={np.round(z[list(HEADLINE)], 2)}"
        assert z.max() < 4.0 and np.sum(z > 3.0) <= 1, f"{what} {side}: z={np.round(z, 2)}"


def test_weighted_equals_analog_when_nothing_absorbs(ctx):
    """k = 0 and no water absorption: every weight stays 1, so the weighted run is the analog run."""
    cfg, parts, grid, zmax = S.full_scene_workload()
    _load(ctx, cfg, parts, grid, zmax)
    n = 1_000_000
    a, _ = ctx.trace(S.run_params(n, seed=7, rng_mode=abi.RNG_PHILOX))
    w, _ = ctx.trace(_weighted(n, seed=7))
    for key in ("hw_native", "hw_mirror", "status_counts", "failure_code_counts", "ic_hist"):
        np.testing.assert_array_equal(w[key], a[key], err_msg=key)
    np.testing.assert_array_equal(w["weight_native"], a["hw_native"].astype(float))
    np.testing.assert_array_equal(w["weight_sq_mirror"], a["hw_mirror"].astype(float))
    assert w["event_counts"][abi.EV_NAMES.index("roulette_kills")] == 0


def test_weighted_unbiased_on_absorbing_conditional(ctx):
    """Absorbing bins under the conditional closure (event model 4, k = 1e-3): the closure's
    absorbed/scattered draw becomes a weight factor (the particle albedo)."""
    cfg, parts, _ = PS.build("absorbing_conditional")
    _load(ctx, cfg, parts)
    n = 4_000_000
    a, _ = ctx.trace(S.run_params(n, seed=11, rng_mode=abi.RNG_PHILOX))
    w, _ = ctx.trace(_weighted(n, seed=12))
    assert a["status_counts"][5] > 1000, "the analog run must see absorption"
    assert w["status_counts"][5] == 0, "a weighted run samples no absorption"
    assert w["device_error"] == 0
    _assert_unbiased(a, n, w, n, "absorbing_conditional")


def test_weighted_unbiased_with_sphere_absorption(ctx):
    """Event laws without the closure absorb inside the sphere walk: each internal chord multiplies the
    weight by exp(-alpha chord) instead of drawing an absorption distance."""
    cfg = S.small_cell_config(particle_event_model="geometric", particle_surface_rms_slope_deg=0.0)
    cfg.validate()
    parts = S.quartz_particles(2000.0, k=3e-4)
    _load(ctx, cfg, parts)
    n = 4_000_000
    a, _ = ctx.trace(S.run_params(n, seed=21, rng_mode=abi.RNG_PHILOX))
    w, _ = ctx.trace(_weighted(n, seed=22))
    assert a["status_counts"][5] > 1000 and w["status_counts"][5] == 0
    _assert_unbiased(a, n, w, n, "geometric law, k = 3e-4")


def test_russian_roulette_is_unbiased_and_kills(ctx):
    """An aggressive roulette (threshold 0.5, survivors at weight 1) must fire and stay unbiased."""
    cfg, parts, _ = PS.build("absorbing_conditional")
    _load(ctx, cfg, parts)
    n = 4_000_000
    a, _ = ctx.trace(S.run_params(n, seed=31, rng_mode=abi.RNG_PHILOX))
    w, _ = ctx.trace(_weighted(n, seed=32, threshold=0.5, survival=1.0))
    kills = int(w["event_counts"][abi.EV_NAMES.index("roulette_kills")])
    assert kills > 1000 and kills == int(w["status_counts"][abi.STATUS_ROULETTE])
    _assert_unbiased(a, n, w, n, "roulette 0.5")


def test_water_absorption_beer_lambert_and_unbiased(ctx):
    """Water absorption (a scene option the reference lacks): ballistic photons reaching the transmitted
    detector cross about one cell diameter of water, so their mean weight is exp(-mu_a L) with L between
    the chord at the throat edge and the diameter; the analog run loses the same fraction of hits."""
    mu_a = 20.0
    clear = S.small_cell_config(particle_surface_rms_slope_deg=0.0)
    absorbing = S.small_cell_config(particle_surface_rms_slope_deg=0.0, water_absorption_per_m=mu_a)
    parts = S.quartz_particles(1e-6)  # effectively no particles: every detected photon is ballistic
    n = 4_000_000
    _load(ctx, absorbing, parts)
    w, _ = ctx.trace(_weighted(n, seed=41))
    a, _ = ctx.trace(S.run_params(n, seed=42, rng_mode=abi.RNG_PHILOX))
    _load(ctx, clear, parts)
    c, _ = ctx.trace(S.run_params(n, seed=43, rng_mode=abi.RNG_PHILOX))
    R = clear.tube_inner_radius_m
    throat = 0.5 * clear.through_bore_diameter_m
    hi, lo = np.exp(-mu_a * 2.0 * np.sqrt(R * R - throat * throat)), np.exp(-mu_a * 2.0 * R)
    mean_w = w["weight_native"][0] / w["hw_native"][0]
    assert lo * 0.995 <= mean_w <= hi * 1.005, (mean_w, lo, hi)  # tilted rays run slightly longer
    assert w["status_counts"][5] == 0 and a["status_counts"][5] > 0
    # analog survival of transmitted hits against the clear cell, and weighted against analog
    pa, pc = a["hw_native"][0] / n, c["hw_native"][0] / n
    ratio = pa / pc
    se = ratio * np.sqrt((1 - pa) / (pa * n) + (1 - pc) / (pc * n))
    assert abs(ratio - mean_w) < 3.0 * se, (ratio, mean_w, se)
    _assert_unbiased(a, n, w, n, "water absorption")


def test_weighted_arguments_are_checked(ctx):
    cfg, parts, _ = PS.build("absorbing_conditional")
    _load(ctx, cfg, parts)
    r = S.run_params(1000, seed=1, rng_mode=abi.RNG_REFERENCE_XORSHIFT, weight_mode=abi.WEIGHT_IMPLICIT)
    with pytest.raises(RuntimeError, match="Philox stream only"):
        ctx.trace(r)
    with pytest.raises(RuntimeError, match="roulette_threshold < roulette_survival"):
        ctx.trace(_weighted(1000, seed=1, threshold=1e-3, survival=1e-3))
    r = S.run_params(1000, seed=1, rng_mode=abi.RNG_PHILOX, weight_mode=7)
    with pytest.raises(RuntimeError, match="unknown weight_mode"):
        ctx.trace(r)


def test_weighted_unbiased_on_dense_absorbing_clay(ctx):
    """The dense stress regime with absorbing clay (20 g/L, optical depth ~100, the reference's kaolin n and k):
    long histories multiply many albedos, so Russian roulette at the default threshold fires, and the weight
    sums still estimate the analog hit counts."""
    cfg, _, _ = PS.build("dense_clay")
    parts = S.kaolin_clay_particles(20000.0)
    _load(ctx, cfg, parts)
    n = 1_000_000
    a, _ = ctx.trace(S.run_params(n, seed=51, rng_mode=abi.RNG_PHILOX))
    w, _ = ctx.trace(_weighted(n, seed=52))
    assert a["status_counts"][5] > 1000 and w["status_counts"][5] == 0
    assert int(w["event_counts"][abi.EV_NAMES.index("roulette_kills")]) > 0
    _assert_unbiased(a, n, w, n, "dense kaolin clay")
