"""GPU: the production path at bench scale against the reference's own code.

The headline workload runs on the counter-based Philox stream with FP32 boundary roots and node-table
field sampling, none of which is the reference's arithmetic, so only statistics can pin it. Here the full
scene is traced with 1e8 photons on the GPU (32 batches of one engine execution) and with 2e7 photons by
the reference's own trace and scoring kernels compiled for the host (32 batches). Standard errors come from
the 32 batch means of each side. Required: |z| < 3 on the transmitted (0), 90-degree (9) and 170-degree (17)
channels, native and mirrored, and on every end status and failure code (rare ones by the pooled
two-proportion statistic, whose batch means are mostly zero).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import oracle_harness as H
from tardiis_and_claritas_gb300 import abi, scene as S

pytestmark = pytest.mark.gpu

K = 32
HEADLINE = (0, 9, 17)


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.close()


def _batch_z(ga, ca):
    """z of the difference of the means of two sets of per-batch fractions, from their batch means."""
    gm, cm = ga.mean(axis=0), ca.mean(axis=0)
    se = np.sqrt(ga.var(axis=0, ddof=1) / ga.shape[0] + ca.var(axis=0, ddof=1) / ca.shape[0])
    return np.where(se > 0, np.abs(gm - cm) / np.where(se > 0, se, 1.0), 0.0)


def _pooled_z(a, na, b, nb):
    p = (a + b) / (na + nb)
    se = np.maximum(np.sqrt(p * (1 - p) * (1.0 / na + 1.0 / nb)), 1.0 / (na + nb))
    return np.abs(a / na - b / nb) / se


def test_full_scene_1e8_gpu_against_2e7_reference(ctx):
    if not H.reference_available():
        pytest.skip("host build of the reference not available")
    cfg, parts, grid, zmax = S.full_scene_workload()
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid, zmax))
    n_g = 100_000_000 // K
    runs = [S.run_params(n_g, seed=20261204, ray_offset=k * n_g, rng_mode=abi.RNG_PHILOX) for k in range(K)]
    gt = ctx.trace_batch(runs)
    assert all(t["device_error"] == 0 for t in gt)
    o = H.OracleRun("reference_fast", cfg, parts, grid=grid, grid_zmax=zmax)
    n_c = 20_000_000 // K
    ct = [o.trace(S.run_params(n_c, seed=7000 + k), threads=os.cpu_count() or 1)[0] for k in range(K)]
    o.close()
    for side in ("hw_native", "hw_mirror"):
        g = np.array([t[side][list(HEADLINE)] for t in gt], float) / n_g
        c = np.array([t[side][list(HEADLINE)] for t in ct], float) / n_c
        z = _batch_z(g, c)
        assert np.all(z < 3.0), f"{side} channels {HEADLINE}: z={np.round(z, 2)}"
    for key in ("status_counts", "failure_code_counts"):
        ga = np.array([t[key] for t in gt], float)
        ca = np.array([t[key] for t in ct], float)
        tot_g, tot_c = ga.sum(axis=0), ca.sum(axis=0)
        frequent = (tot_g / (n_g * K) > 1e-4) & (tot_c >= 200)
        z = np.where(frequent, _batch_z(ga / n_g, ca / n_c), _pooled_z(tot_g, n_g * K, tot_c, n_c * K))
        assert np.all(z < 3.0), f"{key}: z={np.round(z, 2)}"
