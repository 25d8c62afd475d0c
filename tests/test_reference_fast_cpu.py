"""CPU: the speed build of the reference's host code (the timed CPU baseline) against its parity build.

The baseline times the reference's own CUDA_SRC compiled for the host with -O3 and multiply-add
contraction allowed (oracle/Makefile ref_fast); the parity build keeps -O2 without contraction so that its
bits match the CPU restatement. Contraction changes last bits on hosts with FMA, so the two are compared
statistically: tallies and end statuses within binomial standard errors on the full scene.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_harness as H
from tardiis_and_claritas_gb300 import scene as S

pytestmark = pytest.mark.skipif(not H.reference_available(), reason="host build of the reference not available")


def _z(a, na, b, nb):
    pa, pb = a / na, b / nb
    se = np.maximum(np.sqrt(pa * (1 - pa) / na + pb * (1 - pb) / nb), 1.0 / max(na, nb))
    return np.abs(pa - pb) / se


def test_fast_build_matches_parity_build():
    cfg, parts, grid, zmax = S.full_scene_workload()
    n = 200_000
    out = {}
    for kind, seed in (("reference", 5), ("reference_fast", 6)):
        o = H.OracleRun(kind, cfg, parts, grid=grid, grid_zmax=zmax)
        out[kind], _ = o.trace(S.run_params(n, seed=seed))
        o.close()
    a, b = out["reference"], out["reference_fast"]
    for key in ("hw_native", "hw_mirror", "status_counts"):
        z = _z(a[key].astype(float), n, b[key].astype(float), n)
        assert z.max() < 4.5 and np.sum(z > 3.0) <= 1, (key, np.round(z, 2))
