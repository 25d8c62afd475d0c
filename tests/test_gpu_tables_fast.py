"""GPU: the fast phase tables (CLR_TABLES_FAST) equal the reference-order tables to rounding.

The reference builds the phase pdf from S1 = sum c_n (a_n pi_n + b_n tau_n) and S2 in FP64 in a fixed order of
operations (CLARITAS/CLARITAS.py:3561-3581), which the parity build keeps bit for bit. The fast variant
(phase_pdf_fast_kernel) evaluates the same sums with fused multiply-adds on premultiplied coefficients and
two mirrored angles per Legendre recurrence. Its Mie efficiencies are the same kernel's (identical); its
phase CDF must agree within 1e-12 on every bin, from Rayleigh-like to size parameters near 1400.
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


def _tables(ctx, cfg, parts, arithmetic):
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg, table_arithmetic=arithmetic), cfg.sediment_spec())
    return ctx.physics()


@pytest.mark.parametrize("k_imag,n_theta", [(0.0, 1801), (1e-3, 1801), (0.0, 2048)])
def test_fast_tables_equal_reference_tables(ctx, k_imag, n_theta):
    cfg = S.small_cell_config(mie_phase_grid_size=n_theta)
    parts = S.quartz_particles(n_bins=64, d_min_um=0.1, d_max_um=300.0, k=k_imag)
    ref = _tables(ctx, cfg, parts, abi.TABLES_REFERENCE)
    fast = _tables(ctx, cfg, parts, abi.TABLES_FAST)
    for key in ("qext", "qsca", "asym_g", "nstop", "theta"):
        assert np.array_equal(ref[key], fast[key]), key
    a = ref["phase_cdf"].reshape(64, n_theta)
    b = fast["phase_cdf"].reshape(64, n_theta)
    assert np.all(np.diff(b, axis=1) >= 0.0) and np.all(b[:, -1] == 1.0) and np.all(b[:, 0] == 0.0)
    err = np.abs(a - b).max(axis=1)
    assert err.max() <= 1e-12, f"max |dCDF| per bin: {err.max():.3e} (bin {int(err.argmax())})"
    # the photon sampler reads the float copy: the fast tables round to the same floats almost everywhere
    assert np.mean(a.astype(np.float32) != b.astype(np.float32)) < 1e-3


def test_fast_tables_sweep_equals_single_build(ctx):
    scs = S.sweep_workload(6, sampler_seed=3)
    scenes, parts, seds = S.sweep_specs(scs, table_arithmetic=abi.TABLES_FAST)
    ctx.sweep_build(scenes, parts, seds)
    for i, sc in enumerate(scs):
        n_bins, n_theta = int(parts[i].n_bins), int(parts[i].n_theta)
        sw = ctx.sweep_physics(i, n_bins, n_theta)
        ctx.set_scene(scenes[i])
        ctx.build_particles(parts[i], seds[i])
        one = ctx.physics()
        assert np.array_equal(sw["phase_cdf"], one["phase_cdf"]), i


def test_mixed_table_arithmetic_in_one_sweep_rejected(ctx):
    scs = S.sweep_workload(2, sampler_seed=4)
    scenes, parts, seds = S.sweep_specs(scs, table_arithmetic=abi.TABLES_FAST)
    parts[1].table_arithmetic = abi.TABLES_REFERENCE
    with pytest.raises(RuntimeError, match="table_arithmetic"):
        ctx.sweep_build(scenes, parts, seds)
