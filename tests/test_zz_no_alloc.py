"""GPU: the allocation-free Mie/phase entry point against the regular particle build.

clr_mie_phase_noalloc is for callers that cannot allocate device memory themselves (a loop whose
memory belongs to another framework's pool, where a cudaMalloc/cudaFree would synchronise the
device). It runs the same Mie, theta-grid and phase kernels as clr_build_particles with a fixed
file-scope scratch, writing into caller-owned device buffers. Two consecutive calls must both
reproduce the regular build's tables bit for bit (the scratch is reused and only its error word is
reset), a call at the largest sizes the scratch holds must do the same, a failing call must leave the
scratch usable for the next one, and sizes beyond the scratch must be rejected with the limits in the
message. This file is named to be collected last; it passes alone and after the other GPU tests.
"""
from __future__ import annotations

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    yield c
    c.close()


def _device_inputs(parts):
    import torch
    dev = torch.device("cuda", 0)
    return [torch.from_numpy(np.ascontiguousarray(getattr(parts, k))).to(dev)
            for k in ("diameter_m", "n_real", "k_imag")]


def _run_noalloc(ctx, parts, cfg, n_theta):
    import torch
    dev = torch.device("cuda", 0)
    n = parts.diameter_m.size
    d, nr, k = _device_inputs(parts)
    qext = torch.empty(n, dtype=torch.float64, device=dev)
    qsca = torch.empty_like(qext)
    g = torch.empty_like(qext)
    theta = torch.empty(n_theta, dtype=torch.float64, device=dev)
    cdf = torch.empty(n * n_theta, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    ctx.mie_phase_noalloc(d.data_ptr(), nr.data_ptr(), k.data_ptr(), n, float(cfg.n_water),
                          float(cfg.particle_wavelength_m), n_theta, qext.data_ptr(), qsca.data_ptr(), g.data_ptr(),
                          theta.data_ptr(), cdf.data_ptr(), stream.cuda_stream)
    return {"qext": qext.cpu().numpy(), "qsca": qsca.cpu().numpy(), "asym_g": g.cpu().numpy(),
            "theta": theta.cpu().numpy(), "phase_cdf": cdf.cpu().numpy().reshape(n, n_theta)}


def test_noalloc_matches_regular_build_on_consecutive_calls(ctx):
    cfg = S.small_cell_config()
    cfg.validate()
    parts = S.quartz_particles(500.0, n_bins=12, k=1e-4)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec())
    ref = ctx.physics()
    n_theta = int(cfg.mie_phase_grid_size)
    for call in range(2):
        got = _run_noalloc(ctx, parts, cfg, n_theta)
        for key in ("qext", "qsca", "asym_g", "theta", "phase_cdf"):
            np.testing.assert_array_equal(got[key], ref[key], err_msg=f"call {call}: {key}")


def test_noalloc_at_the_scratch_limits(ctx):
    """16 bins and 4097 angles, the outer edge of every scratch array, equal the regular build."""
    from tardiis_and_claritas_gb300 import lib as L
    cfg = S.small_cell_config(mie_phase_grid_size=L.NOALLOC_MAX_THETA)
    cfg.validate()
    parts = S.quartz_particles(500.0, n_bins=L.NOALLOC_MAX_BINS, k=1e-4)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec())
    ref = ctx.physics()
    for call in range(2):
        got = _run_noalloc(ctx, parts, cfg, L.NOALLOC_MAX_THETA)
        for key in ("qext", "qsca", "asym_g", "theta", "phase_cdf"):
            np.testing.assert_array_equal(got[key], ref[key], err_msg=f"call {call}: {key}")


def test_noalloc_failed_call_leaves_the_scratch_usable(ctx):
    """A zero diameter raises the Mie kernel's error code 2 in the shared error word; the next valid
    call must start from a cleared word and give the regular build's tables."""
    cfg = S.small_cell_config()
    cfg.validate()
    bad = S.quartz_particles(500.0, n_bins=8)
    bad.diameter_m = bad.diameter_m.copy()
    bad.diameter_m[3] = 0.0
    with pytest.raises(RuntimeError, match="error code 2"):
        _run_noalloc(ctx, bad, cfg, 1801)
    parts = S.quartz_particles(500.0, n_bins=8)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec())
    ref = ctx.physics()
    got = _run_noalloc(ctx, parts, cfg, 1801)
    for key in ("qext", "qsca", "asym_g", "theta", "phase_cdf"):
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)


def test_noalloc_rejects_sizes_beyond_its_scratch(ctx):
    cfg = S.small_cell_config()
    cfg.validate()
    parts = S.quartz_particles(500.0, n_bins=17)
    with pytest.raises(RuntimeError, match="n_bins must be 1..16 and n_theta 2..4097"):
        _run_noalloc(ctx, parts, cfg, 1801)
    parts = S.quartz_particles(500.0, n_bins=4)
    with pytest.raises(RuntimeError, match="n_theta 2..4097"):
        _run_noalloc(ctx, parts, cfg, 5000)
