"""GPU: light-history diagnostics (voxel track lengths, scatter-event sites, trajectories, heat maps).

They are observational: a trace with them on must give the same histories (tallies) as without. The
voxel deposition must close (deposited = clipped segment length; grid sum = segment total), and, for
rays whose every segment is kept as a representative trajectory, each voxel's track length must equal an
exact FP64 slab intersection of those segments computed here (CLARITAS/CLARITAS.py:3318-3400).
"""
from __future__ import annotations

import numpy as np
import pytest

import parity_scenes as PS
from tardiis_and_claritas_gb300 import forward as F, scene as S

pytestmark = pytest.mark.gpu

N = 60_000


@pytest.fixture(scope="module")
def ctx():
    from tardiis_and_claritas_gb300 import lib as L
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    c = L.Context(0)
    cfg, parts, grid = PS.build("rough_spheroid")
    c.set_scene(cfg.to_scene_params())
    c.build_particles(parts.spec(cfg), cfg.sediment_spec(grid))
    c.cfg = cfg
    yield c
    c.close()


def _box(cfg):
    vg = S.vortex_surface_geometry(cfg.free_surface_model, cfg.zmean, cfg.tube_inner_radius_m,
                                   cfg.vortex_wall_center_height_difference_m, cfg.vortex_core_radius_m,
                                   cfg.gravity_m_s2)
    return max(vg["center_z"], vg["wall_z"]), vg["wall_z"]


def test_diagnostics_do_not_change_histories(ctx):
    run = S.run_params(N, seed=5)
    ctx.set_light()
    base, _ = ctx.trace(run)
    zmax, zvis = _box(ctx.cfg)
    ctx.set_light(True, 16, 16, 24, N, 16, 256, 32, zmax, zvis)
    lit, _ = ctx.trace(run)
    for k in PS.TALLY_KEYS:
        np.testing.assert_array_equal(lit[k], base[k], err_msg=k)
    a = ctx.read_light()
    steps = int(base["event_counts"][20])  # water flights
    assert a["error_count"] == 0 and a["event_outside_count"] == 0
    assert 0.999 * steps <= a["segment_count"] <= steps
    assert abs(a["deposited_length_total"] - a["segment_length_total"]) <= 1e-9 * a["segment_length_total"]
    assert abs(float(a["track_length"].sum(dtype=np.float64)) - a["segment_length_total"]) \
        <= 1e-4 * a["segment_length_total"]
    assert a["scatter_event_total"] == int(a["scatter_event_count"].sum(dtype=np.uint64))
    assert a["scatter_event_total"] >= int(base["event_counts"][0])
    assert np.all(a["post_scatter_track_length"] <= a["track_length"] * (1 + 1e-5) + 1e-12)
    assert a["heatmap_xy"].sum() > 0 and a["heatmap_zy"].sum() > 0
    ctx.set_light()


def _slab_deposit(segs, R, zmin, zmax, nx, ny, nz):
    """Exact track length per voxel of straight segments: split each at every grid plane it crosses."""
    g = np.zeros((nz, ny, nx))
    edges = [np.linspace(-R, R, nx + 1), np.linspace(-R, R, ny + 1), np.linspace(zmin, zmax, nz + 1)]
    for p0, p1 in segs:
        d = p1 - p0
        L = np.linalg.norm(d)
        if not L > 0:
            continue
        ts = [0.0, 1.0]
        for ax in range(3):
            if abs(d[ax]) > 0:
                t = (edges[ax] - p0[ax]) / d[ax]
                ts.extend(t[(t > 0) & (t < 1)])
        ts = np.unique(ts)
        for t0, t1 in zip(ts[:-1], ts[1:]):
            m = p0 + d * (0.5 * (t0 + t1))
            ix = min(max(int(np.floor((m[0] + R) / (2 * R) * nx)), 0), nx - 1)
            iy = min(max(int(np.floor((m[1] + R) / (2 * R) * ny)), 0), ny - 1)
            iz = min(max(int(np.floor((m[2] - zmin) / (zmax - zmin) * nz)), 0), nz - 1)
            g[iz, iy, ix] += (t1 - t0) * L
    return g


def test_voxel_track_lengths_equal_exact_slab_intersection(ctx):
    cfg = ctx.cfg
    zmax, zvis = _box(cfg)
    nx, ny, nz, rays, seg = 12, 12, 16, 64, 4096
    ctx.set_light(True, nx, ny, nz, rays, rays, seg, 0, zmax, zvis)
    ctx.trace(S.run_params(rays, seed=9))
    a = ctx.read_light()
    assert not a["trajectory_overflow"].any()
    segs = []
    for r in range(rays):
        for k in range(a["trajectory_count"][r]):
            p0 = np.array([a["trajectory_x0"][r, k], a["trajectory_y0"][r, k], a["trajectory_z0"][r, k]], np.float64)
            p1 = np.array([a["trajectory_x1"][r, k], a["trajectory_y1"][r, k], a["trajectory_z1"][r, k]], np.float64)
            segs.append((p0, p1))
    assert len(segs) == a["segment_count"] > 0
    want = _slab_deposit(segs, cfg.tube_inner_radius_m, cfg.zmin, zmax, nx, ny, nz)
    # trajectories are stored in FP32: allow the endpoint rounding (1e-7 relative of the cell size)
    np.testing.assert_allclose(a["track_length"], want, rtol=1e-4, atol=1e-8)
    ctx.set_light()


def test_forward_result_light_fields():
    kw = {k: v for k, v in S.small_cell_config().__dict__.items() if k not in ("source_kind", "disc_beam_radius_m")}
    kw["statistics_batch_rays"] = 20_000
    m = F.ClaritasForwardModel(**kw)
    m.register_material("quartz", S.quartz_particles(1.0, n_bins=16))
    res = m.simulate("quartz", 1.0, n_rays=40_000, seed=2, heatmap_size=24,
                     light_transport_config={"enabled": True, "nx": 8, "ny": 8, "nz": 10, "max_rays": 40_000,
                                             "representative_rays": 4, "max_segments_per_ray": 64})
    assert res.heatmap_xy.shape == (24, 24) and res.heatmap_xy.sum() > 0
    d = res.light_transport_diagnostics
    assert d["track_length_m"].shape == (10, 8, 8) and d["error_count"] == 0
    assert d["deposition_closure_relative_error"] < 1e-9 and d["grid_closure_relative_error"] < 1e-4
    assert d["scatter_event_closure_error"] == 0 and d["diagnostic_rays_processed"] == 40_000
    plain = m.simulate("quartz", 1.0, n_rays=40_000, seed=2)
    np.testing.assert_array_equal(plain.hardware_native_hits, res.hardware_native_hits)
    assert plain.heatmap_xy is None and plain.light_transport_diagnostics is None
    m.close()
