"""CPU: the Rankine vortex free surface (this library's surface model 3; the reference has only flat,
parabolic and localized-Scully surfaces, CLARITAS/CLARITAS.py:1503-1527, :708-792).

A stirrer spinning the core r <= a as a solid body and the liquid outside as a free vortex gives the
surface z0 + k r^2 inside and z0 + k a^2 (2 - a^2/r^2) outside. Checked here: its flat and solid-body
limits, continuity of height and slope at r = a, conservation of the liquid volume, the rpm relation, the
CPU oracle's heights and normals, and the oracle's ray/surface crossing against a brute-force root.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

import oracle_harness as H
from tardiis_and_claritas_gb300 import scene as S

R = 0.0125
ZMEAN = 0.020
CORE = 0.005
G = 9.81


@pytest.fixture(scope="module")
def lib():
    L, _ = H.load("port")
    L.clo_surface.restype = C.c_float
    L.clo_surface.argtypes = [C.c_int] + [C.c_float] * 6 + [C.c_void_p]
    L.clo_surface_hit.restype = C.c_float
    L.clo_surface_hit.argtypes = [C.c_int] + [C.c_float] * 10
    return L


def test_rpm_relation_and_flat_limit():
    dh = S.stirrer_rankine_delta_h(600.0, CORE, R)
    w = 600.0 * 2 * math.pi / 60
    assert dh == pytest.approx(w * w / (2 * G) * CORE ** 2 * (2 - CORE ** 2 / R ** 2), rel=1e-14)
    assert 8e-3 < dh < 1e-2  # a ~9 mm dip at 600 rpm with a 5 mm core
    assert S.stirrer_rankine_delta_h(0.0, CORE, R) == 0.0
    vg = S.vortex_surface_geometry("rankine_vortex", ZMEAN, R, 0.0, CORE)
    assert vg["center_z"] == vg["wall_z"] == ZMEAN
    r = np.linspace(0, R, 101)
    np.testing.assert_allclose(S.rankine_surface(r, ZMEAN, R, 1e-12, CORE), ZMEAN, atol=1e-12)


def test_continuity_at_the_core_edge():
    dh = S.stirrer_rankine_delta_h(900.0, CORE, R)
    k, a, z0 = S.rankine_surface_coefficients(ZMEAN, R, dh, CORE)
    eps = 1e-9
    zi, zo = S.rankine_surface([a - eps, a + eps], ZMEAN, R, dh, CORE)
    assert abs(zo - zi) < 1e-9 * max(1.0, dh / eps * 1e-6)
    si = (S.rankine_surface(a - eps, ZMEAN, R, dh, CORE) - S.rankine_surface(a - 2 * eps, ZMEAN, R, dh, CORE)) / eps
    so = (S.rankine_surface(a + 2 * eps, ZMEAN, R, dh, CORE) - S.rankine_surface(a + eps, ZMEAN, R, dh, CORE)) / eps
    assert so == pytest.approx(si, rel=1e-4)
    assert si == pytest.approx(2 * k * a, rel=1e-4)
    # the height difference between wall and centre is the requested dh
    zc, zw = S.rankine_surface([0.0, R], ZMEAN, R, dh, CORE)
    assert zw - zc == pytest.approx(dh, rel=1e-13)


@pytest.mark.parametrize("rpm,core", [(300.0, 0.005), (600.0, 0.005), (1200.0, 0.005), (800.0, 0.002)])
def test_volume_is_conserved(rpm, core):
    """The area mean of the surface height over the disc equals the rest height (liquid volume kept)."""
    dh = S.stirrer_rankine_delta_h(rpm, core, R)
    n = 400_000
    r = (np.arange(n) + 0.5) * (R / n)
    mean = float(np.sum(S.rankine_surface(r, ZMEAN, R, dh, core) * 2 * r) * (R / n) / R ** 2)
    assert mean == pytest.approx(ZMEAN, abs=1e-11)


def test_solid_body_limit_is_the_parabolic_surface():
    dh = 0.004
    r = np.linspace(0, R, 57)
    np.testing.assert_allclose(S.rankine_surface(r, ZMEAN, R, dh, 2 * R), ZMEAN + dh * (r * r / R ** 2 - 0.5),
                               rtol=0, atol=1e-15)


def test_geometry_helper_and_validation():
    dh = S.stirrer_rankine_delta_h(600.0, CORE, R)
    vg = S.vortex_surface_geometry("rankine_vortex", ZMEAN, R, dh, CORE)
    assert vg["wall_z"] - vg["center_z"] == pytest.approx(dh)
    assert vg["equivalent_core_rpm"] == pytest.approx(600.0, rel=1e-12)
    cfg = S.small_cell_config(free_surface_model="rankine_vortex", vortex_wall_center_height_difference_m=dh,
                              vortex_core_radius_m=CORE)
    cfg.validate()
    assert cfg.to_scene_params().free_surface_model == 3
    with pytest.raises(ValueError, match="analytic drift-diffusion"):
        S.small_cell_config(free_surface_model="rankine_vortex", vortex_wall_center_height_difference_m=dh,
                            vortex_core_radius_m=CORE, sediment_transport_model="stokes_drift_diffusion").validate()
    with pytest.raises(ValueError, match="core"):
        S.small_cell_config(free_surface_model="rankine_vortex", vortex_wall_center_height_difference_m=dh,
                            vortex_core_radius_m=0.0).validate()


def test_oracle_height_and_normal(lib):
    dh = S.stirrer_rankine_delta_h(1000.0, CORE, R)
    k, a, _ = S.rankine_surface_coefficients(ZMEAN, R, dh, CORE)
    for r in (0.0, 0.001, 0.0049, 0.0051, 0.009, 0.0125):
        n = np.zeros(3, np.float32)
        z = lib.clo_surface(3, r, 0.0, ZMEAN, R, dh, CORE, n.ctypes.data_as(C.c_void_p))
        assert z == pytest.approx(float(S.rankine_surface(r, ZMEAN, R, dh, CORE)), abs=2e-8)
        slope = 2 * k * r if r <= a else 2 * k * a ** 4 / r ** 3
        want = np.array([slope, 0.0, -1.0]) / math.hypot(slope, 1.0)
        np.testing.assert_allclose(n, want, atol=2e-6)


def _brute_hit(p, v, dh, core):
    """First crossing of z(t) - zs(r(t)) inside the tube by dense sampling and FP64 bisection."""
    t_end = 0.06
    ts = np.linspace(0.0, t_end, 240_001)[1:]
    pts = p[None, :] + ts[:, None] * v[None, :]
    r = np.hypot(pts[:, 0], pts[:, 1])
    inside = r <= R
    f = pts[:, 2] - S.rankine_surface(np.minimum(r, R), ZMEAN, R, dh, core)
    f0 = p[2] - float(S.rankine_surface(math.hypot(p[0], p[1]), ZMEAN, R, dh, core))
    fs = np.concatenate([[f0], f])
    ok = np.concatenate([[True], inside])
    idx = np.nonzero((np.sign(fs[1:]) != np.sign(fs[:-1])) & ok[1:] & ok[:-1])[0]
    if idx.size == 0:
        return math.inf
    lo, hi = (0.0 if idx[0] == 0 else ts[idx[0] - 1]), ts[idx[0]]

    def fn(t):
        q = p + t * v
        return q[2] - float(S.rankine_surface(math.hypot(q[0], q[1]), ZMEAN, R, dh, core))
    flo = fn(lo)
    for _ in range(80):
        m = 0.5 * (lo + hi)
        if (fn(m) < 0) == (flo < 0):
            lo, flo = m, fn(m)
        else:
            hi = m
    return 0.5 * (lo + hi)


@pytest.mark.parametrize("rpm", [600.0, 1200.0])
def test_oracle_ray_crossing_against_brute_force(lib, rpm):
    dh = S.stirrer_rankine_delta_h(rpm, CORE, R)
    rng = np.random.default_rng(1234 + int(rpm))
    checked = 0
    for _ in range(150):
        rr, ph = R * math.sqrt(rng.uniform(0, 0.98)), rng.uniform(0, 2 * math.pi)
        x, y = rr * math.cos(ph), rr * math.sin(ph)
        zs = float(S.rankine_surface(rr, ZMEAN, R, dh, CORE))
        z = zs - rng.uniform(1e-4, 0.01)
        v = rng.normal(size=3)
        v[2] = abs(v[2]) * rng.choice([1.0, 0.3])  # upward rays, some shallow
        v /= np.linalg.norm(v)
        want = _brute_hit(np.array([x, y, z]), v, dh, CORE)
        got = lib.clo_surface_hit(3, x, y, z, *v, ZMEAN, R, dh, CORE)
        if not math.isfinite(want):
            assert got > 1e30 or got > 0.05, (x, y, z, v, got)
            continue
        assert got == pytest.approx(want, rel=2e-5, abs=2e-8), (x, y, z, v, got, want)
        checked += 1
    assert checked >= 40  # the rest leave through the wall first
