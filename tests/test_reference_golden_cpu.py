"""CPU: the oracle and the scene helpers against the golden values of the reference's own validation script.

CLARITAS/validate_claritas.py pins the stirred-cell geometry (test_parabolic_geometry :59-82,
test_scully_reference :204-303), the sediment coefficients (test_parabolic_stokes_analytic :83-110,
test_parabolic_schiller_and_normalization :142-203, test_scully_reference) and the meridional velocity
field (test_scully_reference, test_parabolic_meridional_host :304-357). The same inputs go through
scene.vortex_surface_geometry and the oracle's sediment precompute and meridional velocity
(oracle/claritas_oracle.c), with the reference's tolerances.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

import oracle_harness as H
from tardiis_and_claritas_gb300 import scene as S

ZMEAN, ZMIN, R, D, CORE, DT = 0.049, -0.093, 0.0465, 0.05, 0.02, 0.001
DIAM = np.array([1e-06, 1e-05, 0.0001])


def close(actual, expected, rtol=1e-11, atol=1e-13):
    np.testing.assert_allclose(actual, expected, rtol=rtol, atol=atol)


@pytest.fixture(scope="module")
def lib():
    lib, _ = H.load("port")
    lib.clo_read_sediment.argtypes = [C.c_void_p] + [C.c_void_p] * 6
    lib.clo_read_sediment.restype = C.c_int
    lib.clo_meridional_velocity.restype = C.c_double
    lib.clo_meridional_velocity.argtypes = [C.c_int] + [C.c_double] * 8 + [C.POINTER(C.c_double)]
    return lib


def coefficients(lib, transport, surface, n_quad, n_radial, rho_p=2600.0):
    """The oracle's sediment coefficients for the validation script's cell and three diameters."""
    cfg = S.ModelConfig(free_surface_model=surface, vortex_wall_center_height_difference_m=D,
                        vortex_core_radius_m=CORE, sediment_transport_model=transport)
    sp = cfg.to_scene_params()
    ps = S.Particles(DIAM, np.ones(3), np.full(3, 1.54), np.zeros(3), 1.0, rho_p).spec(cfg)
    ss = cfg.sediment_spec()
    ss.particle_density, ss.water_density, ss.water_viscosity, ss.gravity = rho_p, 997.0, 8.9e-4, 9.81
    ss.eddy_diffusivity, ss.n_quad, ss.n_radial = DT, n_quad, n_radial
    ss.rin, ss.zmin, ss.zmean, ss.vortex_delta_h, ss.vortex_core_radius = R, ZMIN, ZMEAN, D, CORE
    h = C.c_void_p()
    rc = lib.clo_prepare(C.byref(sp), C.byref(ps), C.byref(ss), C.byref(h))
    assert rc == 0, lib.clo_last_error(h)
    out = {k: np.zeros(3) for k in ("A", "B", "norm", "ws")}
    out["radial_log"] = np.zeros((3, n_radial))
    out["radial_slip"] = np.zeros((3, n_radial))
    lib.clo_read_sediment(h, *(out[k].ctypes.data_as(C.c_void_p)
                               for k in ("A", "B", "norm", "ws", "radial_log", "radial_slip")))
    lib.clo_free(h)
    out["r"] = np.linspace(0.0, R, n_radial)
    return out


def test_parabolic_geometry():
    v = S.vortex_surface_geometry("parabolic_vortex", ZMEAN, R, D, -1.0, 9.81)
    close(v["center_z"], ZMEAN - D / 2)
    close(v["wall_z"], ZMEAN + D / 2)
    close(v["angular_velocity_rad_s"] ** 2, 2 * 9.81 * D / R ** 2)
    close(v["vtheta_peak_m_s"], v["angular_velocity_rad_s"] * R)
    close(v["equivalent_rigid_body_rpm"], 203.40092931205768)
    flat = S.vortex_surface_geometry("parabolic_vortex", ZMEAN, R, 0.0, -1.0, 9.81)
    close([flat["center_z"], flat["wall_z"], flat["angular_velocity_rad_s"]], [ZMEAN, ZMEAN, 0.0])


def test_scully_geometry():
    vg = S.vortex_surface_geometry("localized_scully_vortex", ZMEAN, R, D, CORE)
    close([vg["center_z"], vg["wall_z"], vg["angular_velocity_rad_s"], vg["equivalent_core_rpm"]],
          [0.010106395724732792, 0.060106395724732795, 53.90912787903789, 514.7942507833191])


def test_parabolic_stokes_analytic(lib):
    q = coefficients(lib, "stokes_drift_diffusion", "parabolic_vortex", 2048, 257)
    tau = 2600.0 * DIAM * DIAM / (18 * 8.9e-4)
    a = tau * (2 * 9.81 * D / R ** 2) / (2 * DT)
    close(q["A"], a)
    close(q["radial_log"][:, 0], -a * R ** 2)
    close(q["radial_log"][:, -1], 0.0, atol=0.0)
    assert np.all(np.diff(q["radial_log"], axis=1) >= -1e-14)


def _volume_mean(q, surface, transport, n=32768):
    """The validation script's independent volume mean of the normalised field (:112-140)."""
    r = (np.arange(n, dtype=np.float64) + 0.5) * R / n
    if surface == "parabolic_vortex":
        zs = ZMEAN + D * (r * r / R ** 2 - 0.5)
    else:
        vg = S.vortex_surface_geometry(surface, ZMEAN, R, D, CORE)
        zs = ZMEAN - vg["h_bar"] + vg["h_inf"] * r * r / (CORE * CORE + r * r)
    h = zs - ZMIN
    if transport == "stokes_drift_diffusion" and surface == "parabolic_vortex":
        log_r = q["A"][:, None] * (r[None, :] ** 2 - R ** 2)
    else:
        log_r = np.vstack([np.interp(r, q["r"], row) for row in q["radial_log"]])
    b = q["B"][:, None]
    iz = np.where(np.abs(b) < 1e-14, h[None, :], -np.expm1(-b * h[None, :]) / b)
    avg = 2 / (R * R * (ZMEAN - ZMIN)) * np.sum(r[None, :] * np.exp(log_r) * iz, axis=1) * (R / n)
    return avg / q["norm"]


@pytest.mark.parametrize("transport", ["stokes_drift_diffusion", "schiller_naumann_drift_diffusion"])
def test_parabolic_normalization(lib, transport):
    q = coefficients(lib, transport, "parabolic_vortex", 4096, 513)
    assert np.all(np.isfinite(q["norm"])) and np.all(q["norm"] > 0)
    assert np.all(q["radial_log"] <= 1e-14)
    close(_volume_mean(q, "parabolic_vortex", transport), 1.0, rtol=3e-4, atol=3e-6)


def test_parabolic_schiller_slip(lib):
    """The finite-Re radial slip at the wall (its largest value) solves w (1 + 0.15 Re^0.687) = tau omega^2 R."""
    q = coefficients(lib, "schiller_naumann_drift_diffusion", "parabolic_vortex", 8192, 2049)
    w = q["radial_slip"].max(axis=1)
    close(w, q["radial_slip"][:, -1], rtol=0, atol=0)
    re = 997.0 * DIAM * w / 8.9e-4
    tau = 2600.0 * DIAM * DIAM / (18 * 8.9e-4)
    drive = tau * (2 * 9.81 * D / R ** 2) * R
    close(w * (1 + 0.15 * re ** 0.687), drive, rtol=3e-12, atol=1e-15)


def test_scully_coefficients(lib):
    qs = coefficients(lib, "stokes_drift_diffusion", "localized_scully_vortex", 512, 129)
    close(qs["A"], [9.43333905e-05, 0.00943333905, 0.943333905], rtol=5e-09)
    close(qs["radial_log"][:, 0], [-7.96067416e-05, -0.00796067416, -0.796067416], rtol=5e-09)
    q = coefficients(lib, "schiller_naumann_drift_diffusion", "localized_scully_vortex", 512, 129)
    close(q["ws"], [9.81600492e-07, 9.8024982e-05, 0.00856690624], rtol=5e-09)
    close(q["A"], [9.43249639e-05, 0.0094106463, 0.767242433], rtol=5e-09)
    close(q["norm"], [0.99991352, 0.9914242, 0.50525183], rtol=2e-08)
    close(q["radial_log"][:, 0], [-7.95996304e-05, -0.00794152404, -0.647466075], rtol=5e-09)
    close(q["radial_log"][2, [0, 32, 64, 96, 128]],
          [-0.6474660749782518, -0.4573880863269777, -0.21780269501287686, -0.07669369764286141, 0.0], rtol=5e-12)
    logw = np.array([np.interp(0.95 * R, q["r"], row) for row in q["radial_log"]])
    close(np.exp(logw) / q["norm"], [1.0000851691924935, 1.008516884202098, 1.9556481703857034], rtol=5e-12)


def _velocity(lib, fsm, r, z, upeak):
    uz = C.c_double()
    ur = lib.clo_meridional_velocity(fsm, float(r), float(z), ZMIN, ZMEAN, R, D, CORE, float(upeak), C.byref(uz))
    return ur, uz.value


def test_scully_meridional_velocity(lib):
    vg = S.vortex_surface_geometry("localized_scully_vortex", ZMEAN, R, D, CORE)
    upeak = 0.05 * vg["vtheta_peak_m_s"]
    got = np.array([_velocity(lib, 2, r, z, upeak) for r, z in zip([0.0, 0.01, 0.03, R], [-0.05, 0.0, 0.02, 0.05])])
    close(got[:, 0], [0.0, -0.00263629, -0.00217236, 0.0], rtol=2e-06, atol=2e-09)
    close(got[:, 1], [-0.02621261, -0.01772844, 0.00121733, 0.0], rtol=2e-06, atol=2e-09)


def test_parabolic_meridional_velocity(lib):
    vg = S.vortex_surface_geometry("parabolic_vortex", ZMEAN, R, D, -1.0)
    close(vg["vtheta_peak_m_s"], math.sqrt(2 * 9.81 * D / R ** 2) * R)
    upeak = 0.05 * vg["vtheta_peak_m_s"]
    r = np.linspace(0.0, R, 64)
    surface = ZMEAN + D * (r * r / R ** 2 - 0.5)
    bottom = np.array([_velocity(lib, 1, rr, ZMIN, upeak) for rr in r])
    top = np.array([_velocity(lib, 1, rr, zz, upeak) for rr, zz in zip(r, surface)])
    close(bottom[:, 1], 0.0, atol=2e-15)
    close(bottom[[0, -1], 0], 0.0, atol=2e-15)
    close(top[:, 1] - 2 * D * r / R ** 2 * top[:, 0], 0.0, atol=2e-13)  # flow along the free surface
    still = np.array([_velocity(lib, 1, rr, 0.5 * (ZMIN + zz), 0.0) for rr, zz in zip(r, surface)])
    close(still, 0.0, atol=0.0)
    rr, zz, h = 0.021, 0.0, 1e-06  # incompressible: (1/r) d(r ur)/dr + duz/dz = 0
    div = ((_velocity(lib, 1, rr + h, zz, upeak)[0] - _velocity(lib, 1, rr - h, zz, upeak)[0]) / (2 * h)
           + _velocity(lib, 1, rr, zz, upeak)[0] / rr
           + (_velocity(lib, 1, rr, zz + h, upeak)[1] - _velocity(lib, 1, rr, zz - h, upeak)[1]) / (2 * h))
    assert abs(div) < 2e-07, div


def test_free_surface_height_and_normal(lib):
    """The parabolic surface at r = 0 and 20 mm (the validation script's device geometry check, :1130-1160)."""
    lib.clo_surface.restype = C.c_float
    lib.clo_surface.argtypes = [C.c_int] + [C.c_float] * 6 + [C.c_void_p]
    zs, normals = [], []
    for x in (0.0, 0.02):
        n = np.zeros(3, np.float32)
        zs.append(lib.clo_surface(1, x, 0.0, ZMEAN, R, D, CORE, n.ctypes.data_as(C.c_void_p)))
        normals.append(n.astype(np.float64))
    close(zs, ZMEAN + D * (np.array([0.0, 0.02]) ** 2 / R ** 2 - 0.5), rtol=3e-06, atol=3e-07)
    slopes = 2 * D * np.array([0.0, 0.02]) / R ** 2
    want = np.column_stack([slopes, np.zeros(2), -np.ones(2)])
    want /= np.linalg.norm(want, axis=1)[:, None]
    close(np.abs(normals), np.abs(want), rtol=4e-06, atol=3e-07)
    assert np.all(np.sign(np.asarray(normals)[:, 2]) == np.sign(np.asarray(normals)[0, 2]))


@pytest.mark.parametrize("transport", ["stokes_drift_diffusion", "schiller_naumann_drift_diffusion"])
def test_trace_field_lookup_matches_coefficients(lib, transport):
    """The concentration scale the trace looks up (FP32 position, radial lookup, vertical decay) against the
    coefficients it comes from, at the bottom and the beam plane on the axis and at 0.95 R (:1161-1225)."""
    lib.clo_local_scale.restype = C.c_double
    lib.clo_local_scale.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float]
    cfg = S.ModelConfig(free_surface_model="parabolic_vortex", vortex_wall_center_height_difference_m=D,
                        vortex_core_radius_m=CORE, sediment_transport_model=transport)
    sp = cfg.to_scene_params()
    ps = S.Particles(DIAM, np.ones(3), np.full(3, 1.54), np.zeros(3), 1.0, 2600.0).spec(cfg)
    ss = cfg.sediment_spec()
    ss.particle_density, ss.water_density, ss.water_viscosity, ss.gravity = 2600.0, 997.0, 8.9e-4, 9.81
    ss.eddy_diffusivity, ss.n_quad, ss.n_radial = DT, 512, 129
    ss.rin, ss.zmin, ss.zmean, ss.vortex_delta_h, ss.vortex_core_radius = R, ZMIN, ZMEAN, D, CORE
    h = C.c_void_p()
    assert lib.clo_prepare(C.byref(sp), C.byref(ps), C.byref(ss), C.byref(h)) == 0
    b, norm = np.zeros(3), np.zeros(3)
    rl = np.zeros((3, 129))
    lib.clo_read_sediment(h, None, b.ctypes.data_as(C.c_void_p), norm.ctypes.data_as(C.c_void_p), None,
                          rl.ctypes.data_as(C.c_void_p), None)
    xyz = np.array([[0.0, 0.0, -0.093], [0.95 * R, 0.0, -0.093], [0.0, 0.0, 0.0], [0.95 * R, 0.0, 0.0]], np.float32)
    rn = np.linspace(0.0, R, 129)
    for p in range(3):
        got = np.array([lib.clo_local_scale(h, p, *map(float, q)) for q in xyz])
        log_r = np.array([np.interp(float(q[0]), rn, rl[p]) for q in xyz])
        want = np.exp(log_r - b[p] * (xyz[:, 2].astype(np.float64) + 0.093)) / norm[p]
        close(got, want, rtol=2e-05, atol=2e-07)
        assert np.max(got) <= (1.0 / norm[p]) * (1 + 3e-06)
    lib.clo_free(h)


def test_meridional_liquid_cells():
    """Cells of a 16 x 32 (r, z) grid are liquid exactly below the parabolic surface (:1265-1289)."""
    lib, _ = H.load("port")
    lib.clo_meridional_fluid.restype = C.c_int
    lib.clo_meridional_fluid.argtypes = [C.c_int] + [C.c_double] * 7
    nr, nz, ztop = 16, 32, 0.074
    rr = (np.arange(nr) + 0.5) * R / nr
    zz = ZMIN + (np.arange(nz) + 0.5) * (ztop - ZMIN) / nz
    got = np.array([[lib.clo_meridional_fluid(1, r, z, ZMIN, ZMEAN, R, D, CORE) for z in zz] for r in rr], bool)
    want = zz[None, :] < ZMEAN + D * (rr[:, None] ** 2 / R ** 2 - 0.5)
    np.testing.assert_array_equal(got, want)
