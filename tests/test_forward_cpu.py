"""CPU tests of the forward-model facade: restated reference helpers against golden vectors made
by the reference's own functions (tests/golden/make_forward_fixtures.py), configuration handling,
and explicit rejection of features outside the library."""
from __future__ import annotations

import os

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import forward as F, materials as M, scene as S

GOLD = os.path.join(os.path.dirname(__file__), "golden", "forward_fixtures.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.mark.parametrize("case", range(5))
def test_jackknife_matches_reference(gold, case):
    got = F.jackknife_normalized_se(list(gold[f"jk_in_{case}"]))
    np.testing.assert_allclose(got, gold[f"jk_out_{case}"], rtol=1e-12, atol=0, equal_nan=True)


@pytest.mark.parametrize("case", range(6))
def test_histogram_median_matches_reference(gold, case):
    got = F.histogram_median(gold[f"med_in_{case}"])
    want = float(gold[f"med_out_{case}"])
    assert (np.isnan(got) and np.isnan(want)) or got == want


def test_model_takes_reference_keywords_and_validates():
    m = F.ClaritasForwardModel(particle_event_model="geometric", symmetry_average_exact=False)
    assert m.particle_event_model == "geometric" and m.symmetry_average_exact is False
    with pytest.raises(ValueError):
        F.ClaritasForwardModel(legacy_detector_acceptance_deg=95.0)
    with pytest.raises(ValueError):
        F.ClaritasForwardModel(rng="mersenne")


def test_unsupported_features_raise_explicitly():
    m = F.ClaritasForwardModel()
    parts = S.quartz_particles(100.0, n_bins=4)
    # light diagnostics are validated with the reference's rules before anything reaches the device
    with pytest.raises(ValueError, match="max_rays must be >=1"):
        m.simulate(parts, 0.1, n_rays=10, light_transport_config={"enabled": True, "nx": 8, "ny": 8, "nz": 8})
    with pytest.raises(ValueError, match="grid dimensions"):
        m.simulate(parts, 0.1, n_rays=10, light_transport_config={"enabled": True, "max_rays": 5, "nx": 3})
    with pytest.raises(ValueError, match="representative-ray"):
        m.simulate(parts, 0.1, n_rays=10, light_transport_config={"enabled": True, "max_rays": 5, "nx": 4, "ny": 4,
                                                                 "nz": 4})
    with pytest.raises(ValueError, match="heatmap_size"):
        m.simulate(parts, 0.1, n_rays=10, heatmap_size=-1)
    with pytest.raises(NotImplementedError):
        m.simulate(parts, 0.1, n_rays=10, collect_rays=True)
    with pytest.raises(ValueError, match="material must be 'loess' or 'kaolin'"):
        m.simulate("basalt", 0.1, n_rays=10)
    with pytest.raises(ValueError, match="ray_id_start"):
        m.simulate(parts, 0.1, n_rays=10, ray_id_start=2 ** 32)


def test_registered_material_takes_weights_on_its_grid():
    m = F.ClaritasForwardModel()
    parts = S.quartz_particles(100.0, n_bins=5)
    m.register_material("sand", parts)
    p = m._particles("sand", 0.5, [1, 2, 3, 4, 5], "number_fraction")
    assert p.concentration_kg_m3 == 0.5 and p.weight_mode == "number_fraction"
    np.testing.assert_array_equal(p.weight, [1, 2, 3, 4, 5])
    with pytest.raises(ValueError, match="weights must have 5 entries"):
        m._particles("sand", 0.5, [1, 2], "mass_fraction")


def test_path_diagnostics_report_every_partition():
    """The facade turns the device partitions into the reference's path-diagnostics keys: mask scores and
    fractions of the hard-aperture score, the closure errors, acrylic-reflection order (CLARITAS.py:8968-9161)."""
    from tardiis_and_claritas_gb300 import abi
    rng = np.random.default_rng(1)
    m = F.ClaritasForwardModel()
    tot = {"order_hits": rng.integers(0, 50, (2, 6, 18)), "geometric_order_hits": rng.integers(0, 50, (2, 6, 18)),
           "path_sums": rng.integers(0, 50, (abi.N_PATH_SUMS, 2, 18)),
           "path_mask_hits": rng.integers(0, 50, (2, abi.N_PATH_MASKS, 18)),
           "acrylic_order_hits": rng.integers(0, 50, (2, 5, 18)), "conditional_stats": np.zeros(10, np.uint64)}
    denp = 0.5 * (tot["order_hits"][0] + tot["order_hits"][1]).sum(axis=0)
    denp[3] = 0.0
    pd = m._path_diagnostics(tot, denp, True)
    mask = 0.5 * (tot["path_mask_hits"][0] + tot["path_mask_hits"][1])
    for k, name in enumerate(abi.PATH_MASK_NAMES):
        np.testing.assert_array_equal(pd[name + "_scores"], mask[k])
        assert pd[name + "_fraction"][3] == 0.0
    i = abi.PATH_MASK_NAMES.index
    np.testing.assert_allclose(pd["interaction_order_partition_closure_error_scores"],
                               mask[i("any_particle")] - mask[[i("single_interaction"), i("interaction_order_2"),
                                                              i("interaction_order_3"),
                                                              i("interaction_order_4plus")]].sum(axis=0))
    acr = 0.5 * (tot["acrylic_order_hits"][0] + tot["acrylic_order_hits"][1])
    np.testing.assert_array_equal(pd["acrylic_reflection_order_scores"], acr)
    np.testing.assert_allclose(pd["acrylic_reflection_order_partition_closure_error_scores"], denp - acr.sum(axis=0))
    assert pd["acrylic_reflection_order_labels"] == ["0", "1", "2", "3", "4+"]
    native = m._path_diagnostics(tot, denp, False)
    np.testing.assert_array_equal(native["any_wave_scores"], tot["path_mask_hits"][0][i("any_wave")])


def test_provenance_diagnostics_from_device_partitions():
    """The causal outputs of the path diagnostics (CLARITAS.py:9008-9091, :9135-9150) from the device's
    provenance partitions: bin scores cut to the material's bins, per-type scores and fractions, closures."""
    from tardiis_and_claritas_gb300 import abi
    rng = np.random.default_rng(2)
    m = F.ClaritasForwardModel()
    m._physics = {"radius": np.zeros(5)}
    pv = {"bin_hits": np.zeros((6, 2, 64, 18), np.int64), "first_type_hits": rng.integers(0, 9, (2, 8, 18)),
          "last_type_hits": rng.integers(0, 9, (2, 8, 18)), "wall_hits": rng.integers(0, 9, (2, 3, 18)),
          "after_return_hits": rng.integers(0, 9, (2, 18)), "first_backscatter_hits": rng.integers(0, 9, (2, 18)),
          "first_source_hemisphere_hits": rng.integers(0, 9, (2, 18)),
          "first_angle_sum": rng.uniform(0, 90, (2, 18)), "first_angle_count": rng.integers(0, 3, (2, 18)),
          "last_angle_sum": rng.uniform(0, 90, (2, 18)), "last_angle_count": rng.integers(0, 3, (2, 18)),
          "last_type_angle_sum": rng.uniform(0, 90, (2, 8, 18)), "last_type_angle_count": rng.integers(0, 3, (2, 8, 18)),
          "h170_last_angle_hits": rng.integers(0, 9, (2, 8, 6)), "h170_first_angle_hits": rng.integers(0, 9, (2, 6))}
    pv["bin_hits"][0, :, :5] = rng.integers(0, 9, (2, 5, 18))
    sym = lambda a, b: 0.5 * (a + b)  # noqa: E731
    denp = rng.uniform(50, 100, 18)
    anyp = sym(pv["bin_hits"][0, 0], pv["bin_hits"][0, 1]).sum(axis=0)
    out = m._provenance_diagnostics(pv, denp, anyp, sym)
    assert out["first_particle_bin_scores"].shape == (5, 18)
    assert np.all(out["first_particle_bin_partition_closure_error_scores"] == 0.0)
    for code, name in abi.PARTICLE_EVENT_TYPE_NAMES.items():
        want = sym(pv["last_type_hits"][0, code], pv["last_type_hits"][1, code])
        np.testing.assert_array_equal(out[f"last_event_{name}_scores"], want)
        np.testing.assert_allclose(out[f"last_event_{name}_fraction"], want / denp)
    cnt = sym(pv["first_angle_count"][0], pv["first_angle_count"][1])
    mean = out["mean_first_particle_deflection_deg_by_channel"]
    assert np.all(np.isnan(mean[cnt == 0])) and np.all(np.isfinite(mean[cnt > 0]))
    assert set(out["wall_path_scores"]) == set(abi.WALL_PATH_NAMES)
    assert out["H170_last_event_angle_histogram_scores_by_event_code"].shape == (8, 6)


@pytest.mark.parametrize("override", [
    dict(free_surface_model="unknown", vortex_wall_center_height_difference_m=0.05),
    dict(free_surface_model="parabolic_vortex", vortex_wall_center_height_difference_m=-0.01),
    dict(free_surface_model="parabolic_vortex", vortex_wall_center_height_difference_m=float("nan")),
    dict(sediment_eddy_diffusivity_m2_s=0.0), dict(water_density_kg_per_m3=2700.0),
    dict(water_dynamic_viscosity_pa_s=0.0), dict(gravity_m_s2=float("inf")), dict(meridional_circulation_ratio=0.6),
    dict(meridional_grid_nr=8), dict(meridional_solver_check_interval=5), dict(meridional_solver_tolerance=0.1),
    dict(meridional_solver_sor=1.95), dict(aggregation_model="bogus"), dict(aggregation_collision_exposure=-1.0),
    dict(fragmentation_size_exponent=7.0), dict(fragmentation_breakup_exposure=1.0),
    dict(aggregation_step_safety=0.3), dict(aggregation_max_steps=0),
])
def test_fail_closed_configuration(override):
    """Invalid settings are refused at construction, as in the reference's fail-closed configuration test
    (CLARITAS/validate_claritas.py:437-551) and constructor (CLARITAS.py:5754-5999)."""
    with pytest.raises(ValueError):
        S.ModelConfig(**override).validate()


def test_vortex_geometry_rejects_degenerate_inputs():
    for radius in (0.0, float("nan")):
        with pytest.raises(ValueError):
            S.vortex_surface_geometry("parabolic_vortex", 0.05, radius, 0.05, -1.0)
    with pytest.raises(ValueError):
        S.vortex_surface_geometry("parabolic_vortex", 0.05, 1e-300, 1e300, -1.0)
    with pytest.raises(ValueError):
        S.vortex_surface_geometry("localized_scully_vortex", 0.05, 0.0465, 0.05, 1e-200)


class _OracleContext:
    """A stand-in for lib.Context that prepares scenes in the CPU oracle (facade tests without a GPU)."""

    def __init__(self):
        import oracle_harness as H
        self.lib, _ = H.load("port")
        self.h = None

    def set_scene(self, sp):
        self.sp = sp

    def build_particles(self, ps, ss):
        import ctypes as C
        self.h = C.c_void_p()
        assert self.lib.clo_prepare(C.byref(self.sp), C.byref(ps), C.byref(ss), C.byref(self.h)) == 0
        self.n_bins, self.n_theta = int(ps.n_bins), self.lib.clo_n_theta(self.h)

    def physics(self):
        import ctypes as C
        from tardiis_and_claritas_gb300 import abi
        pp, arrays = abi.alloc_physics(self.n_bins, self.n_theta)
        self.lib.clo_read_physics(self.h, C.byref(pp))
        return arrays

    def set_light(self, enabled=False, **kw):
        assert not enabled and not kw.get("heatmap_size"), "light diagnostics are not restated by the oracle"

    def set_provenance(self, enabled):
        self.prov_on = bool(enabled)

    def read_provenance(self):
        return self.prov_acc

    def close(self):
        if self.h:
            self.lib.clo_free(self.h)
            self.h = None

    def trace_batch(self, runs):
        """Each run through the oracle, with the device-only partitions filled from its per-ray outputs
        (the same partitions the device counts)."""
        import ctypes as C
        import provenance_partitions as PP
        from tardiis_and_claritas_gb300 import abi
        from path_partitions import partitions_from_records
        out = []
        self.prov_acc = None
        for run in runs:
            n = int(run.n_rays)
            T = abi.Tallies()
            rec = np.zeros(n, dtype=abi.record_dtype())
            prov = np.zeros((n, 13), np.int32)
            defl = np.zeros((n, 5), np.float32)
            f = self.lib.clo_trace_provenance
            assert f(self.h, C.byref(run), C.byref(T), rec.ctypes.data_as(C.c_void_p),
                     prov.ctypes.data_as(C.c_void_p), defl.ctypes.data_as(C.c_void_p), 0) == 0
            t = T.as_dict()
            order, gorder, sums, masks, acr = partitions_from_records(rec)
            t.update(order_hits=order, geometric_order_hits=gorder, path_sums=sums, path_mask_hits=masks,
                     acrylic_order_hits=acr)
            out.append(t)
            if self.prov_on:
                p = PP.partitions(rec["interaction_count"], rec["native_id"], rec["mirror_id"], prov, defl[:, :2])
                p.pop("causal_path_count", None)
                self.prov_acc = p if self.prov_acc is None else {k: self.prov_acc[k] + p[k] for k in p}
        return out

    def sediment_field(self):
        import ctypes as C
        f = self.lib.clo_read_sediment_field
        f.argtypes = [C.c_void_p, C.c_void_p] + [C.c_void_p] * 4
        nr, nz, it, res = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        f(self.h, None, C.byref(nr), C.byref(nz), C.byref(it), C.byref(res))
        g = np.zeros((self.n_bins, nr.value, nz.value))
        f(self.h, g.ctypes.data_as(C.c_void_p), None, None, None, None)
        return {"grid": g, "nr": nr.value, "nz": nz.value, "iterations": it.value, "max_residual": res.value}


@pytest.mark.parametrize("transport", ["schiller_naumann_drift_diffusion",
                                       "schiller_naumann_meridional_advection_diffusion"])
def test_prepare_returns_the_reference_structure(transport):
    """_prepare_gpu_particle_physics returns the reference's dict (CLARITAS.py:6931-6965): population arrays,
    device tables under its keys, host diagnostics under its keys."""
    m = F.ClaritasForwardModel(particle_event_model="hybrid_mie_excess", free_surface_model="parabolic_vortex",
                               vortex_wall_center_height_difference_m=0.05, sediment_transport_model=transport,
                               meridional_grid_nr=16, meridional_grid_nz=32)
    ctx = _OracleContext()
    ctx.set_scene(m.config.to_scene_params())
    m._ctx = ctx
    parts = S.quartz_particles(500.0, n_bins=8)
    out = m._prepare_gpu_particle_physics(parts, 0.5)
    assert set(out) == {"d", "w", "nidx", "kidx", "n", "device", "host", "ntheta"}
    assert out["n"] == 8 and out["ntheta"] == out["device"]["theta"].size == out["device"]["phase_cdf"].shape[1]
    dev, host = out["device"], out["host"]
    for k in ("radius", "n", "k", "gcdf", "wcdf", "phase_cdf", "theta", "qsca", "qext", "mu_channels",
              "trace_geom_bin", "trace_wave_bin", "sed_majorants"):
        assert k in dev, k
    np.testing.assert_allclose(host["scattering_cross_section_m2"],
                               host["qsca"] * np.pi * host["radius_m"] ** 2, rtol=1e-15)
    np.testing.assert_allclose(host["single_scattering_albedo"], host["qsca"] / host["qext"], rtol=1e-12)
    band = host["mie_phase_probability_165_175_by_bin"]
    assert band.shape == (8,) and np.all(band >= 0) and np.all(band < 1) and np.any(band > 0)
    assert np.all(host["mie_phase_probability_169_171_by_bin"] <= band)
    if transport.endswith("meridional_advection_diffusion"):
        assert dev["sed_grid"].shape == (8, 16, 32) and dev["sed_grid_nr"] == 16
        assert host["meridional_solver_iterations"] >= 1000
        assert host["meridional_solver_max_residual"] <= host["meridional_solver_tolerance"]
    else:
        assert "sed_grid" not in dev and "meridional_solver_iterations" not in host


def test_simulate_on_the_oracle_engine(tmp_path):
    """The whole facade on CPU: simulate() in statistics batches through a stand-in context that traces
    with the oracle (the reference's streams), the ForwardResult, its path diagnostics with every closure
    of the reference, and the per-case files with their integrity reports."""
    from tardiis_and_claritas_gb300 import outputs as O
    kw = {k: v for k, v in S.small_cell_config().__dict__.items() if k not in ("source_kind", "disc_beam_radius_m")}
    kw["statistics_batch_rays"] = 4096
    m = F.ClaritasForwardModel(rng="reference", **kw)
    ctx = _OracleContext()
    ctx.set_scene(m.config.to_scene_params())
    m._ctx = ctx
    m.register_material("quartz", S.quartz_particles(1.0, n_bins=16))
    res = m.simulate("quartz", 2.0, n_rays=16384, seed=3)
    assert res.n_rays == 16384 and res.production_failure_count == 0
    hw = 0.5 * (res.hardware_native_hits + res.hardware_mirror_hits)
    np.testing.assert_allclose(res.hardware_symmetry_scores, hw)
    assert hw.sum() > 0 and np.isfinite(res.hardware_normalized_jackknife_se[hw > 0]).all()
    pd = res.detector_particle_path_diagnostics
    for key in ("exact_particle_order", "exact_geometric_order", "interaction_order", "multiple_branch",
                "acrylic_reflection_order", "first_particle_bin", "last_particle_bin", "causal_last_event",
                "causal_first_event", "wall_path"):
        np.testing.assert_allclose(pd[key + "_partition_closure_error_scores"], 0.0, atol=1e-9, err_msg=key)
    assert pd["first_particle_bin_scores"].shape == (16, 18)
    np.testing.assert_allclose(pd["ballistic_scores"] + pd["any_particle_scores"], hw)
    rows = O.write_detector_outputs(tmp_path, "quartz", 2.0, 860.0, 3, res)
    assert len(rows) == 18
    d = O.write_run_summary(tmp_path, "quartz", 2.0, 860.0, 3, "CPU oracle", 1.0, res, m.config)
    assert d["production_integrity"]["status"] == "ok" and not d["production_integrity"]["fatal"]
    prod, diag = O.write_case_integrity(tmp_path, res)
    O.enforce_case_integrity(prod, diag)
    m.close()


def test_adaptive_simulate_on_the_oracle_engine():
    """The adaptive stopping rule (CLARITAS.py:8818-8880) over statistics batches: it stops at the first batch
    whose cumulative score reaches the target, and the provenance counts only the batches it kept."""
    kw = {k: v for k, v in S.small_cell_config().__dict__.items() if k not in ("source_kind", "disc_beam_radius_m")}
    kw["statistics_batch_rays"] = 2048
    m = F.ClaritasForwardModel(rng="reference", **kw)
    ctx = _OracleContext()
    ctx.set_scene(m.config.to_scene_params())
    m._ctx = ctx
    m.register_material("quartz", S.quartz_particles(1.0, n_bins=16))
    full = m.simulate("quartz", 2.0, n_rays=20480, seed=4)
    per_batch = full.hardware_symmetry_scores.sum() / 10
    res = m.simulate("quartz", 2.0, n_rays=2048, seed=4, target_detector_score=2.5 * per_batch, max_rays=20480)
    assert res.stopped_adaptively and res.n_rays % 2048 == 0 and 2048 <= res.n_rays < 20480
    assert res.hardware_symmetry_scores.sum() >= 2.5 * per_batch
    pd = res.detector_particle_path_diagnostics
    np.testing.assert_allclose(pd["wall_path_partition_closure_error_scores"], 0.0, atol=1e-9)
    np.testing.assert_allclose(pd["first_particle_bin_partition_closure_error_scores"], 0.0, atol=1e-9)
    m.close()


@pytest.mark.parametrize("material", ["loess", "kaolin"])
def test_named_material_runs_through_the_facade(material):
    """The reference's default call, simulate(material, concentration) with a named material (its run_one_case,
    CLARITAS.py:13020): the bundled PSD and optical constants, traced here through the CPU restatement."""
    m = F.ClaritasForwardModel(rng="reference", sediment_transport_model="uniform", free_surface_model="flat",
                               vortex_wall_center_height_difference_m=0.0)
    ctx = _OracleContext()
    ctx.set_scene(m.config.to_scene_params())
    m._ctx = ctx
    prep = m._prepare_gpu_particle_physics(material, 0.5)
    d, w = M.get_material_psd_raw(material)
    n, k = M.get_material_optical_constants(material)
    np.testing.assert_array_equal(prep["d"], d)
    np.testing.assert_array_equal(prep["nidx"], n)
    np.testing.assert_array_equal(prep["kidx"], k)
    r = m.simulate(material, 0.5, n_rays=20_000, seed=3)
    assert np.isfinite(r.normalized_hardware_symmetry_response).all() and r.hardware_native_hits.sum() > 0
