"""GPU: the forward-model facade (ClaritasForwardModel.simulate) against direct traces.

With the reference's streams the facade's batches (statistics_batch_rays each, traced together
through clr_trace_batch) must add up to one direct trace over the same global ray range, the
normalized responses and per-batch rows must follow from the tallies, and adaptive stopping must
stop at the first batch that meets the target (the reference's rule)."""
from __future__ import annotations

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import forward as F, scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model():
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    kw = {k: v for k, v in S.small_cell_config().__dict__.items() if k not in ("source_kind", "disc_beam_radius_m")}
    kw["statistics_batch_rays"] = 50_000
    m = F.ClaritasForwardModel(rng="reference", **kw)
    m.register_material("quartz", S.quartz_particles(1.0, n_bins=32))
    yield m
    m.close()


def test_simulate_equals_direct_trace(model):
    res = model.simulate("quartz", 1.0, n_rays=300_000, seed=77, ray_id_start=1000)
    ctx = model._context()
    direct, _ = ctx.trace(S.run_params(300_000, seed=77, ray_offset=1000))
    np.testing.assert_array_equal(res.hardware_native_hits, direct["hw_native"])
    np.testing.assert_array_equal(res.hardware_mirror_hits, direct["hw_mirror"])
    np.testing.assert_array_equal(res.legacy_native_channel_counts, direct["legacy_native"])
    assert res.n_rays == 300_000 and res.stop_reason == "fixed_n_rays" and len(res.batch_diagnostics) == 6
    assert abs(res.normalized_hardware_symmetry_response.sum() - 1.0) < 1e-12
    assert np.all(np.isfinite(res.hardware_normalized_jackknife_se))
    assert res.entered_water_fraction == direct["ray_flags"][0] / 300_000
    assert res.production_failure_count == int(direct["failure_code_counts"][1:].sum())
    assert res.mu_event_per_m > 0 and res.optical_depth_diameter > 0


def test_adaptive_stop_is_the_first_batch_meeting_the_target(model):
    res = model.simulate("quartz", 1.0, n_rays=50_000, seed=5, target_detector_score=2000.0, max_rays=1_000_000)
    assert res.stop_reason == "target_detector_score" and res.stopped_adaptively
    rows = res.batch_diagnostics
    assert rows[-1]["cumulative_selected_score"] >= 2000.0
    assert len(rows) == 1 or rows[-2]["cumulative_selected_score"] < 2000.0
    fixed = model.simulate("quartz", 1.0, n_rays=res.n_rays, seed=5)
    np.testing.assert_array_equal(fixed.hardware_native_hits, res.hardware_native_hits)


@pytest.mark.parametrize("material", ["loess", "kaolin"])
def test_named_material_default_call(material):
    """The reference's default call with a named material (run_one_case, CLARITAS.py:13020): the bundled
    PSD and per-bin n/k give the CPU restatement's physics tables, and the GPU facade's tallies agree with
    the facade driven through the CPU restatement (reference streams) within binomial errors."""
    import oracle_harness as H
    from test_forward_cpu import _OracleContext
    kw = dict(sediment_transport_model="uniform", free_surface_model="flat", vortex_wall_center_height_difference_m=0.0,
              statistics_batch_rays=250_000)
    g = F.ClaritasForwardModel(**kw)
    prep = g._prepare_gpu_particle_physics(material, 0.5)
    c = F.ClaritasForwardModel(rng="reference", **kw)
    ctx = _OracleContext()
    ctx.set_scene(c.config.to_scene_params())
    c._ctx = ctx
    cprep = c._prepare_gpu_particle_physics(material, 0.5)
    for k in ("qext", "qsca", "phase_cdf"):
        np.testing.assert_allclose(prep["device"][k], cprep["device"][k], rtol=1e-9, atol=1e-12, err_msg=k)
    n_g, n_c = 2_000_000, 200_000
    rg = g.simulate(material, 0.5, n_rays=n_g, seed=11)
    rc = c.simulate(material, 0.5, n_rays=n_c, seed=12)
    g.close()
    for a, b in ((rg.hardware_native_hits, rc.hardware_native_hits), (rg.hardware_mirror_hits, rc.hardware_mirror_hits)):
        a, b = np.asarray(a, float), np.asarray(b, float)
        p = (a + b) / (n_g + n_c)
        se = np.maximum(np.sqrt(p * (1 - p) * (1 / n_g + 1 / n_c)), 1.0 / (n_g + n_c))
        z = np.abs(a / n_g - b / n_c) / se
        assert z.max() < 4.5 and np.sum(z > 3.0) <= 1, np.round(z, 2)
