"""CPU: the batched-sweep scenario sampler (seeded, with the sweep's parameter ranges)."""
from __future__ import annotations

import numpy as np

from tardiis_and_claritas_gb300 import scene as S


def test_sampler_is_seeded_and_in_range():
    a = S.sweep_workload(512)
    b = S.sweep_workload(512)
    assert [x.params for x in a] == [x.params for x in b]
    assert [x.n_photons for x in a] == [x.n_photons for x in b]
    p = {k: np.array([x.params[k] for x in a]) for k in a[0].params}
    n = np.array([x.n_photons for x in a])
    assert n.min() >= 1e5 and n.max() <= 1e7 and 0.9e9 < n.sum() < 1.5e9
    assert p["concentration_mg_l"].min() >= 1.0 and p["concentration_mg_l"].max() <= 1e4
    assert p["median_um"].min() >= 2.0 and p["median_um"].max() <= 200.0
    assert p["sigma_g"].min() >= 1.2 and p["sigma_g"].max() <= 2.0
    assert p["rpm"].min() >= 0.0 and p["rpm"].max() <= 1200.0
    assert p["n_particle"].min() >= 1.5 and p["n_particle"].max() <= 1.6
    assert [x.seed for x in a] == list(range(512))
    # log-uniform draws: the median of log10(photons) sits near the middle of [5, 7]
    assert abs(np.median(np.log10(n)) - 6.0) < 0.15
    assert S.sweep_workload(8, sampler_seed=1)[0].params != a[0].params


def test_sweep_specs_follow_each_scenario():
    scs = S.sweep_workload(4, sampler_seed=2)
    scenes, parts, seds = S.sweep_specs(scs)
    for sc, sp, ps in zip(scs, scenes, parts):
        assert ps.n_bins == 64 and ps.n_theta == 1801
        assert abs(ps.n_real[0] - sc.params["n_particle"]) == 0.0
        assert abs(ps.concentration_kg_m3 - sc.params["concentration_mg_l"] * 1e-3) < 1e-15
        assert sp.sediment_model == 0
        if sc.params["rpm"] > 0:
            assert sp.free_surface_model == 2 and sp.vortex_delta_h > 0
