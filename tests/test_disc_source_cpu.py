"""CPU: the collimated disc beam (this library's source option; the reference has only its LED,
CLARITAS/CLARITAS.py:4650-4697) in the CPU restatement.

A uniform 2 mm disc launched along +y at the sensor-ring radius has no collimator to pass: no photon is
rejected at the source, and in a cell without particles nearly every photon crosses the tube and reaches
the transmitted (0 degree) detector, losing only Fresnel reflections at the six interfaces.
"""
from __future__ import annotations

import oracle_harness as H
from tardiis_and_claritas_gb300 import scene as S


def test_disc_beam_in_a_clear_cell():
    cfg, _, _, _ = S.small_plain_workload()
    assert cfg.source_kind == "collimated_disc"
    parts = S.quartz_particles(1e-6)
    o = H.OracleRun("port", cfg, parts)
    n = 200_000
    t, _ = o.trace(S.run_params(n, seed=5))
    o.close()
    assert t["status_counts"][3] == 0            # nothing rejected at a source without collimator
    assert t["status_counts"].sum() == n
    frac0 = t["hw_native"][0] / n
    assert 0.80 < frac0 < 0.97, frac0          # transmitted, less the Fresnel losses
    assert t["hw_native"][1:].sum() < 0.02 * n  # no particles: hardly anything off axis
