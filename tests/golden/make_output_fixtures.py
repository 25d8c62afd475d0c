"""Golden outputs of the reference's own per-case writers (run where the reference checkout is).

Calls the reference's ``_write_detector_outputs`` (CLARITAS/CLARITAS.py:12653-12696) and ``_summary_dict``
(:12849-12971) on seeded synthetic results, and ``_resolve_model_kwargs`` (the constructor keywords its
batch driver builds the model from), and stores inputs and outputs in ``output_fixtures.json`` beside this
script: the CSV text, the error each corrupted result raises, and the summary dictionary after the
reference's JSON sanitiser. The reference module imports without CuPy. Usage:
python tests/golden/make_output_fixtures.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
from pathlib import Path
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
from ref_extract import reference_root  # noqa: E402


def synthetic_result(seed: int, n_angles: int = 18) -> dict:
    """Plain-data fields of a ForwardResult, enough for both writers."""
    rng = np.random.default_rng(seed)
    native = rng.poisson(rng.uniform(0.0, 4000.0, n_angles)).astype(np.int64)
    mirror = rng.poisson(rng.uniform(0.0, 4000.0, n_angles)).astype(np.int64)
    score = 0.5 * (native + mirror).astype(float)
    frac = rng.dirichlet(np.ones(6), size=n_angles).T  # 6 interaction orders per angle
    order = frac * score[None, :]
    order[5] = score - order[:5].sum(axis=0)
    norm = score / max(score.max(), 1.0)
    jk = rng.uniform(0.0, 0.05, n_angles)
    jk[3] = np.nan  # a channel without a jackknife estimate
    n_rays = int(rng.integers(10_000, 10_000_000))
    return {
        "n_rays": n_rays, "requested_n_rays": n_rays + int(rng.integers(0, 1000)),
        "hardware_symmetry_scores": score.tolist(), "normalized_hardware_symmetry_response": norm.tolist(),
        "hardware_normalized_jackknife_se": [None if not np.isfinite(v) else float(v) for v in jk],
        "hardware_native_hits": native.tolist(), "hardware_mirror_hits": mirror.tolist(),
        "exact_particle_order_scores": order.tolist(),
        "stop_reason": "target_rays_reached", "production_failure_count": int(rng.integers(0, 5)),
        "entered_water_fraction": float(rng.uniform()), "air_exit_fraction": float(rng.uniform()),
        "axial_loss_fraction": float(rng.uniform()), "detector_detection_fraction": float(rng.uniform()),
        "mean_interactions": float(rng.uniform(0, 3)), "mean_geometric_interactions": float(rng.uniform(0, 2)),
        "mean_wave_interactions": float(rng.uniform(0, 1)), "mu_geom_per_m": float(rng.uniform(0, 50)),
        "mu_wave_per_m": float(rng.uniform(0, 50)), "mu_event_per_m": float(rng.uniform(0, 90)),
        "mu_sca_per_m": 40.0 + float(rng.uniform(0, 5)), "mu_ext_per_m": 45.0 + float(rng.uniform(0, 5)),
        "optical_depth_diameter": float(rng.uniform(0, 9)),
        "geometric_optical_depth_diameter": float(rng.uniform(0, 9)),
        "sediment_transport_model": "schiller_naumann_meridional_advection_diffusion",
        "sediment_eddy_diffusivity_m2_s": 1e-4, "sediment_majorant_total_per_m": float(rng.uniform(1, 99)),
        "particle_event_model": "hybrid_mie_exact_rate",
        "closure": {"conditional_outcome_trials": int(rng.integers(0, 999)), "closed": True},
        "conditional_sampler_counts": {"accepted": int(rng.integers(0, 999)), "rejected": int(rng.integers(0, 99))},
        "particle_surface_rms_slope_deg": 6.0, "wave_surface_rms_height_nm": 25.0,
        "number_density_by_bin": rng.uniform(0, 1e9, 12).tolist(),
    }


def as_result(d: dict) -> SimpleNamespace:
    """The synthetic fields as the attribute object both writers read."""
    r = SimpleNamespace(**{k: v for k, v in d.items()
                           if k not in ("exact_particle_order_scores", "closure", "conditional_sampler_counts",
                                        "number_density_by_bin")})
    r.hardware_normalized_jackknife_se = [np.nan if v is None else v for v in d["hardware_normalized_jackknife_se"]]
    r.detector_particle_path_diagnostics = {"exact_particle_order_scores": np.asarray(d["exact_particle_order_scores"]),
                                            "closure": d["closure"],
                                            "conditional_sampler_counts": d["conditional_sampler_counts"]}
    r.particle_diagnostics = {"number_density_by_bin": d["number_density_by_bin"]}
    return r


# corruptions of a valid result and how each is applied
CORRUPTIONS = {
    "short_array": lambda d: d.update(hardware_native_hits=d["hardware_native_hits"][:-1]),
    "negative_score": lambda d: d["hardware_symmetry_scores"].__setitem__(4, -1.0),
    "open_partition": lambda d: d["exact_particle_order_scores"][2].__setitem__(7, d["exact_particle_order_scores"][2][7] + 5.0),
}


def main() -> None:
    sys.path.insert(0, os.path.join(reference_root(), "CLARITAS"))
    import CLARITAS as C  # noqa: N813

    cases = []
    for case, (material, conc, wl, seed) in enumerate((("loess", 0.5, 860.0, 7), ("kaolin", 2.25, 650.0, 11))):
        d = synthetic_result(100 + case)
        res = as_result(d)
        with tempfile.TemporaryDirectory() as tmp:
            C._write_detector_outputs(Path(tmp), material, conc, wl, seed, res)
            csv_text = (Path(tmp) / "detector_response.csv").read_text(encoding="utf-8")
            kw, _, _ = C._resolve_model_kwargs(material, wl)
            summary = C._json_safe(C._summary_dict(material, conc, wl, seed, "GB300-test", 12.5, res,
                                                   res.particle_diagnostics, {"assumed": "test"}, Path(tmp)))
        errors = {}
        for name, corrupt in CORRUPTIONS.items():
            bad = json.loads(json.dumps(d))
            corrupt(bad)
            try:
                with tempfile.TemporaryDirectory() as tmp:
                    C._write_detector_outputs(Path(tmp), material, conc, wl, seed, as_result(bad))
                errors[name] = None
            except Exception as e:  # the reference raises ValueError or its CaseIntegrityError
                errors[name] = [type(e).__name__, str(e)]
        cases.append({"args": [material, conc, wl, seed], "result": d, "csv": csv_text, "errors": errors,
                      "model_kwargs": C._json_safe({k: v for k, v in kw.items()
                                                     if k != "particle_optical_constants_by_material"}),
                      "summary": summary})
    with open(os.path.join(HERE, "output_fixtures.json"), "w") as f:
        json.dump({"cases": cases}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
