"""Generate the provenance golden fixtures from the reference's own code built for the host.

Run where the reference checkout is available (it is read, never modified):

    python oracle/ref_extract.py && python tests/golden/make_provenance_fixtures.py

The host build of the reference (oracle/_ref/libclaritas_ref_host.so) traces a few parity scenes on its
xorshift streams and returns its per-ray provenance outputs (first/last particle, geometric and wave bin,
first/last event type and deflection, acrylic returns); tests/provenance_partitions.py partitions the
detected rays as the reference's host does. tests/test_gpu_provenance.py compares the device counts of the
same runs with these partitions.
"""
from __future__ import annotations

import json
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from tardiis_and_claritas_gb300 import scene as S  # noqa: E402
import oracle_harness as H  # noqa: E402
import parity_scenes as PS  # noqa: E402
import provenance_partitions as PP  # noqa: E402

N_RAYS = 262144
SCENES = ("rough_spheroid", "c1_smooth_coherent", "hybrid_excess", "absorbing_conditional", "reflective_bores",
          "scully_surface")
# scenes whose per-ray provenance of the first N_PER_RAY rays is kept, with the record fields that identify
# a ray's path (status, interaction counts, detector ids)
PER_RAY = ("rough_spheroid", "hybrid_excess", "absorbing_conditional")
N_PER_RAY = 8192
KEYS = ("status", "interaction_count", "geometric", "wave", "coherent", "morphology", "native_id", "mirror_id")
OUT = os.path.join(HERE, "provenance_fixtures.npz")


def main():
    if not H.reference_available():
        raise SystemExit("host build of the reference unavailable: run oracle/ref_extract.py first")
    out = {}
    meta = {"n_rays": N_RAYS, "machine": platform.machine(), "scenes": list(SCENES), "per_ray": list(PER_RAY),
            "n_per_ray": N_PER_RAY, "keys": list(KEYS)}
    for name in SCENES:
        cfg, parts, grid = PS.build(name)
        ref = H.OracleRun("reference", cfg, parts, grid=grid)
        tal, rec, prov, defl = ref.trace_provenance(S.run_params(N_RAYS, seed=PS.seed_of(name)))
        ref.close()
        part = PP.partitions(rec["interaction_count"], rec["native_id"], rec["mirror_id"], prov, defl)
        for k, v in part.items():
            out[f"{name}/{k}"] = v
        if name in PER_RAY:
            out[f"{name}/ray_keys"] = np.stack([rec[k][:N_PER_RAY] for k in KEYS], axis=1).astype(np.int16)
            rp = prov[:N_PER_RAY].copy()
            rp[:, PP.ACR_RETURN] = rp[:, PP.ACR_RETURN] > 0  # counts kept as flags (the device keeps flags)
            rp[:, PP.AFTER_RETURN] = rp[:, PP.AFTER_RETURN] > 0
            out[f"{name}/ray_prov"] = np.clip(rp, -1, 127).astype(np.int8)
            out[f"{name}/ray_defl"] = defl[:N_PER_RAY, :2]
            out[f"{name}/ray_paths"] = defl[:N_PER_RAY, 2:]
        out[f"{name}/hw_native"] = tal["hw_native"]
        out[f"{name}/hw_mirror"] = tal["hw_mirror"]
        print(name, "detected", int(tal["hw_native"].sum()), "types", part["last_type_hits"].sum(axis=(0, 2)).tolist())
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
