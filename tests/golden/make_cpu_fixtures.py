"""Generate the CPU golden fixtures from the reference's own code built for the host.

Run where the reference checkout is available (it is read, never modified):

    python oracle/ref_extract.py && python tests/golden/make_cpu_fixtures.py

The host build of the reference (oracle/_ref/libclaritas_ref_host.so, recipe in
oracle/Makefile) runs every scene of tests/parity_scenes.py; the fixture keeps
the physics-table digests, the digest of all per-ray records, a compact integer
view and the tallies, and for a scene whose sediment field the meridional solver
makes, the field's digest, its first bin, the iteration count and final residual.
tests/test_oracle_cpu.py pins the C restatement (oracle/claritas_oracle.c) to
this file bit for bit.
"""
from __future__ import annotations

import hashlib
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

N_RAYS = 8192
N_COMPACT = 2048
OUT = os.path.join(HERE, "cpu_ref_fixtures.npz")


def main():
    if not H.reference_available():
        raise SystemExit("host build of the reference unavailable: run oracle/ref_extract.py first")
    out = {}
    meta = {"n_rays": N_RAYS, "n_compact": N_COMPACT, "machine": platform.machine(), "scenes": {}}
    for name in PS.CPU_SCENES:
        cfg, parts, grid = PS.build(name)
        ref = H.OracleRun("reference", cfg, parts, grid=grid)
        ph = ref.physics()
        tal, rec = ref.trace(S.run_params(N_RAYS, seed=PS.seed_of(name)), records=True)
        meta["scenes"][name] = {"records_sha256": PS.records_digest(rec), "physics_sha256": PS.physics_digests(ph),
                                "event_counts": tal["event_counts"][:PS.EVENT_KEYS].tolist(),
                                "conditional_stats": [int(v) for v in tal["conditional_stats"]]}
        if name in PS.SOLVED_FIELD:
            f = ref.sediment_field()
            meta["scenes"][name]["field"] = {"nr": int(f["grid"].shape[1]), "nz": int(f["grid"].shape[2]),
                                             "iterations": f["iterations"], "max_residual": f["max_residual"],
                                             "sha256": hashlib.sha256(f["grid"].tobytes()).hexdigest()}
            out[f"{name}/field_bin0"] = f["grid"][0]
        out[f"{name}/compact"] = PS.compact(rec, N_COMPACT).astype(np.int16)
        for k in PS.TALLY_KEYS:
            out[f"{name}/{k}"] = tal[k]
        print(name, tal["status_counts"][:9].tolist())
        ref.close()
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
