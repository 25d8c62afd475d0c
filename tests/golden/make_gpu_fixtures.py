"""Generate the GPU golden fixtures from the reference's own kernels.

Run on a machine with a GB300 (sm_103a) after oracle/ref_extract.py has written
oracle/_ref/claritas_cuda_src.inc from the reference checkout:

    python tests/golden/make_gpu_fixtures.py --out tests/golden/gpu_ref_fixtures.npz
    python tests/golden/make_gpu_fixtures.py --scenes moment_constrained \
        --out tests/golden/gpu_ref_moment_fixtures.npz

It compiles oracle/ref_gpu_driver.cu (the reference's CUDA_SRC plus a launcher
that replays the reference host's launch sequence) into
oracle/_ref/libclaritas_ref_gpu.so, runs every scene of tests/parity_scenes.py
with the reference's xorshift seeding, and stores per scene: digests of the
physics tables, the digest of all per-ray records, a compact integer view of
the first records, and the detector tallies. tests/test_gpu_parity.py compares
the library against this file bit for bit.
"""
from __future__ import annotations

import argparse
import hashlib
import ctypes as C
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from tardiis_and_claritas_gb300 import abi, scene as S  # noqa: E402
import parity_scenes as PS  # noqa: E402

ORACLE = os.path.join(ROOT, "oracle")
SRC = os.path.join(ORACLE, "_ref", "claritas_cuda_src.inc")
# The bit-exact target is the reference source compiled without multiply-add contraction, as the
# library's parity kernels are; CLR_REF_FMAD=true builds the reference as CuPy/NVRTC deploy it
# (contraction on) for the agreement-rate fixture.
FMAD = os.environ.get("CLR_REF_FMAD", "false")
SO = os.path.join(ORACLE, "_ref", "libclaritas_ref_gpu.so" if FMAD == "true" else "libclaritas_ref_gpu_nofma.so")
N_RAYS = 131072
N_COMPACT = 4096


def build():
    if not os.path.exists(SRC):
        raise FileNotFoundError(f"{SRC} missing: run oracle/ref_extract.py where the reference is checked out")
    if os.path.exists(SO) and os.path.getmtime(SO) > max(os.path.getmtime(SRC),
                                                         os.path.getmtime(os.path.join(ORACLE, "ref_gpu_driver.cu"))):
        return SO
    cmd = ["nvcc", "-std=c++17", "-O3", f"-fmad={FMAD}", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
           "-shared", "-w", "-I", os.path.join(ROOT, "include"), "-I", ORACLE,
           os.path.join(ORACLE, "ref_gpu_driver.cu"), "-o", SO]
    t = time.time()
    subprocess.run(cmd, check=True)
    print(f"built {SO} in {time.time() - t:.0f} s", flush=True)
    return SO


def load():
    lib = C.CDLL(build())
    P = C.POINTER
    lib.clrefgpu_prepare.argtypes = [P(abi.SceneParams), P(abi.ParticleSpec), P(abi.SedimentSpec), P(C.c_void_p)]
    lib.clrefgpu_trace.argtypes = [C.c_void_p, P(abi.RunParams), P(abi.Tallies), C.c_void_p]
    lib.clrefgpu_read_physics.argtypes = [C.c_void_p, P(abi.ParticlePhysics)]
    lib.clrefgpu_n_theta.argtypes = [C.c_void_p]
    lib.clrefgpu_last_error.argtypes = [C.c_void_p]
    lib.clrefgpu_last_error.restype = C.c_char_p
    lib.clrefgpu_free.argtypes = [C.c_void_p]
    lib.clrefgpu_read_sediment_field.argtypes = [C.c_void_p, C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int),
                                                 P(C.c_double)]
    return lib


def field_of(lib, h, n_bins: int) -> dict:
    """The reference's (r, z) sediment field of a model-3 scene: digest, shape, solver statistics, bin 0."""
    nr, nz, it, res = C.c_int(), C.c_int(), C.c_int(), C.c_double()
    lib.clrefgpu_read_sediment_field(h, None, C.byref(nr), C.byref(nz), C.byref(it), C.byref(res))
    g = np.zeros((n_bins, nr.value, nz.value), dtype=np.float64)
    lib.clrefgpu_read_sediment_field(h, g.ctypes.data_as(C.c_void_p), None, None, None, None)
    return {"sha256": hashlib.sha256(g.tobytes()).hexdigest(), "nr": nr.value, "nz": nz.value,
            "iterations": it.value, "max_residual": res.value, "bin0": g[0]}


def run_scene(lib, name: str, n_rays: int = N_RAYS):
    cfg, parts, grid = PS.build(name)
    sp, ps, ss = cfg.to_scene_params(), parts.spec(cfg, PS.moments(name, parts.diameter_m.size)), cfg.sediment_spec(grid)
    h = C.c_void_p()
    rc = lib.clrefgpu_prepare(C.byref(sp), C.byref(ps), C.byref(ss), C.byref(h))
    if rc != 0:
        raise RuntimeError(f"{name}: reference prepare failed {rc}: {lib.clrefgpu_last_error(h).decode()}")
    nt = lib.clrefgpu_n_theta(h)
    pp, arrays = abi.alloc_physics(parts.diameter_m.size, nt)
    lib.clrefgpu_read_physics(h, C.byref(pp))
    field = field_of(lib, h, parts.diameter_m.size) if sp.sediment_model == 3 else None
    run = S.run_params(n_rays, seed=PS.seed_of(name))
    T = abi.Tallies()
    rec = np.zeros(n_rays, dtype=abi.record_dtype())
    rc = lib.clrefgpu_trace(h, C.byref(run), C.byref(T), rec.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise RuntimeError(f"{name}: reference trace failed {rc}: {lib.clrefgpu_last_error(h).decode()}")
    lib.clrefgpu_free(h)
    return arrays, T.as_dict(), rec, field


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden", "gpu_ref_fixtures.npz"))
    ap.add_argument("--rays", type=int, default=N_RAYS)
    ap.add_argument("--scenes", default="", help="comma-separated scene names (default: every parity scene)")
    a = ap.parse_args()
    lib = load()
    out = {}
    meta = {"n_rays": a.rays, "n_compact": N_COMPACT, "scenes": {}}
    for name in (a.scenes.split(",") if a.scenes else PS.SCENES):
        t = time.time()
        ph, tal, rec, field = run_scene(lib, name, a.rays)
        meta["scenes"][name] = {"records_sha256": PS.records_digest(rec), "physics_sha256": PS.physics_digests(ph),
                                "seed": PS.seed_of(name), "event_counts": tal["event_counts"][:PS.EVENT_KEYS].tolist(),
                                "conditional_stats": [int(v) for v in tal["conditional_stats"]]}
        if field is not None:
            out[f"{name}/field_bin0"] = field.pop("bin0")
            meta["scenes"][name]["field"] = field
        out[f"{name}/compact"] = PS.compact(rec, N_COMPACT).astype(np.int16)
        for k in PS.TALLY_KEYS:
            out[f"{name}/{k}"] = tal[k]
        print(f"{name}: {time.time() - t:.1f} s status={tal['status_counts'][:9].tolist()}", flush=True)
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    np.savez_compressed(a.out, **out)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
