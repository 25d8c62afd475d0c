"""In-tree build of libclaritas_gb.so (nvcc, sm_103a only).

Translation units compile in parallel (the two photon-kernel instantiation
units dominate); the link step produces tardiis_and_claritas_gb300/_lib/libclaritas_gb.so.
A stamp over sources, headers and flags skips the build when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libclaritas_gb.so")

SOURCES = ["clr_api.cu", "precompute.cu", "trace_xor.cu", "trace_philox.cu", "wave_xor.cu", "wave_philox.cu",
           "calibrate.cu", "noalloc.cu", "surrogate.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + ARCH
# Per-unit flags. The FP64 precompute and the xorshift parity kernels are compiled without
# multiply-add contraction: their results are then fixed by the source's operation order alone,
# which is the reference's, instead of by where the compiler happens to fuse a*b+c (that depends
# on inlining and common-subexpression context, which necessarily differ between two programs).
# The Philox production kernels keep contraction.
UNIT_FLAGS: dict = {"precompute.cu": ["-fmad=false"], "trace_xor.cu": ["-fmad=false"], "wave_xor.cu": ["-fmad=false"]}
if os.environ.get("CLR_ALL_NOFMA"):
    UNIT_FLAGS = {s: ["-fmad=false"] for s in SOURCES}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found (CUDA toolkit required to build libclaritas_gb.so)")


def _digest() -> str:
    h = hashlib.sha256()
    h.update(" ".join(NVCC_FLAGS).encode())
    h.update(repr(sorted(UNIT_FLAGS.items())).encode())
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            if name.endswith((".cu", ".cuh", ".h")):
                with open(os.path.join(d, name), "rb") as f:
                    h.update(name.encode())
                    h.update(f.read())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    stamp = os.path.join(BUILD_DIR, "stamp")
    dig = _digest()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB_PATH
    cc = nvcc()

    def compile_one(src: str):
        obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        cmd = [cc] + NVCC_FLAGS + UNIT_FLAGS.get(src, []) + ["-I", INCLUDE, "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        with open(os.path.join(BUILD_DIR, src + ".log"), "w") as f:
            f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-4000:]}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [cc, "-shared"] + ARCH + ["-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(dig)
    if verbose:
        print(f"built {LIB_PATH}")
    return LIB_PATH


def _short_name(mangled: str) -> str:
    """Demangled kernel name without namespaces (falls back to the mangled name)."""
    try:
        name = subprocess.run(["c++filt", mangled], capture_output=True, text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return mangled[:100]
    for junk in ("clr::", "(anonymous namespace)::", "void "):
        name = name.replace(junk, "")
    return name.split("(")[0][:100]


def resource_report() -> str:
    """ptxas register/stack summary of the last build (from the per-unit logs)."""
    out = []
    for src in SOURCES:
        p = os.path.join(BUILD_DIR, src + ".log")
        if not os.path.exists(p):
            continue
        entry = None
        for line in open(p):
            if "Compiling entry function" in line:
                entry = line.split("'")[1]
            elif "Used" in line and "registers" in line and entry:
                out.append(f"{src}: {_short_name(entry)} :: {line.strip().replace('ptxas info    : ', '')}")
                entry = None
    return "\n".join(out)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(resource_report())
