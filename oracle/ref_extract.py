"""Extract the reference's embedded CUDA source for the host/GPU reference builds.

Test infrastructure only. The reference ships its device code as the Python
string ``CUDA_SRC`` (CLARITAS/CLARITAS.py:1119-5212). This script imports the
reference module read-only (it defers CuPy, CLARITAS/CLARITAS.py:5653-5656, so
the import works without a GPU) and writes that string, byte for byte, to
``oracle/_ref/claritas_cuda_src.inc``. Nothing it writes is committed:
``oracle/_ref/`` is git-ignored. Run from anywhere::

    python oracle/ref_extract.py [--reference DIR]

The reference checkout is found by ``reference_root()``: the directory named by the
CLARITAS_REFERENCE_DIR environment variable, else a checkout named ``reference`` beside
this repository.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "claritas_cuda_src.inc")


def reference_root() -> str:
    """The reference checkout: $CLARITAS_REFERENCE_DIR, else ``reference`` beside this repository."""
    env = os.environ.get("CLARITAS_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def extract(reference_root_dir: str | None = None) -> str:
    mod_dir = os.path.join(reference_root_dir or reference_root(), "CLARITAS")
    if not os.path.isfile(os.path.join(mod_dir, "CLARITAS.py")):
        raise FileNotFoundError(f"reference module not found under {mod_dir}")
    sys.path.insert(0, mod_dir)
    try:
        import CLARITAS  # noqa: N813  (reference module name)
    finally:
        sys.path.pop(0)
    src = CLARITAS.CUDA_SRC
    os.makedirs(OUT_DIR, exist_ok=True)
    digest = hashlib.sha256(src.encode()).hexdigest()
    old = None
    if os.path.exists(OUT):
        with open(OUT, encoding="utf-8") as f:
            old = f.read()
    if old != src:
        with open(OUT, "w", encoding="utf-8") as f:
            f.write(src)
    with open(os.path.join(OUT_DIR, "claritas_cuda_src.sha256"), "w") as f:
        f.write(digest + "\n")
    return OUT


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None, help="reference checkout (default: reference_root())")
    a = ap.parse_args()
    print(extract(a.reference))
