"""Golden vectors for the facade's restated reference helpers (run where the reference checkout is).

Calls the reference's own ``_jackknife_normalized_se`` and ``_histogram_median``
(CLARITAS/CLARITAS.py:5231-5262) on seeded inputs and stores inputs and outputs in
``forward_fixtures.npz`` beside this script. Usage: python tests/golden/make_forward_fixtures.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
from ref_extract import reference_root  # noqa: E402

REF = os.path.join(reference_root(), "CLARITAS")


def main() -> None:
    sys.path.insert(0, REF)
    import CLARITAS as C  # noqa: N813  (the reference module; CuPy is imported lazily there)

    rng = np.random.default_rng(20261203)
    out = {}
    for case, n_batches in enumerate((2, 3, 5, 17, 40)):
        scores = rng.poisson(rng.uniform(0.5, 400.0, 18), size=(n_batches, 18)).astype(float)
        if case == 4:
            scores[3] = 0.0  # an empty batch
        out[f"jk_in_{case}"] = scores
        out[f"jk_out_{case}"] = np.asarray(C._jackknife_normalized_se(list(scores)), dtype=float)
    for case in range(6):
        hist = rng.integers(0, 7, size=int(rng.integers(1, 40))).astype(np.int64)
        if case == 0:
            hist[:] = 0
        out[f"med_in_{case}"] = hist
        out[f"med_out_{case}"] = np.array(C._histogram_median(hist), dtype=float)
    np.savez(os.path.join(os.path.dirname(os.path.abspath(__file__)), "forward_fixtures.npz"), **out)


if __name__ == "__main__":
    main()
