"""Write materials.npz, the named particle populations of the reference, beside this script.

The reference ships two measured particle-size distributions with per-bin complex refractive indices,
'loess' (38 bins) and 'kaolin' (37 bins), as module data (CLARITAS/CLARITAS.py:249-418, :531-703) read
through get_material_psd_raw (:5215) and get_material_optical_constants (:1082). This script imports the
reference module (it needs no GPU: CuPy is imported lazily there) and stores exactly what those two
functions return, so that simulate("loess", c) can run where the reference is absent. Run it where the
reference checkout is: python tardiis_and_claritas_gb300/make_materials.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "materials.npz")


def main() -> None:
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    from ref_extract import reference_root
    sys.path.insert(0, os.path.join(reference_root(), "CLARITAS"))
    import CLARITAS as C  # noqa: N813  (the reference module)

    out = {}
    for m in ("loess", "kaolin"):
        d, w = C.get_material_psd_raw(m)
        n, k = C.get_material_optical_constants(m)
        out[f"{m}_diameter_m"] = np.asarray(d, dtype=np.float64)
        out[f"{m}_weights"] = np.asarray(w, dtype=np.float64)
        out[f"{m}_n_real"] = np.asarray(n, dtype=np.float64)
        out[f"{m}_k_imag"] = np.asarray(k, dtype=np.float64)
    np.savez(OUT, **out)
    print(OUT, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
