"""The reference's named particle populations ('loess', 'kaolin') and their optical constants.

Data: materials.npz beside this module, written by make_materials.py from the reference's own accessors
(get_material_psd_raw, CLARITAS/CLARITAS.py:5215; get_material_optical_constants, :1082): per material the
diameter bins, the raw (unnormalised) source weights and the per-bin real and imaginary refractive index.
The functions below keep the reference's names, argument meaning and errors.
"""
from __future__ import annotations

import os

import numpy as np

_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "materials.npz")
_data = None
MATERIALS = ("loess", "kaolin")


def _table() -> dict:
    global _data
    if _data is None:
        with np.load(_PATH) as z:
            _data = {k: z[k].copy() for k in z.files}
    return _data


def _name(material: str) -> str:
    m = str(material).strip().lower()
    if m not in MATERIALS:
        raise ValueError("material must be 'loess' or 'kaolin'")
    return m


def get_material_psd_raw(material: str):
    """Diameter bins (m) and raw source weights, not normalised (:5215-5222)."""
    m, t = _name(material), _table()
    return t[f"{m}_diameter_m"].copy(), t[f"{m}_weights"].copy()


def get_material_psd(material: str):
    """Diameter bins and weights normalised to sum 1 (:5225-5228)."""
    d, w = get_material_psd_raw(material)
    return d, w / w.sum()


def get_material_optical_constants(material: str, profile_override=None, n_fallback: float = 1.59):
    """Per-bin n and k of a material, optionally replaced by profile_override[material] = {'n_real': ...,
    'k_imag': ...} (the constructor's particle_optical_constants_by_material), with the reference's checks
    (:1082-1112)."""
    m, t = _name(material), _table()
    d = t[f"{m}_diameter_m"]
    n, k = t[f"{m}_n_real"].copy(), t[f"{m}_k_imag"].copy()
    if profile_override:
        q = profile_override.get(m, profile_override.get(material, None))
        if q is not None:
            n = np.asarray(q.get("n_real", n), dtype=np.float64)
            k = np.asarray(q.get("k_imag", k), dtype=np.float64)
    if n.size != d.size or k.size != d.size:
        raise ValueError(f"{m} complex-optics profile must contain {d.size} n and k values")
    if np.any(~np.isfinite(n)) or np.any(~np.isfinite(k)) or np.any(n <= 0) or np.any(k < 0):
        raise ValueError(f"{m} complex-optics profile contains invalid n/k values")
    return n, k
