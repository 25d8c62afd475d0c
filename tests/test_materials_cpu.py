"""CPU: the reference's named particle populations bundled with the library.

materials.npz holds, for 'loess' (38 bins) and 'kaolin' (37 bins), what the reference's accessors return:
get_material_psd_raw (CLARITAS/CLARITAS.py:5215) and get_material_optical_constants (:1082). Where the
reference checkout is present the bundled arrays must equal those functions' outputs exactly; everywhere
the accessors must keep the reference's normalisation, override and error behaviour.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from tardiis_and_claritas_gb300 import forward as F, materials as M

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_module():
    sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
    from ref_extract import reference_root
    mod = os.path.join(reference_root(), "CLARITAS")
    if not os.path.isfile(os.path.join(mod, "CLARITAS.py")):
        pytest.skip("reference checkout not present")
    sys.path.insert(0, mod)
    import CLARITAS  # noqa: N813
    return CLARITAS


@pytest.mark.parametrize("material", ["loess", "kaolin"])
def test_bundled_tables_equal_the_reference(material):
    C = _reference_module()
    d, w = M.get_material_psd_raw(material)
    rd, rw = C.get_material_psd_raw(material)
    np.testing.assert_array_equal(d, rd)
    np.testing.assert_array_equal(w, rw)
    n, k = M.get_material_optical_constants(material)
    rn, rk = C.get_material_optical_constants(material)
    np.testing.assert_array_equal(n, rn)
    np.testing.assert_array_equal(k, rk)
    nd, wd = M.get_material_psd(material)
    rnd, rwd = C.get_material_psd(material)
    np.testing.assert_array_equal(wd, rwd)
    prof = {material: {"k_imag": np.zeros(d.size)}}
    np.testing.assert_array_equal(M.get_material_optical_constants(material, prof)[1],
                                  C.get_material_optical_constants(material, prof)[1])


def test_accessor_rules():
    assert M.get_material_psd_raw("loess")[0].size == 38 and M.get_material_psd_raw(" Kaolin ")[0].size == 37
    assert M.get_material_psd("kaolin")[1].sum() == pytest.approx(1.0)
    with pytest.raises(ValueError, match="material must be 'loess' or 'kaolin'"):
        M.get_material_psd_raw("sand")
    with pytest.raises(ValueError, match="must contain 38 n and k values"):
        M.get_material_optical_constants("loess", {"loess": {"n_real": [1.5]}})
    with pytest.raises(ValueError, match="invalid n/k"):
        M.get_material_optical_constants("kaolin", {"kaolin": {"k_imag": -np.ones(37)}})


def test_facade_particles_of_a_named_material():
    m = F.ClaritasForwardModel(density_kg_per_m3=2650.0)
    p = m._particles("kaolin", 0.5, None, "mass_fraction")
    d, w = M.get_material_psd_raw("kaolin")
    np.testing.assert_array_equal(p.diameter_m, d)
    np.testing.assert_array_equal(p.weight, w)
    assert p.density_kg_m3 == 2650.0 and p.concentration_kg_m3 == 0.5
    with pytest.raises(ValueError, match="requires 37 PSD weights"):
        m._particles("kaolin", 0.5, [1.0, 2.0], "mass_fraction")
