"""CPU checks of the C ABI: the library builds for sm_103a, loads without a GPU,
exports every entry point include/claritas_gb.h declares, and its struct sizes
match the Python mirror."""
from __future__ import annotations

import ctypes as C
import os
import re

import pytest

from tardiis_and_claritas_gb300 import abi, build_ext, lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def library():
    build_ext.build()
    return L.load()


def declared_functions():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(inc, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(clr_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_binding_surface():
    assert declared_functions() == sorted(L.exported_symbols())


def test_library_exports_every_declared_symbol(library):
    for name in declared_functions():
        assert hasattr(library, name), name


def test_struct_sizes_match(library):
    mirror = [abi.SceneParams, abi.ParticleSpec, abi.SedimentSpec, abi.RunParams, abi.RayRecord, abi.Tallies,
              abi.ParticlePhysics, abi.PathProvenance, abi.EngineConfig]
    for i, cls in enumerate(mirror):
        assert library.clr_abi_sizeof(i) == C.sizeof(cls), cls.__name__
    assert library.clr_abi_sizeof(99) == -1


def test_version_and_null_arguments(library):
    assert b"sm_103a" in library.clr_version()
    assert library.clr_destroy(None) == abi.CLR_ERR_INVALID_ARGUMENT
    assert library.clr_create(None, 0) == abi.CLR_ERR_INVALID_ARGUMENT


def test_resource_report_available(library):
    rep = build_ext.resource_report()
    assert "photon_kernel" in rep and "registers" in rep


def test_header_is_plain_c(tmp_path):
    """include/claritas_gb.h is consumable from C (cgo, JNI, ctypes generators): it compiles as strict C99."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "h.c"
    src.write_text('#include "claritas_gb.h"\nint main(void) { clr_tallies t; clr_path_provenance p; '
                   '(void)t; (void)p; return 0; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-fsyntax-only", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
