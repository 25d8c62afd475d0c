"""Load and drive the CPU oracles from tests (test infrastructure only).

Two CPU implementations are available:
  * the port   -- oracle/_build/libclaritas_oracle.so, our plain-C restatement;
  * the reference -- oracle/_ref/libclaritas_ref_host.so, the reference's own
    CUDA_SRC compiled as host C++ (only where the reference checkout was present
    to extract it; see oracle/ref_extract.py).
Both take the same C-ABI structs as the product (include/claritas_gb.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from tardiis_and_claritas_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
PORT_SO = os.path.join(ORACLE_DIR, "_build", "libclaritas_oracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libclaritas_ref_host.so")
REF_FAST_SO = os.path.join(ORACLE_DIR, "_ref", "libclaritas_ref_host_fast.so")
REF_SRC = os.path.join(ORACLE_DIR, "_ref", "claritas_cuda_src.inc")

_libs: dict = {}


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "port"], check=True)
    return PORT_SO


def reference_available() -> bool:
    if os.path.exists(REF_SO):
        return True
    if os.path.exists(REF_SRC):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref"], check=True)
        return os.path.exists(REF_SO)
    return False


def _bind(lib, prefix):
    p = prefix
    getattr(lib, p + "prepare").argtypes = [C.POINTER(abi.SceneParams), C.POINTER(abi.ParticleSpec),
                                            C.POINTER(abi.SedimentSpec), C.POINTER(C.c_void_p)]
    getattr(lib, p + "prepare").restype = C.c_int
    getattr(lib, p + "trace").argtypes = [C.c_void_p, C.POINTER(abi.RunParams), C.POINTER(abi.Tallies),
                                          C.c_void_p, C.c_int]
    getattr(lib, p + "trace").restype = C.c_int
    getattr(lib, p + "read_physics").argtypes = [C.c_void_p, C.POINTER(abi.ParticlePhysics)]
    getattr(lib, p + "read_physics").restype = C.c_int
    getattr(lib, p + "n_theta").argtypes = [C.c_void_p]
    getattr(lib, p + "n_theta").restype = C.c_int
    getattr(lib, p + "last_error").argtypes = [C.c_void_p]
    getattr(lib, p + "last_error").restype = C.c_char_p
    getattr(lib, p + "free").argtypes = [C.c_void_p]
    getattr(lib, p + "free").restype = None
    getattr(lib, p + "read_sediment_field").argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_int),
                                                        C.POINTER(C.c_int), C.POINTER(C.c_int),
                                                        C.POINTER(C.c_double)]
    getattr(lib, p + "read_sediment_field").restype = C.c_int
    return lib


def load(kind: str = "port"):
    if kind in _libs:
        return _libs[kind]
    if kind == "port":
        if not os.path.exists(PORT_SO):
            build_port()
        lib = _bind(C.CDLL(PORT_SO), "clo_")
        lib.clo_erfinv.argtypes = [C.c_double]
        lib.clo_erfinv.restype = C.c_double
        lib.clo_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.clo_trace_provenance.argtypes = [C.c_void_p, C.POINTER(abi.RunParams), C.POINTER(abi.Tallies),
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.clo_trace_provenance.restype = C.c_int
        prefix = "clo_"
    elif kind in ("reference", "reference_fast"):
        if not reference_available():
            raise FileNotFoundError("host build of the reference is not available")
        so = REF_SO
        if kind == "reference_fast":  # the timed CPU baseline: the same source built with -O3 and contraction
            subprocess.run(["make", "-s", "-C", ORACLE_DIR, "ref_fast"], check=True)
            so = REF_FAST_SO
        lib = _bind(C.CDLL(so), "clref_")
        lib.clref_trace_provenance.argtypes = [C.c_void_p, C.POINTER(abi.RunParams), C.POINTER(abi.Tallies),
                                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        lib.clref_trace_provenance.restype = C.c_int
        prefix = "clref_"
    else:
        raise ValueError(kind)
    _libs[kind] = (lib, prefix)
    return _libs[kind]


class OracleRun:
    """Prepared scene in one of the CPU oracles."""

    def __init__(self, kind, cfg, particles, grid=None, moments=None, grid_zmax=None):
        self.lib, self.p = load(kind)
        self.cfg = cfg
        self.sp = cfg.to_scene_params()
        self.ps = particles.spec(cfg, moments)
        self.ss = cfg.sediment_spec(grid, grid_zmax)
        self.h = C.c_void_p()
        rc = getattr(self.lib, self.p + "prepare")(C.byref(self.sp), C.byref(self.ps), C.byref(self.ss),
                                                   C.byref(self.h))
        if rc != 0:
            msg = getattr(self.lib, self.p + "last_error")(self.h).decode()
            getattr(self.lib, self.p + "free")(self.h)
            self.h = C.c_void_p()
            raise RuntimeError(f"{kind} oracle prepare failed ({rc}): {msg}")
        self.n_bins = particles.diameter_m.size
        self.n_theta = getattr(self.lib, self.p + "n_theta")(self.h)

    def physics(self) -> dict:
        pp, arrays = abi.alloc_physics(self.n_bins, self.n_theta)
        getattr(self.lib, self.p + "read_physics")(self.h, C.byref(pp))
        arrays["phase_cdf"] = arrays["phase_cdf"].reshape(self.n_bins, self.n_theta)
        return arrays

    def sediment_field(self) -> dict:
        """The model-3 field [bins][nr][nz] with the solver's iterations and final largest residual."""
        f = getattr(self.lib, self.p + "read_sediment_field")
        nr, nz, it, res = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        f(self.h, None, C.byref(nr), C.byref(nz), C.byref(it), C.byref(res))
        grid = np.zeros((self.n_bins, nr.value, nz.value))
        f(self.h, grid.ctypes.data_as(C.c_void_p), None, None, None, None)
        return {"grid": grid, "iterations": it.value, "max_residual": res.value}

    def trace(self, run: abi.RunParams, records: bool = False, threads: int = 0):
        T = abi.Tallies()
        rec = None
        ptr = None
        if records:
            rec = np.zeros(int(run.n_rays), dtype=abi.record_dtype())
            ptr = rec.ctypes.data_as(C.c_void_p)
        rc = getattr(self.lib, self.p + "trace")(self.h, C.byref(run), C.byref(T), ptr, int(threads))
        if rc != 0:
            raise RuntimeError(getattr(self.lib, self.p + "last_error")(self.h).decode())
        return T.as_dict(), rec

    def trace_provenance(self, run: abi.RunParams, threads: int = 0):
        """Tallies, per-ray records, and per ray the reference's provenance outputs
        (int [n][13]: first/last event type, last event order, first backscatter, first source hemisphere,
        first/last particle, geometric and wave bin, acrylic returns after a particle event, particle events
        after a return) and float [n][5]: first and last deflection (deg), path and optical path inside
        particles, water path after the last event (-1 without one)."""
        T = abi.Tallies()
        n = int(run.n_rays)
        rec = np.zeros(n, dtype=abi.record_dtype())
        prov = np.zeros((n, 13), np.int32)
        defl = np.zeros((n, 5), np.float32)
        rc = getattr(self.lib, self.p + "trace_provenance")(
            self.h, C.byref(run), C.byref(T), rec.ctypes.data_as(C.c_void_p), prov.ctypes.data_as(C.c_void_p),
            defl.ctypes.data_as(C.c_void_p), int(threads))
        if rc != 0:
            raise RuntimeError(getattr(self.lib, self.p + "last_error")(self.h).decode())
        return T.as_dict(), rec, prov, defl

    def close(self):
        if self.h:
            getattr(self.lib, self.p + "free")(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
