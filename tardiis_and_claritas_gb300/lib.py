"""ctypes binding of libclaritas_gb.so.

The library is loaded from the package's in-tree build (tardiis_and_claritas_gb300/_lib).
There is no fallback path: if the library is missing or fails to load, every
call raises, so a run can never silently fall back to CPU code.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import abi
from .build_ext import LIB_PATH

_lock = threading.Lock()
_lib = None

# limits of clr_mie_phase_noalloc's fixed device scratch (CLR_NOALLOC_MAX_BINS / _THETA)
NOALLOC_MAX_BINS = 16
NOALLOC_MAX_THETA = 4097


class ClaritasLibraryError(RuntimeError):
    pass


def load(build_if_missing: bool = False):
    """Load (and optionally build) libclaritas_gb.so."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise ClaritasLibraryError(
                    f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
            from .build_ext import build
            build()
        lib = C.CDLL(LIB_PATH)
        P = C.POINTER
        sig = {
            "clr_create": ([P(C.c_void_p), C.c_int], C.c_int),
            "clr_destroy": ([C.c_void_p], C.c_int),
            "clr_last_error": ([C.c_void_p], C.c_char_p),
            "clr_version": ([], C.c_char_p),
            "clr_set_scene": ([C.c_void_p, P(abi.SceneParams)], C.c_int),
            "clr_build_particles": ([C.c_void_p, P(abi.ParticleSpec), P(abi.SedimentSpec)], C.c_int),
            "clr_read_particle_physics": ([C.c_void_p, P(abi.ParticlePhysics)], C.c_int),
            "clr_trace": ([C.c_void_p, P(abi.RunParams), P(abi.Tallies), C.c_void_p], C.c_int),
            "clr_trace_host_records": ([C.c_void_p, P(abi.RunParams), P(abi.Tallies), C.c_void_p], C.c_int),
            "clr_trace_batch": ([C.c_void_p, P(abi.RunParams), C.c_int, P(abi.Tallies)], C.c_int),
            "clr_abi_sizeof": ([C.c_int], C.c_int64),
            "clr_last_kernel_ms": ([C.c_void_p, P(C.c_float)], C.c_int),
            "clr_last_launches": ([C.c_void_p, P(C.c_int64), P(C.c_int64)], C.c_int),
            "clr_last_engine_stats": ([C.c_void_p, P(C.c_double), C.c_int], C.c_int),
            "clr_set_engine_config": ([C.c_void_p, P(abi.EngineConfig)], C.c_int),
            "clr_mie_phase_noalloc": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                       C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p], C.c_int),
            "clr_calibrate": ([C.c_void_p, C.c_int, P(C.c_double)], C.c_int),
            "clr_sweep_build": ([C.c_void_p, C.c_int, P(abi.SceneParams), P(abi.ParticleSpec), P(abi.SedimentSpec)],
                                C.c_int),
            "clr_sweep_trace": ([C.c_void_p, P(abi.RunParams), C.c_int, P(abi.Tallies)], C.c_int),
            "clr_sweep_read_particle_physics": ([C.c_void_p, C.c_int, P(abi.ParticlePhysics)], C.c_int),
            "clr_mlp_create": ([P(C.c_void_p), C.c_int, C.c_int, C.c_uint64], C.c_int),
            "clr_mlp_destroy": ([C.c_void_p], C.c_int),
            "clr_mlp_last_error": ([C.c_void_p], C.c_char_p),
            "clr_mlp_set_params": ([C.c_void_p, P(C.c_float), C.c_int64], C.c_int),
            "clr_mlp_get_params": ([C.c_void_p, P(C.c_float), C.c_int64], C.c_int),
            "clr_mlp_forward": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p], C.c_int),
            "clr_mlp_gradients": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, P(C.c_float), P(C.c_float)],
                                  C.c_int),
            "clr_mlp_train": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_float,
                               P(C.c_float)], C.c_int),
            "clr_mlp_last_ms": ([C.c_void_p, P(C.c_float)], C.c_int),
            "clr_mlp_set_loss_weights": ([C.c_void_p, C.c_void_p], C.c_int),
            "clr_bf16_gemm_n256": ([C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_void_p,
                                    C.c_int64, C.c_void_p], C.c_int),
            "clr_read_sediment_field": ([C.c_void_p, C.c_void_p, P(C.c_int32), P(C.c_int32), P(C.c_int32),
                                         P(C.c_double)], C.c_int),
            "clr_set_light_diagnostics": ([C.c_void_p, P(abi.LightConfig)], C.c_int),
            "clr_read_light_diagnostics": ([C.c_void_p, P(abi.LightResult)], C.c_int),
            "clr_set_path_provenance": ([C.c_void_p, C.c_int], C.c_int),
            "clr_read_path_provenance": ([C.c_void_p, P(abi.PathProvenance)], C.c_int),
            "clr_read_path_provenance_records": ([C.c_void_p, C.c_void_p, C.c_int64], C.c_int),
        }
        for name, (argt, rest) in sig.items():
            f = getattr(lib, name)
            f.argtypes = argt
            f.restype = rest
        _lib = lib
        return lib


def exported_symbols() -> list[str]:
    return ["clr_create", "clr_destroy", "clr_last_error", "clr_version", "clr_set_scene", "clr_build_particles",
            "clr_read_particle_physics", "clr_trace", "clr_trace_host_records", "clr_trace_batch", "clr_abi_sizeof",
            "clr_last_kernel_ms", "clr_last_launches", "clr_last_engine_stats", "clr_set_engine_config", "clr_calibrate",
            "clr_mie_phase_noalloc", "clr_sweep_build",
            "clr_sweep_trace", "clr_sweep_read_particle_physics", "clr_mlp_create", "clr_mlp_destroy",
            "clr_mlp_last_error", "clr_mlp_set_params", "clr_mlp_get_params", "clr_mlp_forward", "clr_mlp_gradients",
            "clr_mlp_train", "clr_mlp_set_loss_weights", "clr_mlp_last_ms", "clr_bf16_gemm_n256", "clr_read_sediment_field",
            "clr_set_light_diagnostics", "clr_read_light_diagnostics", "clr_set_path_provenance",
            "clr_read_path_provenance", "clr_read_path_provenance_records"]


def decode_provenance(raw):
    """Unpack clr_read_path_provenance_records words into the reference's per-ray provenance columns."""
    import numpy as np
    raw = np.asarray(raw, np.uint32)
    x, y = raw[:, 0], raw[:, 1]
    prov = np.zeros((raw.shape[0], 13), np.int32)

    def byte(v, k):
        b = ((v >> (8 * k)) & 0xFF).astype(np.int32)
        return np.where(b == 0xFF, -1, b)
    prov[:, 0] = (y >> 16) & 0xF
    prov[:, 1] = (y >> 20) & 0xF
    prov[:, 2] = -1
    prov[:, 3] = (y >> 24) & 1
    prov[:, 4] = (y >> 25) & 1
    prov[:, 5], prov[:, 6], prov[:, 7], prov[:, 8] = byte(x, 0), byte(x, 1), byte(x, 2), byte(x, 3)
    prov[:, 9], prov[:, 10] = byte(y, 0), byte(y, 1)
    prov[:, 11] = (y >> 26) & 1
    prov[:, 12] = (y >> 27) & 1
    defl = raw[:, 2:4].copy().view(np.float32)
    return prov, defl


class Context:
    """One library context (one CUDA stream, the resident tables of one scene)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.clr_create(C.byref(self.h), int(device))
        if rc != 0:
            raise ClaritasLibraryError(f"clr_create failed ({rc}): no usable CUDA device {device}")
        self.n_bins = 0
        self.n_theta = 0

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.clr_last_error(self.h).decode(errors="replace")
            raise RuntimeError(f"{what} failed ({rc}): {msg}")

    def set_scene(self, sp: abi.SceneParams):
        self._check(self.lib.clr_set_scene(self.h, C.byref(sp)), "clr_set_scene")

    def build_particles(self, ps: abi.ParticleSpec, ss: abi.SedimentSpec):
        self._check(self.lib.clr_build_particles(self.h, C.byref(ps), C.byref(ss)), "clr_build_particles")
        self.n_bins = int(ps.n_bins)
        self.n_theta = int(ps.n_theta)

    def physics(self) -> dict:
        pp, arrays = abi.alloc_physics(self.n_bins, self.n_theta)
        self._check(self.lib.clr_read_particle_physics(self.h, C.byref(pp)), "clr_read_particle_physics")
        arrays["phase_cdf"] = arrays["phase_cdf"].reshape(self.n_bins, self.n_theta)
        return arrays

    def sediment_field(self) -> dict:
        """The (r, z) sediment field of the current model-3 scene and its solver statistics."""
        import numpy as np
        nr, nz, it, res = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double()
        self._check(self.lib.clr_read_sediment_field(self.h, None, C.byref(nr), C.byref(nz), C.byref(it),
                                                     C.byref(res)), "clr_read_sediment_field")
        g = np.zeros((self.n_bins, nr.value, nz.value), dtype=np.float64)
        self._check(self.lib.clr_read_sediment_field(self.h, g.ctypes.data_as(C.c_void_p), None, None, None, None),
                    "clr_read_sediment_field")
        return {"grid": g, "nr": int(nr.value), "nz": int(nz.value), "iterations": int(it.value),
                "max_residual": float(res.value)}

    def set_light(self, enabled: bool = False, nx: int = 1, ny: int = 1, nz: int = 1, max_rays: int = 0,
                  representative_rays: int = 0, max_segments_per_ray: int = 0, heatmap_size: int = 0,
                  zmax: float = 0.0, heat_zmax: float = 0.0):
        """Light-history diagnostics (voxel track lengths, event sites, trajectories) and heat maps of the
        following traces; all off by default."""
        c = abi.LightConfig(int(bool(enabled)), int(nx), int(ny), int(nz), int(max_rays), int(representative_rays),
                            int(max_segments_per_ray), int(heatmap_size), float(zmax), float(heat_zmax))
        self._check(self.lib.clr_set_light_diagnostics(self.h, C.byref(c)), "clr_set_light_diagnostics")
        self._light = c

    def read_light(self) -> dict:
        import numpy as np
        c = self._light
        vox = (c.nz, c.ny, c.nx) if c.enabled else (0, 0, 0)
        rep = min(c.representative_rays, c.max_rays) if c.enabled else 0
        seg = c.max_segments_per_ray if c.enabled else 0
        vis = c.heatmap_size
        a = {"track_length": np.zeros(vox, np.float32), "post_scatter_track_length": np.zeros(vox, np.float32),
             "scatter_event_weight": np.zeros(vox, np.float32), "scatter_event_count": np.zeros(vox, np.uint32),
             "heatmap_xy": np.zeros((vis, vis), np.float32), "heatmap_zy": np.zeros((vis, vis), np.float32)}
        for k in ("x0", "y0", "z0", "x1", "y1", "z1"):
            a["trajectory_" + k] = np.zeros((rep, seg), np.float32)
        a["trajectory_order"] = np.zeros((rep, seg), np.int32)
        a["trajectory_count"] = np.zeros(rep, np.int32)
        a["trajectory_overflow"] = np.zeros(rep, np.int32)
        r = abi.LightResult()
        for name, arr in a.items():
            if arr.size:
                setattr(r, name, arr.ctypes.data_as(C.POINTER(np.ctypeslib.as_ctypes_type(arr.dtype))))
        self._check(self.lib.clr_read_light_diagnostics(self.h, C.byref(r)), "clr_read_light_diagnostics")
        for k in ("segment_length_total", "deposited_length_total", "segment_count", "scatter_event_total",
                  "error_count", "boundary_adjustment_count", "event_outside_count", "first_outside_ray",
                  "first_outside_set"):
            a[k] = getattr(r, k)
        a["first_outside_xyz_tol"] = list(r.first_outside_xyz_tol)
        return a

    def set_provenance(self, enabled: bool):
        """Count the particle-event provenance partitions of detected rays in the following traces (each
        trace call resets them; the wavefront engine counts them)."""
        self._check(self.lib.clr_set_path_provenance(self.h, int(bool(enabled))), "clr_set_path_provenance")

    def read_provenance(self) -> dict:
        """The provenance partitions of the last trace call (arrays indexed [.., side, ..], side 0 native)."""
        p = abi.PathProvenance()
        self._check(self.lib.clr_read_path_provenance(self.h, C.byref(p)), "clr_read_path_provenance")
        return p.as_dict()

    def read_provenance_records(self, n_rays: int):
        """Per-ray provenance of the last trace with records, decoded: int32 [n][13] in the reference's
        order (first/last event type, last order (not kept: -1), first backscatter, first source hemisphere,
        first/last particle, geometric and wave bin (-1 none), acrylic return, particle after a return) and
        float32 [n][2] first/last deflection."""
        import numpy as np
        raw = np.zeros((int(n_rays), 4), np.uint32)
        self._check(self.lib.clr_read_path_provenance_records(self.h, raw.ctypes.data_as(C.c_void_p), int(n_rays)),
                    "clr_read_path_provenance_records")
        return decode_provenance(raw)

    def trace(self, run: abi.RunParams, records: bool = False):
        import numpy as np
        T = abi.Tallies()
        rec = None
        if records:
            rec = np.zeros(int(run.n_rays), dtype=abi.record_dtype())
            rc = self.lib.clr_trace_host_records(self.h, C.byref(run), C.byref(T), rec.ctypes.data_as(C.c_void_p))
        else:
            rc = self.lib.clr_trace(self.h, C.byref(run), C.byref(T), None)
        self._check(rc, "clr_trace")
        return T.as_dict(), rec

    def trace_batch(self, runs: list) -> list:
        """Trace several runs of the current scene together; one tally dict per run."""
        n = len(runs)
        arr = (abi.RunParams * n)(*runs)
        outs = (abi.Tallies * n)()
        self._check(self.lib.clr_trace_batch(self.h, arr, n, outs), "clr_trace_batch")
        return [outs[i].as_dict() for i in range(n)]

    def sweep_build(self, scenes: list, particles: list, sediments: list):
        """Build the tables of many scenarios (scene params, particle specs and sediment specs, one each)."""
        n = len(scenes)
        if not (len(particles) == len(sediments) == n):
            raise ValueError("one scene, particle spec and sediment spec per scenario")
        sa = (abi.SceneParams * n)(*scenes)
        pa = (abi.ParticleSpec * n)(*particles)
        qa = (abi.SedimentSpec * n)(*sediments)
        self._check(self.lib.clr_sweep_build(self.h, n, sa, pa, qa), "clr_sweep_build")
        self.sweep_shape = [(int(p.n_bins), int(p.n_theta)) for p in particles]

    def sweep_trace(self, runs: list) -> list:
        """Trace every scenario of the built sweep together (runs[i] traces scenario i)."""
        n = len(runs)
        arr = (abi.RunParams * n)(*runs)
        outs = (abi.Tallies * n)()
        self._check(self.lib.clr_sweep_trace(self.h, arr, n, outs), "clr_sweep_trace")
        return [outs[i].as_dict() for i in range(n)]

    def sweep_physics(self, scenario: int, n_bins: int, n_theta: int) -> dict:
        """The resident tables of one scenario of the built sweep (as physics())."""
        pp, arrays = abi.alloc_physics(n_bins, n_theta)
        self._check(self.lib.clr_sweep_read_particle_physics(self.h, int(scenario), C.byref(pp)),
                    "clr_sweep_read_particle_physics")
        arrays["phase_cdf"] = arrays["phase_cdf"].reshape(n_bins, n_theta)
        return arrays

    def trace_device(self, run: abi.RunParams, records_ptr: int | None = None):
        T = abi.Tallies()
        self._check(self.lib.clr_trace(self.h, C.byref(run), C.byref(T), C.c_void_p(records_ptr) if records_ptr else None),
                    "clr_trace")
        return T

    def last_kernel_ms(self) -> float:
        v = C.c_float()
        self._check(self.lib.clr_last_kernel_ms(self.h, C.byref(v)), "clr_last_kernel_ms")
        return float(v.value)

    def last_launches(self) -> tuple[int, int]:
        """(kernel launches, wavefront passes) of the last trace."""
        n, p = C.c_int64(), C.c_int64()
        self._check(self.lib.clr_last_launches(self.h, C.byref(n), C.byref(p)), "clr_last_launches")
        return int(n.value), int(p.value)

    def engine_stats(self) -> dict:
        """Engine profile of the last trace: passes, launches, tail-kernel photons and ms, device ms."""
        v = (C.c_double * 5)()
        self._check(self.lib.clr_last_engine_stats(self.h, v, 5), "clr_last_engine_stats")
        return {"passes": int(v[0]), "launches": int(v[1]), "tail_photons": int(v[2]), "tail_ms": float(v[3]),
                "trace_ms": float(v[4])}

    def set_engine_config(self, config: dict | None = None):
        """Scheduling settings for the following traces ({} or None: defaults); keys as abi.EngineConfig,
        stage_blocks as {stage name: blocks per SM}."""
        c = abi.EngineConfig.from_dict(config)
        self._check(self.lib.clr_set_engine_config(self.h, C.byref(c) if config is not None else None),
                    "clr_set_engine_config")

    def mie_phase_noalloc(self, diameter_ptr: int, n_real_ptr: int, k_imag_ptr: int, n_bins: int, n_medium: float,
                          wavelength_m: float, n_theta: int, qext_ptr: int, qsca_ptr: int, asym_g_ptr: int,
                          theta_ptr: int, phase_cdf_ptr: int, stream_ptr: int = 0):
        """clr_mie_phase_noalloc on caller-owned device buffers (pointers as integers)."""
        self._check(self.lib.clr_mie_phase_noalloc(
            self.h, C.c_void_p(diameter_ptr), C.c_void_p(n_real_ptr), C.c_void_p(k_imag_ptr), int(n_bins),
            float(n_medium), float(wavelength_m), int(n_theta), C.c_void_p(qext_ptr), C.c_void_p(qsca_ptr),
            C.c_void_p(asym_g_ptr), C.c_void_p(theta_ptr), C.c_void_p(phase_cdf_ptr),
            C.c_void_p(stream_ptr) if stream_ptr else None), "clr_mie_phase_noalloc")

    def calibrate(self, which: int) -> float:
        v = C.c_double()
        self._check(self.lib.clr_calibrate(self.h, int(which), C.byref(v)), "clr_calibrate")
        return float(v.value)

    def close(self):
        if self.h:
            self.lib.clr_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Network:
    """The surrogate network (clr_mlp): device pointers are passed as integers (e.g. tensor.data_ptr())."""

    N_PARAMS = 199939

    def __init__(self, device: int = 0, max_batch: int = 65536, seed: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.clr_mlp_create(C.byref(self.h), int(device), int(max_batch), int(seed))
        if rc != 0:
            raise ClaritasLibraryError(f"clr_mlp_create failed ({rc})")
        self.max_batch = int(max_batch)

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.clr_mlp_last_error(self.h).decode(errors="replace")
            raise RuntimeError(f"{what} failed ({rc}): {msg}")

    def set_params(self, p):
        import numpy as np
        a = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.lib.clr_mlp_set_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), a.size),
                    "clr_mlp_set_params")

    def get_params(self):
        import numpy as np
        a = np.zeros(self.N_PARAMS, dtype=np.float32)
        self._check(self.lib.clr_mlp_get_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), a.size),
                    "clr_mlp_get_params")
        return a

    def forward(self, x_ptr: int, n: int, y_ptr: int, stream: int = 0):
        self._check(self.lib.clr_mlp_forward(self.h, C.c_void_p(x_ptr), int(n), C.c_void_p(y_ptr),
                                             C.c_void_p(stream) if stream else None), "clr_mlp_forward")

    def gradients(self, x_ptr: int, t_ptr: int, n: int):
        import numpy as np
        g = np.zeros(self.N_PARAMS, dtype=np.float32)
        loss = C.c_float()
        self._check(self.lib.clr_mlp_gradients(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), int(n),
                                               g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)),
                    "clr_mlp_gradients")
        return float(loss.value), g

    def train(self, x_ptr: int, t_ptr: int, idx_ptr: int, n_index: int, batch: int, lr: float) -> float:
        loss = C.c_float()
        self._check(self.lib.clr_mlp_train(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), C.c_void_p(idx_ptr),
                                           int(n_index), int(batch), float(lr), C.byref(loss)), "clr_mlp_train")
        return float(loss.value)

    def set_loss_weights(self, w_ptr: int):
        """Per-output loss weights [rows][3] on the device for the following gradients/train calls (0: none)."""
        self._check(self.lib.clr_mlp_set_loss_weights(self.h, C.c_void_p(w_ptr) if w_ptr else None),
                    "clr_mlp_set_loss_weights")

    def last_ms(self) -> float:
        v = C.c_float()
        self._check(self.lib.clr_mlp_last_ms(self.h, C.byref(v)), "clr_mlp_last_ms")
        return float(v.value)

    def close(self):
        if self.h:
            self.lib.clr_mlp_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bf16_gemm_n256(a_ptr: int, lda: int, b_ptr: int, ldb: int, M: int, K: int, c_ptr: int, ldc: int,
                   stream: int = 0):
    """C[M][256] = A[M][K] . B[256][K]^T on the tensor cores (BF16 in, FP32 out)."""
    rc = load().clr_bf16_gemm_n256(C.c_void_p(a_ptr), int(lda), C.c_void_p(b_ptr), int(ldb), int(M), int(K),
                                   C.c_void_p(c_ptr), int(ldc), C.c_void_p(stream) if stream else None)
    if rc != 0:
        raise RuntimeError(f"clr_bf16_gemm_n256 failed ({rc})")

