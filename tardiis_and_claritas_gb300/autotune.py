"""Per-GPU, per-scene tuning of the wavefront engine's scheduling settings (clr_engine_config).

The reference has no counterpart: it launches its trace kernel with one thread per ray, 256 threads per
block, over chunks of rays, and lets the hardware schedule them (CLARITAS/CLARITAS.py:7307 and :7637-7640,
the launch of trace_kernel). The wavefront engine instead fixes how many water flights a FLIGHT visit
takes, how many pass graphs run between two host reads of the live flag, when the single-thread tail
kernel takes over, how long a rare stage's queue grows before it runs and how many blocks per SM each
stage kernel keeps resident. None of these change a
photon's draws or arithmetic, so any setting gives the same integer tallies (the GPU test checks this);
they only move the trace time, and the best values depend on the GPU and on the scene (how long photons
live, how often they meet the walls).

`tune` runs a one-sweep coordinate search from the defaults: every candidate value of one setting is timed
(device time of whole traces, the median of `reps`), a value is kept when it beats the incumbent by more
than `min_gain`, and the winner is timed once more against the defaults, interleaved, before it is
accepted. Results are cached in a JSON file by (compute capability and SM count, scene key, photons per
trace); `engine_tuning.json` beside this file ships results of the same search for known GPUs and workloads.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import statistics
from typing import Callable

from . import abi

# groups of alternatives, searched in this order; at most one change of a group is kept
SPACE: list[tuple[str, list[dict]]] = [
    ("flight_steps", [{"flight_steps": v} for v in (2, 3, 6, 8)]),
    ("pass_batch", [{"pass_batch": v} for v in (4, 16)]),
    ("tail_photons", [{"tail_photons": v} for v in (16384, 32768, 131072, 262144)]),
    ("rare_batch", [{"rare_batch": v} for v in (2048, 4096, 16384, 32768)]),
    ("acr_budget", [{"acr_budget": v} for v in (64, 128, 512)]),
] + [(f"blocks:{stage}", [{"stage_blocks": {stage: b}} for b in blocks])
     for stage, blocks in (("FLIGHT", (1,)), ("GEN", (1, 2)), ("SIDE", (1, 2)), ("GEOM", (1,)), ("BOTTOM", (2,)),
                           ("TOP", (2,)), ("FIN", (1,)))]


def cache_path() -> str:
    p = os.environ.get("CLR_TUNING_CACHE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "tardiis_and_claritas_gb300", "engine_tuning.json")


# host arrays of the specs that enter the key by value: (field, length from the spec)
_ARRAYS = {"diameter_m": "n_bins", "weight": "n_bins", "n_real": "n_bins", "k_imag": "n_bins"}


def scene_key(scene: abi.SceneParams, particles: abi.ParticleSpec, sediment: abi.SedimentSpec) -> str:
    """Hash of the values that shape photon lifetimes: the scene struct, the particle/sediment scalars and
    the particle bins' diameters, weights and optical constants. Pointer values do not enter: the same
    scene built from other host buffers has the same key. Host pointers only (the ABI's specs are host)."""
    h = hashlib.sha1(bytes(scene))
    for s in (particles, sediment):
        for name, t in s._fields_:
            v = getattr(s, name)
            if hasattr(t, "contents"):
                if s is particles and name in _ARRAYS and v:
                    n = int(getattr(s, _ARRAYS[name]))
                    h.update(name.encode() + bytes(C.cast(v, C.POINTER(C.c_double * n)).contents))
                continue
            h.update(f"{name}={v!r};".encode())
    return h.hexdigest()[:16]


def _merge(cfg: dict, change: dict) -> dict:
    out = dict(cfg)
    for k, v in change.items():
        if k == "stage_blocks":
            sb = dict(out.get("stage_blocks", {}))
            sb.update(v)
            out["stage_blocks"] = sb
        else:
            out[k] = v
    return out


def _candidates(cfg: dict, group: str) -> list[dict]:
    out = []
    for name, changes in SPACE:
        if name != group:
            continue
        for change in changes:
            cand = _merge(cfg, change)
            if cand != cfg:
                out.append(cand)
    return out


SHIPPED_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "engine_tuning.json")


def device_key(major: int, minor: int, sm_count: int) -> str:
    """The GPU part of a tuning key: compute capability and SM count (names differ between drivers)."""
    return f"sm{int(major)}{int(minor)}x{int(sm_count)}"


def entry_key(device: str, key: str, photons: int) -> str:
    return f"{device}|{key}|{int(photons).bit_length()}"


def load_shipped() -> dict:
    """Settings this package ships, found by the same search on the GPUs named in their keys."""
    try:
        with open(SHIPPED_TABLE) as f:
            return json.load(f).get("entries", {})
    except (OSError, ValueError):
        return {}


def load_cache(path: str | None = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def store_cache(entries: dict, path: str | None = None) -> None:
    path = path or cache_path()
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(entries, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def search(time_config: Callable[[dict], float], *, reps: int = 2, min_gain: float = 0.015,
           confirm_reps: int = 3) -> dict:
    """Coordinate search over SPACE with `time_config(cfg) -> seconds` (one trace). Host-only logic: the
    GPU enters through time_config, so the search itself is tested on the CPU with a model of the cost."""
    trials = []
    time_config({})  # untimed: the first trace of a context pays for its pool and graph set-up

    def med(cfg):
        ts = [time_config(cfg) for _ in range(reps)]
        trials.append({"config": cfg, "s": ts})
        return statistics.median(ts)

    best = {}
    best_t = med(best)
    base_t = best_t
    landscape = []  # (group, candidate, its median / the incumbent's median when it was tried)
    for name, _ in SPACE:
        group_best, group_t = best, best_t
        for cand in _candidates(best, name):
            t = med(cand)
            landscape.append((name, cand, t / best_t))
            if t < group_t * (1.0 - min_gain):
                group_best, group_t = cand, t
        best, best_t = group_best, group_t
    accepted = best
    if best:
        # interleaved confirmation against the defaults: the search may have kept a lucky draw
        tb, td = [], []
        for _ in range(confirm_reps):
            tb.append(time_config(best))
            td.append(time_config({}))
        mb, md = statistics.median(tb), statistics.median(td)
        trials.append({"config": best, "s": tb, "confirm": True})
        trials.append({"config": {}, "s": td, "confirm": True})
        if not mb < md * (1.0 - min_gain):
            accepted = {}
        base_t, best_t = md, (mb if accepted else md)
    return {"config": accepted, "trace_s": best_t, "default_trace_s": base_t,
            "gain": base_t / best_t - 1.0 if best_t > 0 else 0.0, "trials": len(trials),
            "landscape": [{"group": g, "config": c, "relative_time": round(r, 4)} for g, c, r in landscape]}


def tune(ctx, make_run: Callable[[int], abi.RunParams] | None = None, *, key: str, photons: int, device: str,
         reps: int = 2, use_cache: bool = True, cache_file: str | None = None,
         trace: Callable[[int], object] | None = None) -> dict:
    """Tune the engine settings of `ctx`'s current scene and leave the winner set on the context.

    make_run(i) returns the run of trial i (give disjoint photon ranges), or trace(i) runs trial i itself
    (a batch or sweep trace of the context); key is scene_key(...) of the scene the context holds, or a name
    of a workload; device is device_key(...). A result in the user's cache, else in the package's shipped
    table, is used without a search. Returns {"config", "gain", "trace_s", "default_trace_s", "trials",
    "landscape", "cached": "user" | "shipped" | False}."""
    if trace is None:
        if make_run is None:
            raise ValueError("tune needs make_run or trace")
        trace = lambda i: ctx.trace(make_run(i))  # noqa: E731
    ek = entry_key(device, key, photons)
    if use_cache:
        for source, entries in (("user", load_cache(cache_file)), ("shipped", load_shipped())):
            if ek in entries:
                res = dict(entries[ek])
                ctx.set_engine_config(res["config"] or None)
                res["cached"] = source
                return res
    counter = [0]

    def time_config(cfg: dict) -> float:
        ctx.set_engine_config(cfg or None)
        trace(counter[0])
        counter[0] += 1
        return ctx.last_kernel_ms() * 1e-3

    res = search(time_config, reps=reps)
    ctx.set_engine_config(res["config"] or None)
    res["cached"] = False
    if use_cache:
        entries = load_cache(cache_file)
        entries[ek] = {k: res[k] for k in ("config", "gain", "trace_s", "default_trace_s", "trials", "landscape")}
        try:
            store_cache(entries, cache_file)
        except OSError:
            pass
    return res
