#!/usr/bin/env python3
"""Benchmark of the photon-transport hot path (photons/s at fixed tally error).

One "step" traces one batch of photons of the full-scene workload through the
library's wavefront photon engine (transport, detector scoring and tallies; one
CUDA graph of stage kernels per pass). Both arms run the same analog estimator;
each line reports the per-channel standard error it reached and the figure of
merit 1 / (relative SE^2 x time), so the speed ratio at equal tally error is
measured, not assumed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload full|small|sweep]
  python bench.py --impl reference ...   # the reference's own CPU implementation

With --workload sweep a step builds and traces the 512-scenario batched sweep (per-scenario Mie
tables, rates and photon counts log-uniform over 1e5-1e7) and the metric is scenarios/s.

Multi-GPU (torchrun, one rank per GPU): replicas over disjoint photon ranges
(counter-based Philox streams), no data-path collective; value = all photons /
max-over-ranks time ("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Per photon of the wavefront engine on the full scene (counter-based stream), from ncu captures of a small
# trace of the same scene summed over every stage kernel: warp instructions issued (the issue-slot cross-check
# of the roofline, 4 schedulers x SMs x clock) and DRAM bytes read + written (the traffic figure). The
# roofline's achieved work itself comes from the event counters of the timed traces (workcount.py).
PER_PHOTON = {"full": {"warp_inst": 289.7, "dram_bytes": 889.0}}
HEADLINE_CHANNELS = (0, 9, 17)  # transmitted, nephelometric (90 deg) and nearest-backscatter (170 deg) detectors


def channel_error(tallies: list, seconds: float) -> dict:
    """Per headline channel: native hits, relative standard error of the hit fraction (binomial; weighted
    runs: from the weight sums) and the figure of merit 1 / (relative SE^2 x seconds). The ratio of two
    arms' figures of merit is their speed ratio at equal tally error."""
    import numpy as np
    n = float(sum(int(t["n_rays"]) for t in tallies))
    out = {}
    for j in HEADLINE_CHANNELS:
        hits = float(sum(int(t["hw_native"][j]) for t in tallies))
        w = float(sum(float(t["weight_native"][j]) for t in tallies))
        w2 = float(sum(float(t["weight_sq_native"][j]) for t in tallies))
        mean = w / n if n else 0.0
        var = max(w2 / n - mean * mean, 0.0) / n if n else 0.0
        rel = float(np.sqrt(var) / mean) if mean > 0 else None
        out[str(j)] = {"hits": int(hits), "mean_per_photon": mean, "rel_se": rel,
                       "fom_per_s": (1.0 / (rel * rel * seconds)) if rel and seconds > 0 else None}
    out["photons"] = int(n)
    out["seconds"] = seconds
    return out


def equal_error_speedup(gpu: dict, cpu: dict) -> dict:
    """Per headline channel: GPU figure of merit / CPU figure of merit (speed ratio at equal tally error)."""
    out = {}
    for j in HEADLINE_CHANNELS:
        a, b = gpu[str(j)]["fom_per_s"], cpu[str(j)]["fom_per_s"]
        out[str(j)] = (a / b) if a and b else None
    return out


def workload(name: str):
    from tardiis_and_claritas_gb300 import scene as S
    if name == "full":
        cfg, parts, grid, zmax = S.full_scene_workload()
        return cfg, parts, grid, zmax, 100_000_000
    cfg, parts, grid, zmax = S.small_plain_workload()
    return cfg, parts, grid, zmax, 1_000_000


def workload_config(name: str, n: int, rng: str) -> dict:
    if name == "full":
        return {"workload": "full scene: 63-bin clay/silt/sand mixture (2/20/100 um, sigma_g 1.4, 0.3/0.5/0.2) at "
                            "500 mg/L in a 64x64 (r,z) Rouse(P=0.3) x radial-depletion field, stirred free surface "
                            "(600 rpm, 5 mm core; localized-vortex surface), r=12.5 mm cell, smooth spheres with "
                            "FP64 Mie phase tables (1801 angles), 860 nm",
                "photons_per_step": n, "rng": rng, "l2": "flushed between steps (256 MiB write)"}
    return {"workload": "small plain MC: 64 lognormal quartz bins (median 20 um, sigma_g 1.6) at 100 mg/L, uniform, "
                        "flat surface, r=12.5 mm cell, 2 mm collimated disc beam at the sensor plane, Mie tables "
                        "1801 angles, 860 nm",
            "photons_per_step": n, "rng": rng, "l2": "flushed between steps (256 MiB write)"}


SWEEP_SCENARIOS = 512
SWEEP_WORKLOAD = ("batched sweep: 512 scenarios in the r=12.5 mm cell (40 mm water), seeds 0..511, sampled with "
                  "numpy PCG64(0): photons log-uniform 1e5-1e7, concentration log-uniform 1-1e4 mg/L, median "
                  "diameter log-uniform 2-200 um, sigma_g U(1.2,2.0), stirrer rpm U(0,1200) (localized-vortex "
                  "surface, 5 mm core), particle index U(1.50,1.60); 64 lognormal bins over 1-200 um, FP64 Mie "
                  "phase tables (1801 angles) per scenario, 860 nm, uniform sediment")


def optical_depth_proxy(sc) -> float:
    """Radius x extinction of the scenario's particles with Q_ext = 2 (a ranking key for CPU cost)."""
    p = sc.particles
    w = p.weight / p.weight.sum()
    return 1.5 * 2.0 * p.concentration_kg_m3 / p.density_kg_m3 * float((w / p.diameter_m).sum()) * \
        sc.cfg.tube_inner_radius_m


def sweep_cpu_estimate(scs: list, threads: int, seconds: float, n_sample: int = 16):
    """Scenarios/s of the reference's CPU path on a bounded sample of the sweep. The scenarios are ranked
    by optical depth and n_sample of them, evenly spaced in that ranking (the densest included), are
    prepared (particle precompute, timed) and traced on a photon sample (timed). Every scenario of the
    sweep is then charged the precompute time and per-photon time of the sampled scenario nearest to it
    in the ranking, times its own photon count; the rate is scenarios over the summed time."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_harness as H
    from tardiis_and_claritas_gb300 import scene as S
    kind = "reference" if H.reference_available() else "port"
    build = "reference_fast" if kind == "reference" else "port"  # the reference's source built with -O3
    order = sorted(range(len(scs)), key=lambda i: optical_depth_proxy(scs[i]))
    m_s = min(n_sample, len(scs))
    ranks = sorted({round(k * (len(scs) - 1) / max(m_s - 1, 1)) for k in range(m_s)})
    idx = [order[r] for r in ranks]
    budget = seconds / len(idx)
    traced, cost = 0, {}
    for i in idx:
        sc = scs[i]
        t0 = time.perf_counter()
        o = H.OracleRun(build, sc.cfg, sc.particles)
        t_prep = time.perf_counter() - t0
        # grow the photon sample until it takes about its share of the time budget (or is the whole run)
        m = min(sc.n_photons, 2000)
        while True:
            t1 = time.perf_counter()
            o.trace(S.run_params(m, seed=sc.seed + 7), threads=threads)
            dt = time.perf_counter() - t1
            if m >= sc.n_photons or dt >= 0.5 * budget:
                break
            m = int(min(sc.n_photons, m * min(8.0, max(2.0, budget / max(dt, 1e-4)))))
        o.close()
        traced += m
        cost[i] = (t_prep, dt / m)
    total = 0.0
    for r, i in enumerate(order):
        near = idx[min(range(len(ranks)), key=lambda k: abs(ranks[k] - r))]
        t_prep, t_photon = cost[near]
        total += t_prep + scs[i].n_photons * t_photon
    return {"value": len(scs) / total, "unit": "scenarios/s", "cores": threads, "kind": kind,
            "sample": f"{len(idx)} of {len(scs)} scenarios spread over the optical-depth ranking: precompute "
                      f"timed, {traced} photons traced; each scenario charged the nearest sampled scenario's "
                      f"precompute and per-photon time times its own photon count"}


def run_sweep(args, ctx, rank: int, world: int, local_rank: int, dist, dev) -> dict:
    """The batched sweep: one step = clr_sweep_build + clr_sweep_trace of every scenario."""
    import numpy as np
    import torch
    from tardiis_and_claritas_gb300 import abi, scene as S
    scs = S.sweep_workload(SWEEP_SCENARIOS, sampler_seed=rank)
    rng_mode = abi.RNG_PHILOX if args.rng == "philox" else abi.RNG_REFERENCE_XORSHIFT
    tables = args.tables if args.tables != "auto" else ("fast" if rng_mode == abi.RNG_PHILOX else "reference")
    scenes, parts, seds = S.sweep_specs(scs, table_arithmetic=abi.TABLES_FAST if tables == "fast"
                                        else abi.TABLES_REFERENCE)
    n_photons = sum(sc.n_photons for sc in scs)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def runs(step: int):
        return [S.run_params(sc.n_photons, seed=sc.seed + 1000 * step, rng_mode=rng_mode, scenario_id=i)
                for i, sc in enumerate(scs)]

    for w in range(args.warmup):
        ctx.sweep_build(scenes, parts, seds)
        ctx.sweep_trace(runs(w))
    tuning = None
    if args.tune == "auto":
        from tardiis_and_claritas_gb300 import autotune as AT
        props = torch.cuda.get_device_properties(dev)
        # trials trace steps no timed step uses (their seeds follow the timed steps')
        tuning = AT.tune(ctx, key=f"sweep{SWEEP_SCENARIOS}-seed{rank}-{args.rng}", photons=n_photons, reps=1,
                         device=AT.device_key(props.major, props.minor, props.multi_processor_count),
                         trace=lambda i: ctx.sweep_trace(runs(args.warmup + args.steps + 1 + i)))
    torch.cuda.synchronize()
    if dist:
        dist.barrier(device_ids=[local_rank])
    sampler = ClockSampler(local_rank)
    sampler.start()
    build_ms, trace_ms, walls = [], [], []
    launches = passes = 0
    all_tallies = []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.sweep_build(scenes, parts, seds)
        build_ms.append(ctx.last_kernel_ms())
        T = ctx.sweep_trace(runs(args.warmup + k))
        trace_ms.append(ctx.last_kernel_ms())
        walls.append(time.perf_counter() - t0)
        nl, npass = ctx.last_launches()
        launches += nl
        passes += npass
        all_tallies.extend(T)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    dev_ms = float(sum(build_ms) + sum(trace_ms))
    wall_s = float(sum(walls))
    if dist:
        t = torch.tensor([dev_ms, wall_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms, wall_s = float(t[0].item()), float(t[1].item())
    value = world * SWEEP_SCENARIOS * args.steps / (dev_ms * 1e-3)
    e2e = world * SWEEP_SCENARIOS * args.steps / wall_s
    h2d = sum(int(p.n_bins) * (4 * 8 + 2 * 8 + 1) for p in parts) + SWEEP_SCENARIOS * (
        abi.C.sizeof(abi.SceneParams) + abi.C.sizeof(abi.RunParams) + 8)
    d2h = SWEEP_SCENARIOS * (abi.C.sizeof(abi.Tallies) + 8 * 8 + 4 * 8 + 4) + 4
    from tardiis_and_claritas_gb300 import workcount as WC
    trace_s = float(sum(trace_ms)) * 1e-3 / args.steps
    # roofline of the sweep's trace from its own event counters (workcount.py) against the FP32 lane rate
    wk = WC.work(all_tallies)
    lane_peak = ctx.calibrate(0) / 2.0
    ach = wk["fp32_ops"] / (float(sum(trace_ms)) * 1e-3)
    roofline = {"bound": "fp32-issue", "unit": "Tops/s", "achieved": ach / 1e12, "peak": lane_peak / 1e12,
                "frac": ach / lane_peak, "ops_per_photon": wk["ops_per_photon"],
                "peak_source": "FP32 FFMA lane-operation rate measured in this run by the library's calibration kernel",
                "work": "FP32-equivalent operations from the event counters of the timed sweep traces (workcount.py)",
                "traffic": None,
                "dominant": "the sweep's trace: all wavefront stage kernels over every scenario's photons"}
    line = {"metric": "scenarios/s (at fixed tally error)", "value": value, "unit": "scenarios/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 transport, f64 Mie",
            "data": "synthetic (seeded)",
            "config": {"workload": SWEEP_WORKLOAD, "scenarios": SWEEP_SCENARIOS, "photons_per_step": n_photons,
                       "rng": args.rng, "tables": tables, "l2": "flushed between steps (256 MiB write); tables exceed L2"},
            "e2e": {"value": e2e, "unit": "scenarios/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "steps": args.steps,
                    "includes": "host wall time of clr_sweep_build (scenario upload, batched Mie/phase tables, rates) "
                                "+ clr_sweep_trace (all scenarios, tallies to host)"},
            "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline,
            "sweep": {"build_ms": float(np.mean(build_ms)), "trace_ms": float(np.mean(trace_ms)),
                      "photons_per_s": n_photons / trace_s, "passes_per_trace": passes / args.steps,
                      "detected_native_total": int(sum(int(t["hw_native"].sum()) for t in T)),
                      "engine_settings": {"tuned": tuning["config"], "gain_over_defaults": tuning["gain"],
                                          "source": {"user": "tuning cache", "shipped": "the package's tuning "
                                                     "table (same search, same GPU type)"}.get(tuning["cached"],
                                                                                              "searched in this run"),
                                          "trials": tuning["trials"]} if tuning else None}}
    ctx.set_engine_config(None)
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = sweep_cpu_estimate(scs, os.cpu_count() or 1, args.cpu_seconds)
    return line


def run_surrogate(args, rank: int, world: int, local_rank: int, dist, dev) -> dict:
    """Surrogate workload: Monte Carlo training data from the batched sweep, training of the tensor-core
    network, check against Monte Carlo with 100x the photons, then timed inference (a step = one
    batch of 65536 queries)."""
    import numpy as np
    import torch
    from tardiis_and_claritas_gb300 import lib as L, surrogate as G
    ctx = L.Context(local_rank)
    t0 = time.perf_counter()
    train = G.make_dataset(ctx, args.sur_train, args.sur_photons, sampler_seed=1000 + rank, seed_base=0)
    test = G.make_dataset(ctx, args.sur_test, 100 * args.sur_photons, sampler_seed=2000 + rank, seed_base=10 ** 6)
    # the precision judge: few held-out scenarios at many photons, so that the judge's own noise is a small
    # part of the measured difference (a few scenarios per engine execution keeps each trace bounded)
    judge = G.make_dataset(ctx, args.sur_judge, int(args.sur_judge_photons), sampler_seed=4000 + rank,
                           seed_base=2 * 10 ** 6, chunk=8) if args.sur_judge > 0 else None
    data_s = time.perf_counter() - t0
    model = G.Surrogate(local_rank, max_batch=65536, seed=rank)
    hist = model.fit(train, epochs=args.sur_epochs, batch=2048)
    err = G.mc_error(model, test)
    base = G.linear_baseline(train, test)
    judged = {"held_out_at_100x_photons": G.judged_error(model, test)}
    if judge is not None:
        judged["precision_judge"] = G.judged_error(model, judge)
    # the same network trained with 1/(noise variance + floor^2) label weights, for comparison
    judged_u = None
    if getattr(args, "sur_compare_weighted", True):
        model_u = G.Surrogate(local_rank, max_batch=65536, seed=rank)
        model_u.fit(train, epochs=args.sur_epochs, batch=2048, weight_floor=G.WEIGHT_FLOOR_REL)
        judged_u = {"held_out_at_100x_photons": G.judged_error(model_u, test)}
        if judge is not None:
            judged_u["precision_judge"] = G.judged_error(model_u, judge)
        model_u.close()
    # surrogate-in-the-loop inversion of concentration (Monte Carlo as check and fallback)
    inv = G.inversion_study(ctx, model, n=args.inv_scenarios, photons=4_000_000, mc_only=args.inv_mc_only,
                            sampler_seed=3000 + rank) if args.inv_scenarios > 0 else None
    ctx.close()
    batch = 65536
    x = torch.randn(batch, 6, generator=torch.Generator().manual_seed(1)).to(dev)
    for _ in range(args.warmup):
        model.predict_device(x)
    torch.cuda.synchronize()
    if dist:
        dist.barrier(device_ids=[local_rank])
    sampler = ClockSampler(local_rank)
    sampler.start()
    ms = []
    for _ in range(args.steps):
        model.predict_device(x)
        ms.append(model.net.last_ms())
    torch.cuda.synchronize()
    clocks = sampler.stop()
    dev_s = float(sum(ms)) * 1e-3
    if dist:
        t = torch.tensor([dev_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_s = float(t.item())
    value = world * batch * args.steps / dev_s
    speed = G.query_speed(model, batch=batch, reps=max(3, args.steps))
    flop_q = 2.0 * (6 * 256 + 3 * 256 * 256 + 256 * 3)
    peaks = measured_peaks()
    peak = peaks.get("bf16_tflops") or 1900.0
    ach = flop_q * value / world / 1e12
    mc_s_per_scen = train.mc_seconds / len(train.x)
    mc_s_check = test.mc_seconds / len(test.x)
    line = {"metric": "surrogate queries/s (error vs Monte Carlo stated)", "value": value,
            "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 weights/activations, f32 accumulation", "data": "synthetic (seeded); labels from this MC",
            "config": {"workload": "surrogate MLP 6-256x4(SiLU)-3 of the sweep's detector signals (channels 9, 0, 17); "
                                   f"trained on {args.sur_train} sweep scenarios at {args.sur_photons:.0e} photons, "
                                   f"checked on {args.sur_test} held-out scenarios at {100 * args.sur_photons:.0e} "
                                   f"photons and {args.sur_judge} at {args.sur_judge_photons:.0e}; inference batch "
                                   "65536",
                       "inference_batch": batch, "l2": "inputs resident (3 MB); weights L2-resident by design"},
            "e2e": {"value": speed["e2e_queries_per_s"] * world, "unit": "queries/s",
                    "h2d_bytes_per_step": batch * 6 * 4, "d2h_bytes_per_step": batch * 3 * 4},
            "gpu_launches": args.steps, "clocks": clocks,
            "roofline": {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                         "peak_source": "bf16_tflops of MEASURED_PEAKS.json" if peaks.get("bf16_tflops") else "fallback",
                         "traffic": None, "flop_per_query": flop_q},
            "surrogate": {"vs_mc": err, "judged": judged,
                          "weighted_loss": {"weight_floor": G.WEIGHT_FLOOR_REL, "judged": judged_u},
                          "judge": {"scenarios": args.sur_judge, "photons_each": int(args.sur_judge_photons)},
                          "linear_baseline": base,
                          "train": {"scenarios": len(train.x), "photons_each": args.sur_photons,
                                    "epochs": args.sur_epochs, "final_loss": hist[-1][2],
                                    "kept_epoch": model.best_epoch, "validation_share": 0.05,
                                    "loss": "unweighted mean squared error of the standardised log10 signals",
                                    "train_seconds": model.train_seconds,
                                    "ms_per_epoch": float(np.median([h[3] for h in hist]))},
                          "mc": {"data_seconds_wall": data_s, "train_labels_device_s_per_scenario": mc_s_per_scen,
                                 "check_device_s_per_scenario": mc_s_check},
                          "speedup_vs_mc_at_training_photons": (value / world) * mc_s_per_scen,
                          "speedup_vs_mc_at_check_photons": (value / world) * mc_s_check,
                          "inversion": inv}}
    model.close()
    return line


def _timed_traces(ctx, runs: list, flush) -> tuple:
    """Device seconds and tallies of one trace per run, L2 flushed before each."""
    import torch
    ms, tallies = 0.0, []
    for r in runs:
        flush.zero_()
        torch.cuda.synchronize()
        T, _ = ctx.trace(r)
        ms += ctx.last_kernel_ms()
        tallies.append(T)
    return ms * 1e-3, tallies


def rankine_subrecord(ctx, args, rng_mode, flush) -> dict:
    """The full scene as specified (a Rankine vortex from the 600 rpm stirrer with a 5 mm core) traced on the
    GPU, with the CPU restatement of this library's Rankine surface as its CPU baseline (the reference has
    no Rankine surface, so the headline line uses its localized-vortex stand-in)."""
    from tardiis_and_claritas_gb300 import scene as S
    cfg, parts, grid, zmax = S.full_scene_workload(surface="rankine_vortex")
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec(grid, zmax))
    n, k = 100_000_000, 2
    _timed_traces(ctx, [S.run_params(n // 10, seed=5, rng_mode=rng_mode)], flush)
    secs, tallies = _timed_traces(ctx, [S.run_params(n, seed=11 + i, rng_mode=rng_mode) for i in range(k)], flush)
    out = {"workload": "full scene with the Rankine free surface (600 rpm stirrer, 5 mm core, dip "
                       f"{1e3 * cfg.vortex_wall_center_height_difference_m:.2f} mm), otherwise as the headline",
           "photons_per_step": n, "steps": k, "value": n * k / secs, "unit": "photons/s",
           "tally_error": channel_error(tallies, secs)}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_harness as H
        o = H.OracleRun("port", cfg, parts, grid=grid, grid_zmax=zmax)
        threads = os.cpu_count() or 1
        m = 200_000
        t = time.perf_counter()
        T, _ = o.trace(S.run_params(m, seed=3), threads=threads)
        dt = time.perf_counter() - t
        o.close()
        cpu_err = channel_error([T], dt)
        out["cpu_baseline"] = {"value": m / dt, "unit": "photons/s", "cores": threads, "kind": "port",
                               "sample": f"{m} photons, {dt:.1f} s", "tally_error": cpu_err}
        out["equal_error_speedup"] = equal_error_speedup(out["tally_error"], cpu_err)
    return out


def weighted_subrecord(ctx, args) -> dict:
    """The dense stress case (2 um clay, sigma_g 1.5, 20 g/L: optical depth above 100 across the cell; a
    1200 rpm Rankine stirrer) with the clay absorbing as the reference's kaolin table says (k 1e-4 to 8e-4 by
    diameter), traced analog and weighted (implicit capture, Russian roulette below a weight of 1e-4,
    survivors at 1e-3): photons/s and tally error of each, and the weighted estimator's gain at equal
    error. A bounded number of photons per run (the specification's 1e9 would take minutes)."""
    from tardiis_and_claritas_gb300 import abi, scene as S
    dh = S.stirrer_rankine_delta_h(1200.0, 0.005, 0.0125)
    cfg = S.small_cell_config(free_surface_model="rankine_vortex", vortex_wall_center_height_difference_m=dh,
                              vortex_core_radius_m=0.005, particle_surface_rms_slope_deg=0.0,
                              wave_surface_rms_height_m=0.0)
    cfg.validate()
    parts = S.kaolin_clay_particles(20000.0, n_bins=16, median_um=2.0, sigma_g=1.5, d_min_um=0.5, d_max_um=10.0)
    ctx.set_scene(cfg.to_scene_params())
    ctx.build_particles(parts.spec(cfg), cfg.sediment_spec())
    import torch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    n = 500_000
    out = {"workload": "dense stress: 16-bin clay (median 2 um, sigma_g 1.5, 0.5-10 um) with the kaolin table's n and "
                       "k at 20 g/L, Rankine 1200 rpm, 5 mm core, smooth spheres",
           "photons_per_run": n}
    for name, mode in (("analog", abi.WEIGHT_ANALOG), ("weighted", abi.WEIGHT_IMPLICIT)):
        def mk(seed, mode=mode):
            return S.run_params(n, seed=seed, rng_mode=abi.RNG_PHILOX, weight_mode=mode,
                                roulette_threshold=1e-4, roulette_survival=1e-3)
        _timed_traces(ctx, [mk(1)], flush)
        secs, tallies = _timed_traces(ctx, [mk(2), mk(3)], flush)
        t = tallies[-1]
        out[name] = {"value": 2 * n / secs, "unit": "photons/s", "tally_error": channel_error(tallies, secs),
                     "roulette_kills": int(t["event_counts"][abi.EV_NAMES.index("roulette_kills")]),
                     "water_steps_per_photon": float(t["event_counts"][abi.EV_NAMES.index("water_steps")]) / n,
                     "status_counts": [int(v) for v in t["status_counts"][:10]]}
    out["weighted_gain_at_equal_error"] = equal_error_speedup(out["weighted"]["tally_error"],
                                                              out["analog"]["tally_error"])
    return out


def surrogate_subrecord(args, rank, world, local_rank, dev) -> dict:
    """The surrogate (C4) in the default line, reduced: 16384 training scenarios at 1e6 photons (the full
    C4 size, 262144, is `--workload surrogate`), judged on 128 held-out scenarios at 1e8 photons with the
    judge's noise removed, and timed inference on 65536-query batches. About 90 s of GPU."""
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup = 10, 3
    sub.sur_train, sub.sur_test, sub.sur_photons, sub.sur_epochs = 16384, 128, 1_000_000, 400
    sub.sur_judge, sub.inv_scenarios, sub.sur_compare_weighted = 0, 0, False
    line = run_surrogate(sub, rank, world, local_rank, None, dev)
    sur = line["surrogate"]
    return {"metric": line["metric"], "value": line["value"], "unit": line["unit"], "e2e": line["e2e"],
            "roofline": line["roofline"], "workload": line["config"]["workload"],
            "judged_error": sur["judged"]["held_out_at_100x_photons"], "median_error": sur["vs_mc"],
            "linear_baseline": sur["linear_baseline"], "train": sur["train"], "mc": sur["mc"],
            "speedup_vs_mc_at_training_photons": sur["speedup_vs_mc_at_training_photons"],
            "speedup_vs_mc_at_check_photons": sur["speedup_vs_mc_at_check_photons"],
            "reduced": "16384 training scenarios of the C4 sampler (C4: 262144) and 128 judge scenarios at 1e8 "
                       "photons (C4: 4096); the full size runs with --workload surrogate"}


def sweep_subrecord(args, ctx, rank, world, local_rank, dev) -> dict:
    """The 512-scenario batched sweep (scenarios/s) in the default line: two timed steps."""
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup = 2, 1
    line = run_sweep(sub, ctx, rank, world, local_rank, None, dev)
    keep = ("metric", "value", "unit", "steps", "ms_per_step", "e2e", "roofline", "sweep", "cpu_baseline")
    out = {k: line[k] for k in keep if k in line}
    out["workload"] = SWEEP_WORKLOAD
    out["tables"] = line["config"]["tables"]
    return out


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.index, self.samples, self.proc, self.thread = index, [], None, None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE, text=True)
        except (FileNotFoundError, OSError):
            return

        def read():
            for line in self.proc.stdout:
                self.samples.append([c.strip() for c in line.split(",")])

        self.thread = threading.Thread(target=read, daemon=True)
        self.thread.start()

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx.append(float(s[2]))
                for nm, v in zip(names, s[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


class CpuReference:
    """The reference's own CPU implementation of the path (its kernel source compiled for the host) or, where
    that build is absent, the CPU restatement; prepared once, then timed on bounded samples of the workload."""

    def __init__(self, name: str, threads: int):
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle_harness as H
        cfg, parts, grid, zmax, _ = workload(name)
        self.kind = "reference" if H.reference_available() else "port"
        # the reference's own source built for speed (-O3, contraction allowed); the port where it is absent
        self.build = "reference_fast" if self.kind == "reference" else "port"
        self.o = H.OracleRun(self.build, cfg, parts, grid=grid, grid_zmax=zmax)
        self.threads = threads
        self.probe = 20_000 if name == "full" else 200_000
        self.tallies = []

    def sample_size(self, seconds: float) -> int:
        from tardiis_and_claritas_gb300 import scene as S
        t = time.perf_counter()
        self.o.trace(S.run_params(self.probe, seed=7), threads=self.threads)
        dt = time.perf_counter() - t
        return max(self.probe, int(self.probe * seconds / max(dt, 1e-3)))

    def time(self, n: int, seed: int) -> float:
        """Seconds to trace n photons; the run's tallies are kept in self.tallies."""
        from tardiis_and_claritas_gb300 import scene as S
        t = time.perf_counter()
        T, _ = self.o.trace(S.run_params(n, seed=seed), threads=self.threads)
        dt = time.perf_counter() - t
        self.tallies.append(T)
        return dt

    def close(self):
        self.o.close()


def run_reference_arm(args, rank: int, world: int):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    name = args.workload
    if name == "surrogate":
        # the reference has no surrogate: it answers each query with its Monte Carlo (CPU here), at the
        # surrogate's training photon count
        from tardiis_and_claritas_gb300 import scene as S
        p = args.sur_photons
        scs = S.sweep_workload(SWEEP_SCENARIOS, sampler_seed=2000, photons=(p, p))
        vals = [sweep_cpu_estimate(scs, threads, args.cpu_seconds) for _ in range(max(1, args.steps))]
        value = sum(v["value"] for v in vals) / len(vals)
        line = {"impl": "reference", "metric": "surrogate queries/s (error vs Monte Carlo stated)",
                "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32/f64", "data": "synthetic (seeded)",
                "config": {"workload": f"one Monte Carlo run of {p:.0e} photons per query (sweep scenarios)"},
                "cpu_baseline": dict(vals[-1], value=value, unit="queries/s"),
                "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if name == "sweep":
        from tardiis_and_claritas_gb300 import scene as S
        scs = S.sweep_workload(SWEEP_SCENARIOS)
        for _ in range(args.warmup):
            sweep_cpu_estimate(scs[:1], threads, 1.0)
        vals = [sweep_cpu_estimate(scs, threads, args.cpu_seconds) for _ in range(args.steps)]
        value = sum(v["value"] for v in vals) / len(vals)
        cpu = dict(vals[-1], value=value)
        line = {"impl": "reference", "metric": "scenarios/s (at fixed tally error)", "value": value,
                "unit": "scenarios/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32/f64", "data": "synthetic (seeded)",
                "config": {"workload": SWEEP_WORKLOAD, "scenarios": SWEEP_SCENARIOS, "rng": "reference xorshift"},
                "cpu_baseline": cpu,
                "e2e": {"value": value, "unit": "scenarios/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    _, _, _, _, n_gpu = workload(name)
    ref = CpuReference(name, threads)
    n = ref.sample_size(args.cpu_seconds)
    for i in range(args.warmup):
        ref.time(max(n // 10, ref.probe), seed=100 + i)
    ref.tallies = []
    total_t = sum(ref.time(n, seed=200 + k) for k in range(args.steps))
    tallies = ref.tallies
    ref.close()
    total_n = n * args.steps
    value = total_n / total_t
    cfg_line = workload_config(name, n, "reference xorshift")
    cfg_line["gpu_arm_photons_per_step"] = n_gpu
    line = {"impl": "reference", "metric": "photons/s (at fixed tally error)", "value": value, "unit": "photons/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64",
            "data": "synthetic (seeded)", "config": cfg_line,
            "cpu_baseline": {"value": value, "unit": "photons/s", "cores": threads, "kind": ref.kind,
                             "build": "the reference's CUDA_SRC as host C++, -O3, OpenMP over photons"
                             if ref.kind == "reference" else "the CPU restatement, -O2, OpenMP over photons",
                             "sample": f"{n} photons of the same workload per step, {args.steps} steps"},
            "tally_error": channel_error(tallies, total_t),
            "e2e": {"value": value, "unit": "photons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["full", "small", "sweep", "surrogate"], default="full")
    ap.add_argument("--sur-train", type=int, default=262144, help="surrogate: training scenarios")
    ap.add_argument("--sur-test", type=int, default=256, help="surrogate: held-out scenarios checked by Monte Carlo")
    ap.add_argument("--sur-judge", type=int, default=64, help="surrogate: held-out scenarios of the precision judge")
    ap.add_argument("--sur-judge-photons", type=float, default=2e9,
                    help="surrogate: photons per scenario of the precision judge")
    ap.add_argument("--sur-photons", type=int, default=1_000_000, help="surrogate: photons per training scenario")
    ap.add_argument("--sur-epochs", type=int, default=400, help="surrogate: training epochs")
    ap.add_argument("--inv-scenarios", type=int, default=1024, help="surrogate: scenarios of the inversion study")
    ap.add_argument("--inv-mc-only", type=int, default=64, help="surrogate: of those, also inverted by MC alone")
    ap.add_argument("--rng", choices=["philox", "xorshift"], default="philox")
    ap.add_argument("--photons", type=int, default=0, help="override photons per step")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample length")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true",
                    help="full workload: skip the Rankine, sweep and weighted sub-records")
    ap.add_argument("--e2e-steps", type=int, default=3, help="steps of the end-to-end leg (0: skip it)")
    ap.add_argument("--tables", choices=["auto", "reference", "fast"], default="auto",
                    help="phase-table arithmetic of the sweep build (auto: fast on the Philox stream, the reference's "
                         "order of operations on the parity stream)")
    ap.add_argument("--tune", choices=["auto", "off"], default="auto",
                    help="tune the wavefront engine's scheduling settings for this GPU and scene before timing "
                         "(tallies are the same under any setting; the search is outside the timed region)")
    ap.add_argument("--engine", choices=["wavefront", "persistent"], default="wavefront",
                    help="photon engine (the persistent kernel is kept for comparison)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="gloo" if args.impl == "reference" else "nccl")
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return

    import numpy as np
    import torch
    from tardiis_and_claritas_gb300 import abi, lib as L, scene as S
    from tardiis_and_claritas_gb300 import workcount as WC

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if dist:
        dist.barrier(device_ids=[local_rank])
    if args.workload == "surrogate":
        line = run_surrogate(args, rank, world, local_rank, dist, dev)
        if rank == 0:
            print(json.dumps(line), flush=True)
        if dist:
            dist.barrier(device_ids=[local_rank])
            dist.destroy_process_group()
        return
    ctx = L.Context(local_rank)
    if args.workload == "sweep":
        line = run_sweep(args, ctx, rank, world, local_rank, dist, dev)
        if rank == 0:
            print(json.dumps(line), flush=True)
        ctx.close()
        if dist:
            dist.barrier(device_ids=[local_rank])
            dist.destroy_process_group()
        return
    cfg, parts, grid, zmax, n = workload(args.workload)
    if args.photons:
        n = args.photons
    rng_mode = abi.RNG_PHILOX if args.rng == "philox" else abi.RNG_REFERENCE_XORSHIFT
    sp = cfg.to_scene_params()
    ss = cfg.sediment_spec(grid, zmax)
    ps = parts.spec(cfg)
    ctx.set_scene(sp)
    ctx.build_particles(ps, ss)
    fp64_peak = ctx.calibrate(1)
    fp32_peak = ctx.calibrate(0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def run(step: int):
        # disjoint photon ranges per rank and step (counter-based streams: partition independent)
        off = S.replica_ray_offset(rank, step, args.warmup + args.steps + max(args.e2e_steps, 0), n)
        return S.run_params(n, seed=20261203, ray_offset=off, rng_mode=rng_mode,
                            flags=abi.RUN_PERSISTENT_KERNEL if args.engine == "persistent" else 0)

    for w in range(args.warmup):
        ctx.trace(run(w))
    tuning = None
    if args.tune == "auto" and args.engine == "wavefront":
        from tardiis_and_claritas_gb300 import autotune as AT
        props = torch.cuda.get_device_properties(dev)
        # trial photons come from a range no timed step uses (after every rank's steps)
        base = S.replica_ray_offset(world, 0, args.warmup + args.steps + max(args.e2e_steps, 0), n)
        tuning = AT.tune(ctx, lambda i: S.run_params(n, seed=20261203, ray_offset=(base + i * n) % ((1 << 32) - n),
                                                     rng_mode=rng_mode),
                         key=AT.scene_key(sp, ps, ss), photons=n,
                         device=AT.device_key(props.major, props.minor, props.multi_processor_count))
    torch.cuda.synchronize()
    if dist:
        dist.barrier(device_ids=[local_rank])
    sampler = ClockSampler(local_rank)
    sampler.start()
    kernel_ms = []
    tallies = []
    wall0 = time.perf_counter()
    launches = passes = 0
    tail_ms, tail_n = [], []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        T, _ = ctx.trace(run(args.warmup + k))
        kernel_ms.append(ctx.last_kernel_ms())
        es = ctx.engine_stats()
        launches += es["launches"]
        passes += es["passes"]
        tail_ms.append(es["tail_ms"])
        tail_n.append(es["tail_photons"])
        tallies.append(T)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    total_ms = float(sum(kernel_ms))
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * n * args.steps / (total_ms * 1e-3)

    # end to end through the public API: host PSD/grid inputs (pinned) -> precompute -> trace -> tallies to host
    e2e_steps = max(0, min(args.steps, args.e2e_steps))
    pinned = {k: torch.from_numpy(getattr(parts, k)).pin_memory() for k in ("diameter_m", "weight", "n_real", "k_imag")}
    grid_pin = torch.from_numpy(np.ascontiguousarray(grid)).pin_memory() if grid is not None else None
    ps_e = abi.ParticleSpec.from_buffer_copy(ps)
    for k, tsr in pinned.items():
        setattr(ps_e, k, abi.C.cast(tsr.data_ptr(), abi.PD))
    ss_e = abi.SedimentSpec.from_buffer_copy(ss)
    if grid_pin is not None:
        ss_e.grid = abi.C.cast(grid_pin.data_ptr(), abi.PD)
    h2d = sum(t.numel() * 8 for t in pinned.values()) + (grid_pin.numel() * 8 if grid_pin is not None else 0) \
        + abi.C.sizeof(abi.SceneParams) + abi.C.sizeof(abi.RunParams)
    d2h = abi.C.sizeof(abi.Tallies)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        ctx.set_scene(sp)
        ctx.build_particles(ps_e, ss_e)
        ctx.trace(run(args.warmup + args.steps + k))
    e2e_t = max(time.perf_counter() - t0, 1e-9)
    if dist:
        t = torch.tensor([e2e_t], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e = world * n * e2e_steps / e2e_t if e2e_steps else None

    sched = np.sum([t["sched_stats"] for t in tallies], axis=0)
    launch_s = total_ms * 1e-3 / args.steps
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = measured_peaks().get("sm_max_mhz") or 2070.0
    # roofline: algorithmic FP32-equivalent operations from this run's own event counters (workcount.py)
    # against the FP32 lane-operation rate of this GPU (its FFMA throughput, measured by the library's
    # calibration kernel in this run, one FMA = one operation)
    wk = WC.work(tallies)
    lane_peak = fp32_peak / 2.0
    ach = wk["fp32_ops"] / (total_ms * 1e-3)  # this GPU's work over the (max-over-ranks) device time
    roofline = {"bound": "fp32-issue", "unit": "Tops/s", "achieved": ach / 1e12, "peak": lane_peak / 1e12,
                "frac": ach / lane_peak,
                "peak_source": "FP32 FFMA lane-operation rate measured in this run by the library's calibration "
                               "kernel (MEASURED_PEAKS.json has no FP32 figure)",
                "work": "FP32-equivalent operations counted from the event counters of the timed traces x the "
                        "per-event table of workcount.py",
                "ops_per_photon": wk["ops_per_photon"], "events_per_photon": wk["events_per_photon"],
                "fp64": {"achieved_tflops": wk["fp64_flops"] / (total_ms * 1e-3) / 1e12,
                         "peak_tflops": fp64_peak / 1e12,
                         "frac": wk["fp64_flops"] / (total_ms * 1e-3) / fp64_peak,
                         "peak_source": "measured DFMA loop (library calibration kernel, same GPU)"},
                "traffic": None,
                "dominant": "one trace: all wavefront stage kernels (they run concurrently inside each pass graph)"}
    per = PER_PHOTON.get(args.workload) if (rng_mode == abi.RNG_PHILOX and args.engine == "wavefront") else None
    if per:
        issue_peak = 4.0 * sms * sm_mhz * 1e6  # warp instructions per second
        wi = per["warp_inst"] * n / launch_s
        roofline["traffic"] = per["dram_bytes"] * n
        roofline["traffic_unit"] = "DRAM bytes per trace (ncu dram__bytes_read+write per photon x photons)"
        roofline["hbm"] = {"achieved_gbs": per["dram_bytes"] * n / launch_s / 1e9,
                           "peak_gbs": measured_peaks().get("hbm_gbs")}
        roofline["issue_slot_cross_check"] = {
            "warp_inst_per_photon": per["warp_inst"], "achieved_twarp_inst_s": wi / 1e12,
            "peak_twarp_inst_s": issue_peak / 1e12, "frac": wi / issue_peak,
            "source": f"ncu smsp__inst_executed.sum per photon of a small trace; 4 schedulers x {sms} SMs x "
                      f"{sm_mhz:.0f} MHz"}
    stage_names = ["gen", "entry", "flight", "cond", "geom", "morph", "top", "bottom", "side", "acryl", "fin"]
    cfg_line = workload_config(args.workload, n, args.rng)
    cfg_line["engine"] = args.engine
    line = {"metric": "photons/s (at fixed tally error)", "value": value, "unit": "photons/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 transport, f64 Mie",
            "data": "synthetic (seeded)", "config": cfg_line,
            "e2e": {"value": e2e, "unit": "photons/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "steps": e2e_steps, "includes": "scene upload, Mie/table/rate/field precompute, trace, tally readback"},
            "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline,
            "tally_error": channel_error(tallies, total_ms * 1e-3),
            "engine": {"passes_per_trace": passes / args.steps, "wall_s": wall,
                       "tail_ms_per_trace": float(np.mean(tail_ms)) if tail_ms else 0.0,
                       "tail_photons_per_trace": float(np.mean(tail_n)) if tail_n else 0.0,
                       "stage_visits_per_photon": {stage_names[i]: float(sched[i] / (n * args.steps))
                                                   for i in range(len(stage_names))},
                       "fp32_peak_tflops": fp32_peak / 1e12,
                       "settings": {"tuned": tuning["config"], "defaults": abi.ENGINE_DEFAULTS,
                                    "gain_over_defaults": tuning["gain"], "trials": tuning["trials"],
                                    "cached": tuning["cached"],
                                    "search_s": None if tuning["cached"] else
                                    tuning["trials"] * tuning["default_trace_s"],
                                    "best_alternatives": sorted(tuning.get("landscape", []),
                                                                key=lambda e: e["relative_time"])[:4]}
                       if tuning else {"tuned": None, "defaults": abi.ENGINE_DEFAULTS}}}
    ctx.set_engine_config(None)  # the sub-records run their own scenes at the default settings
    if args.workload == "full" and rank == 0 and not args.no_extras:
        line["rankine"] = rankine_subrecord(ctx, args, rng_mode, flush)
        line["sweep"] = sweep_subrecord(args, ctx, rank, world, local_rank, dev)
        line["weighted"] = weighted_subrecord(ctx, args)
        try:
            line["surrogate"] = surrogate_subrecord(args, rank, world, local_rank, dev)
        except Exception as e:  # the headline line must not depend on the sub-record
            line["surrogate"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0 and world == 1 and not args.no_cpu:
        ref = CpuReference(args.workload, os.cpu_count() or 1)
        ns = ref.sample_size(args.cpu_seconds)
        dt = ref.time(ns, seed=8)
        line["cpu_baseline"] = {"value": ns / dt, "unit": "photons/s", "cores": ref.threads, "kind": ref.kind,
                                "build": "the reference's CUDA_SRC as host C++, -O3, OpenMP over photons"
                                if ref.kind == "reference" else "the CPU restatement, -O2, OpenMP over photons",
                                "sample": f"{ns} photons of the same workload, {dt:.1f} s"}
        cpu_err = channel_error(ref.tallies[-1:], dt)
        line["cpu_baseline"]["tally_error"] = cpu_err
        line["equal_error_speedup"] = equal_error_speedup(line["tally_error"], cpu_err)
        ref.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.barrier(device_ids=[local_rank])
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
