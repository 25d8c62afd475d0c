"""Algorithmic work of a photon-transport run, from the run's own event counters.

The photon Monte Carlo is bound by instruction issue and divergence, not by HBM or the tensor cores, so its
roofline counts arithmetic: FP32-equivalent lane operations per event, counted once from the device source
and multiplied by the event counts every trace returns (clr_tallies). Counting convention (per lane):
an FP32 add, multiply, fused multiply-add, min/max, compare or select is 1; a division or square root 8
(the IEEE sequences); a log, exp, pow, sin or cos 8; rsqrt 2; a uniform draw of the counter-based stream 30
(a quarter of one Philox4x32-10 block: ten rounds of two 32-bit multiplies (lo and hi words), four xors and
two adds, plus the float conversion and buffer shift). FP64 work is counted separately as FP64 flops.
Loads, stores, address arithmetic, queue traffic and loop control are not algorithmic work and are not
counted; the issue-slot figure of the profile measures them.

Event types, the counter each is scaled by, and the code they run (file CLARITAS/CLARITAS.py of the
reference for the physics, csrc/ of this package for the code counted):
  photon              n_rays                     seeding, LED spot (Box-Muller: 2 draws, log, sqrt,
                                                 sin, cos), Beta(a+1, b) radiance polar angle by two
                                                 Marsaglia-Tsang gammas and sin(x)/x rejection (~1.2
                                                 tries), azimuth, normalisation, collimator test
                                                 (:4650-4697; source_segment, o_beta_radiance_polar)
  source_accepted     ray_flags[SOURCE_ACCEPTED] outer-wall hit (FP64), Fresnel, refraction, the
                                                 acrylic solid to the water (:4699-4732; entry_segment)
  water_step          event_counts[WATER_STEPS]  medium checks, surface height, free-path draw and log,
                                                 the straight-segment clearance test, move (:4734-4799;
                                                 water_flight, flight_clear)
  collision_candidate interactions + nulls       field lookup at four (r, z) nodes and the Woodcock
                                                 acceptance draw (:4780-4799; node_lookup)
  particle_event      event_counts[INTERACTIONS] channel draw and size-bin choice by node alias
                                                 tables (:4810-4816; node_sample_bin)
  coherent_mie        event_counts[COHERENT]     inverse-CDF angle (11-step binary search), azimuth,
                                                 rotation (:2632-2652; o_mie_direction)
  geometric_sphere    event_counts[GEOMETRIC]    sphere placement, accessibility, entry interface,
                                                 chord, exit interface (:2436-2599; f_sphere_sampled)
  particle_reflection PARTICLE_REFLECTIONS       one more interface and chord inside a particle
  morphology          event_counts[MORPHOLOGY]   spheroid entry, chords and exit (:2783-2849)
  boundary            cell, top, bottom events   the exact wall/surface roots of a boundary flight,
                                                 normal, Fresnel, reflection or refraction (:4982-5065)
  closure_trial       conditional_stats[1] + [2] a rejected candidate history of a conditional
                                                 closure (:4491-4536)
  scored_exit         ray_flags[VALID_AIR]       the 18 bores tested for the native and mirrored ray,
                                                 photodiode angle, legacy windows (:4237-4436)
"""
from __future__ import annotations

import numpy as np

from . import abi

# FP32-equivalent lane operations per event (see the module docstring for the convention and the code)
OPS = {
    "photon": 650,
    "source_accepted": 350,
    "water_step": 140,
    "collision_candidate": 85,
    "particle_event": 120,
    "coherent_mie": 180,
    "geometric_sphere": 480,
    "particle_reflection": 160,
    "morphology": 600,
    "boundary": 270,
    "closure_trial": 250,
    "scored_exit": 1150,
}
# FP64 flops per event (the double-precision root and acrylic arithmetic the reference keeps)
FP64_FLOPS = {"source_accepted": 90, "boundary": 60}

_EV = {name: i for i, name in enumerate(abi.EV_NAMES)}
RF_SOURCE_ACCEPTED = 8   # CLR_RF_SOURCE_ACCEPTED
RF_VALID_AIR = 11        # CLR_RF_VALID_AIR


def event_counts(t: dict) -> dict:
    """Counts of each event type in one run's tallies (a dict as returned by lib.Context.trace)."""
    ev = np.asarray(t["event_counts"], dtype=np.float64)
    rf = np.asarray(t["ray_flags"], dtype=np.float64)
    cs = np.asarray(t["conditional_stats"], dtype=np.float64)
    return {
        "photon": float(t["n_rays"]),
        "source_accepted": float(rf[RF_SOURCE_ACCEPTED]),
        "water_step": float(ev[_EV["water_steps"]]),
        "collision_candidate": float(ev[_EV["interactions"]] + ev[_EV["null_collisions"]]),
        "particle_event": float(ev[_EV["interactions"]]),
        "coherent_mie": float(ev[_EV["coherent"]]),
        "geometric_sphere": float(ev[_EV["geometric"]]),
        "particle_reflection": float(ev[_EV["particle_reflections"]]),
        "morphology": float(ev[_EV["morphology"]]),
        "boundary": float(ev[_EV["cell_inner"]] + ev[_EV["cell_outer"]] + ev[_EV["top"]] + ev[_EV["bottom_inner"]]
                          + ev[_EV["bottom_outer"]]),
        "closure_trial": float(cs[1] + cs[2]),
        "scored_exit": float(rf[RF_VALID_AIR]),
    }


def work(tallies: list) -> dict:
    """Summed algorithmic work of several runs: FP32-equivalent operations, FP64 flops, the counts."""
    counts = {k: 0.0 for k in OPS}
    for t in tallies:
        for k, v in event_counts(t).items():
            counts[k] += v
    ops = sum(OPS[k] * counts[k] for k in OPS)
    fp64 = sum(FP64_FLOPS.get(k, 0) * counts[k] for k in OPS)
    photons = max(counts["photon"], 1.0)
    return {"fp32_ops": ops, "fp64_flops": fp64, "counts": counts, "ops_per_photon": ops / photons,
            "events_per_photon": {k: v / photons for k, v in counts.items()}}
