"""The reference host's partitions of detected rays by per-ray counters, restated over per-ray records (test
infrastructure): interaction and geometric order, per-channel counter sums, the event-history masks
(CLARITAS/CLARITAS.py:5265-5321) and the acrylic-reflection order (:8114-8123), in the layout of the device
counts in clr_tallies.
"""
from __future__ import annotations

import numpy as np

from tardiis_and_claritas_gb300 import abi

SUM_FIELDS = ("interaction_count", "geometric", "wave", "coherent", "morphology", "entry_reflections",
              "internal_reflections")


def history_masks(rec):
    """The reference's event-history masks (CLARITAS/CLARITAS.py:5265-5321) over the per-ray records."""
    ic, g, w = rec["interaction_count"], rec["geometric"], rec["wave"]
    coh, mor = rec["coherent"], rec["morphology"]
    per, pir, pabs = rec["entry_reflections"], rec["internal_reflections"], rec["absorptions"]
    single, multiple, surface = ic == 1, ic >= 2, (g > 0) | (mor > 0)
    m = {
        "any_particle": ic > 0, "any_geometric": g > 0, "any_wave": w > 0, "any_coherent_wave": coh > 0,
        "any_morphology_wave": mor > 0, "any_entry_reflection": per > 0, "any_internal_reflection": pir > 0,
        "ballistic": ic == 0, "single_interaction": single, "single_entry_reflection": single & (per > 0),
        "multiple_interaction": multiple, "interaction_order_2": ic == 2, "interaction_order_3": ic == 3,
        "interaction_order_4plus": ic >= 4, "exactly_one_geometric": single & (g == 1) & (w == 0),
        "exactly_one_wave": single & (g == 0) & (w == 1), "single_coherent_wave_escape": single & (coh == 1),
        "single_external_entry_reflection_escape": single & (per > 0),
        "single_internal_reflection_escape": single & (pir > 0),
        "single_surface_transmission_escape": single & surface & (per == 0) & (pir == 0) & (pabs == 0),
        "mixed_geometric_wave": multiple & (g > 0) & (w > 0),
        "geometric_only_multiple": multiple & (g > 0) & (w == 0),
        "wave_only_multiple": multiple & (g == 0) & (w > 0),
        "multiple_with_entry_reflection": multiple & (per > 0),
        "multiple_with_internal_reflection": multiple & (pir > 0),
    }
    return [m[k] for k in abi.PATH_MASK_NAMES]


def partitions_from_records(rec):
    order = np.zeros((2, 6, 18), np.int64)
    gorder = np.zeros((2, 6, 18), np.int64)
    sums = np.zeros((len(SUM_FIELDS), 2, 18), np.int64)
    masks = np.zeros((2, abi.N_PATH_MASKS, 18), np.int64)
    acr = np.zeros((2, 5, 18), np.int64)
    oi = np.minimum(rec["interaction_count"], 5)
    gi = np.minimum(rec["geometric"], 5)
    ai = np.minimum(rec["cell_inner_reflections"] + rec["cell_outer_reflections"]
                    + rec["bottom_inner_reflections"] + rec["bottom_outer_reflections"], 4)
    hm = history_masks(rec)
    for side, key in ((0, "native_id"), (1, "mirror_id")):
        ids = rec[key]
        ok = (ids >= 0) & (ids < 18)
        np.add.at(order[side], (oi[ok], ids[ok]), 1)
        np.add.at(gorder[side], (gi[ok], ids[ok]), 1)
        np.add.at(acr[side], (ai[ok], ids[ok]), 1)
        for k, f in enumerate(SUM_FIELDS):
            np.add.at(sums[k, side], ids[ok], rec[f][ok].astype(np.int64))
        for k, mk in enumerate(hm):
            np.add.at(masks[side, k], ids[ok & mk], 1)
    return order, gorder, sums, masks, acr
