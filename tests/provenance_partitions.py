"""The reference host's causal partitions of detected rays, restated over per-ray arrays (test infrastructure).

CLARITAS/CLARITAS.py:8063-8160 (first/last bin, event type and deflection, wall paths, acrylic returns)
and :8470-8481 (the H170 deflection histograms) build, from the per-ray outputs of trace_kernel and the
detector ids of score_detectors_kernel, one 18-vector per partition and detector side. The arrays here
have the layout of clr_path_provenance (include/claritas_gb.h), so that device counts compare directly.
"""
from __future__ import annotations

import numpy as np

N_DET = 18
N_TYPES = 8
H170_EDGES = np.asarray([0.0, 30.0, 60.0, 90.0, 120.0, 150.0, 180.0001])

# columns of the reference's per-ray provenance ints (oracle_harness.OracleRun.trace_provenance)
FIRST_TYPE, LAST_TYPE, LAST_ORDER, FIRST_BACK, FIRST_HEMI = 0, 1, 2, 3, 4
BIN_COLS = (5, 6, 7, 8, 9, 10)  # first/last particle, geometric, wave bin
ACR_RETURN, AFTER_RETURN = 11, 12


def partitions(ic, native_id, mirror_id, prov, defl, max_bins: int = 64) -> dict:
    """defl: [n][2] first/last deflection, or [n][5] with the path inside particles, its optical length
    and the water path after the last event, which add the causal path sums (:8142-8160)."""
    ic = np.asarray(ic)
    first_type, last_type = prov[:, FIRST_TYPE], prov[:, LAST_TYPE]
    first_angle = defl[:, 0].astype(np.float64)
    last_angle = defl[:, 1].astype(np.float64)
    valid = last_type > 0
    with np.errstate(invalid="ignore"):
        fav = valid & np.isfinite(first_angle) & (first_angle >= 0.0)
        lav = valid & np.isfinite(last_angle) & (last_angle >= 0.0)
    acr = prov[:, ACR_RETURN] > 0
    wall = np.where(ic == 0, 0, np.where(acr, 2, 1))
    out = {
        "bin_hits": np.zeros((6, 2, max_bins, N_DET), np.int64),
        "first_type_hits": np.zeros((2, N_TYPES, N_DET), np.int64),
        "last_type_hits": np.zeros((2, N_TYPES, N_DET), np.int64),
        "wall_hits": np.zeros((2, 3, N_DET), np.int64),
        "after_return_hits": np.zeros((2, N_DET), np.int64),
        "first_backscatter_hits": np.zeros((2, N_DET), np.int64),
        "first_source_hemisphere_hits": np.zeros((2, N_DET), np.int64),
        "first_angle_sum": np.zeros((2, N_DET)), "first_angle_count": np.zeros((2, N_DET), np.int64),
        "last_angle_sum": np.zeros((2, N_DET)), "last_angle_count": np.zeros((2, N_DET), np.int64),
        "last_type_angle_sum": np.zeros((2, N_TYPES, N_DET)),
        "last_type_angle_count": np.zeros((2, N_TYPES, N_DET), np.int64),
        "h170_last_angle_hits": np.zeros((2, N_TYPES, 6), np.int64),
        "h170_first_angle_hits": np.zeros((2, 6), np.int64),
    }
    paths = defl.shape[1] >= 5
    if paths:
        ip, io, wa = (defl[:, k].astype(np.float64) for k in (2, 3, 4))
        with np.errstate(invalid="ignore"):
            path_valid = valid & np.isfinite(ip) & np.isfinite(io) & np.isfinite(wa) & (wa >= 0.0)
        for k in ("causal_internal_path_sum", "causal_internal_opl_sum", "causal_post_last_water_path_sum",
                  "causal_last_order_sum"):
            out[k] = np.zeros((2, N_DET))
        out["causal_path_count"] = np.zeros((2, N_DET), np.int64)
    for side, ids in enumerate((np.asarray(native_id), np.asarray(mirror_id))):
        ok = (ids >= 0) & (ids < N_DET)
        for k, col in enumerate(BIN_COLS):
            b = prov[:, col]
            m = ok & (b >= 0) & (b < max_bins)
            np.add.at(out["bin_hits"][k, side], (b[m], ids[m]), 1)
        for code in range(1, N_TYPES):
            np.add.at(out["first_type_hits"][side, code], ids[ok & (first_type == code)], 1)
            np.add.at(out["last_type_hits"][side, code], ids[ok & (last_type == code)], 1)
            m = ok & lav & (last_type == code)
            np.add.at(out["last_type_angle_sum"][side, code], ids[m], last_angle[m])
            np.add.at(out["last_type_angle_count"][side, code], ids[m], 1)
        np.add.at(out["wall_hits"][side], (wall[ok], ids[ok]), 1)
        np.add.at(out["after_return_hits"][side], ids[ok & (prov[:, AFTER_RETURN] > 0)], 1)
        np.add.at(out["first_backscatter_hits"][side], ids[ok & valid & (prov[:, FIRST_BACK] > 0)], 1)
        np.add.at(out["first_source_hemisphere_hits"][side], ids[ok & valid & (prov[:, FIRST_HEMI] > 0)], 1)
        np.add.at(out["first_angle_sum"][side], ids[ok & fav], first_angle[ok & fav])
        np.add.at(out["first_angle_count"][side], ids[ok & fav], 1)
        np.add.at(out["last_angle_sum"][side], ids[ok & lav], last_angle[ok & lav])
        np.add.at(out["last_angle_count"][side], ids[ok & lav], 1)
        if paths:
            m = ok & path_valid
            for k, v in (("causal_internal_path_sum", ip), ("causal_internal_opl_sum", io),
                         ("causal_post_last_water_path_sum", wa),
                         ("causal_last_order_sum", prov[:, LAST_ORDER].astype(np.float64))):
                np.add.at(out[k][side], ids[m], v[m])
            np.add.at(out["causal_path_count"][side], ids[m], 1)
        h = ok & (ids == 17)
        for b in range(6):
            lo, hi = H170_EDGES[b], H170_EDGES[b + 1]
            am = h & lav & (last_angle >= lo) & (last_angle < hi)
            out["h170_last_angle_hits"][side, 0, b] += int(am.sum())
            for code in range(1, N_TYPES):
                out["h170_last_angle_hits"][side, code, b] += int((am & (last_type == code)).sum())
            out["h170_first_angle_hits"][side, b] += int((h & fav & (first_angle >= lo) & (first_angle < hi)).sum())
    return out
