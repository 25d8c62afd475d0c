"""CPU: the phase-angle search guide returns the whole-table search's index, restated in numpy.

The photon kernels draw a scattering angle by finding the first index j with u <= cdf[j] (clamped to the
last index) in a bin's FP32 phase CDF, as the reference's sampler does. phase_guide_kernel stores, per bin,
guide[k] = that index for u = k/256 (k = 0..256); the kernels then search only [guide[k], guide[k+1]] with
k = floor(256 u). Here the same arithmetic in float32 is checked against the whole-table search for draws
at, next to and between the cell edges, on forward-peaked, flat-tailed, stepped and two-point tables.
"""
from __future__ import annotations

import numpy as np

G = 256


def search(cdf: np.ndarray, u: np.float32, lo: int = 0, hi: int | None = None) -> int:
    hi = cdf.size - 1 if hi is None else hi
    while lo < hi:
        mid = (lo + hi) >> 1
        if u <= cdf[mid]:
            hi = mid
        else:
            lo = mid + 1
    return lo


def guide_of(cdf: np.ndarray) -> np.ndarray:
    return np.array([search(cdf, np.float32(k) / np.float32(G)) for k in range(G + 1)], dtype=np.int64)


def guided(cdf: np.ndarray, guide: np.ndarray, u: np.float32) -> int:
    k = min(int(np.float32(u) * np.float32(G)), G - 1)
    return search(cdf, u, int(guide[k]), int(guide[k + 1]))


def _tables(rng):
    nt = 1801
    th = np.linspace(0.0, np.pi, nt)
    peaked = np.cumsum(np.exp(-th / 0.01) + 1e-7)           # strongly forward-peaked, flat tail
    steps = np.cumsum(np.where(rng.uniform(size=nt) < 0.05, rng.uniform(size=nt), 0.0))  # long flat runs
    noisy = np.cumsum(rng.uniform(size=nt) ** 4)
    out = []
    for c in (peaked, steps, noisy):
        c = (c - c[0]) / (c[-1] - c[0])
        c = np.maximum.accumulate(c.astype(np.float32))
        c[-1] = np.float32(1.0)
        out.append(c)
    out.append(np.array([0.0, 1.0], dtype=np.float32))       # the two-point placeholder table
    return out


def test_guided_search_equals_whole_table_search():
    rng = np.random.default_rng(11)
    for cdf in _tables(rng):
        guide = guide_of(cdf)
        assert np.all(np.diff(guide) >= 0) and guide[0] >= 0 and guide[-1] <= cdf.size - 1
        edges = np.arange(G + 1, dtype=np.float32) / np.float32(G)
        draws = np.concatenate([
            rng.uniform(size=4000).astype(np.float32), edges[:-1],
            np.nextafter(edges[1:], np.float32(0)), np.nextafter(edges[:-1], np.float32(1)),
            cdf, np.nextafter(cdf, np.float32(0)), np.nextafter(cdf, np.float32(1)),
            np.array([0.0, np.nextafter(np.float32(1), np.float32(0)), 1.0], dtype=np.float32)])
        for u in draws:
            u = np.float32(min(max(u, 0.0), 1.0))
            assert guided(cdf, guide, u) == search(cdf, u), (cdf.size, float(u))
