"""Surrogate of the detector signals, trained on batched Monte Carlo and checked against it.

The reference answers every scenario query with a full Monte Carlo run (ClaritasForwardModel.simulate,
CLARITAS/CLARITAS.py:7160). Here a small network (libclaritas_gb.so's clr_mlp: 6 -> 256 x4 SiLU -> 3, BF16
tensor-core training and inference) maps the scenario parameters of the batched sweep to three detector
signals, and the Monte Carlo stays both its training-data source and the reference its error is measured
against:

  inputs  (6): log10 concentration [mg/L], log10 median diameter [um], sigma_g, stirrer rpm / 1000,
               particle refractive index, log10 geometric optical depth (radius x 3 C Q / (2 rho d_32),
               Q = 2: a closed form of the inputs, no Mie evaluation needed at query time)
  outputs (3): log10 of the detected fraction (symmetric score (native + mirror) / 2 per launched photon,
               plus half a count) at the 90-degree aperture (channel 9), the transmitted one (channel 0)
               and the rearmost, 170-degree one (channel 17, the backscatter signal).

Scenarios come from the sweep sampler (scene.sweep_workload); Monte Carlo labels from clr_sweep_build +
clr_sweep_trace, 512 scenarios per engine execution.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import abi, lib as L, scene as S

CHANNELS = (9, 0, 17)
SIGNAL_NAMES = ("signal_90deg", "signal_transmitted", "signal_backscatter_170deg")
FEATURE_NAMES = ("log10_concentration_mg_l", "log10_median_um", "sigma_g", "rpm_per_1000", "particle_index",
                 "log10_optical_depth")


def optical_depth(sc: S.SweepScenario) -> float:
    """Radius x extinction for Q_ext = 2 (geometric optics) of the scenario's size distribution."""
    p = sc.particles
    w = p.weight / p.weight.sum()
    return 1.5 * 2.0 * p.concentration_kg_m3 / p.density_kg_m3 * float((w / p.diameter_m).sum()) * \
        sc.cfg.tube_inner_radius_m


def features(scs: list) -> np.ndarray:
    out = np.zeros((len(scs), 6))
    for i, sc in enumerate(scs):
        q = sc.params
        out[i] = (math.log10(q["concentration_mg_l"]), math.log10(q["median_um"]), q["sigma_g"], q["rpm"] / 1000.0,
                  q["n_particle"], math.log10(max(optical_depth(sc), 1e-12)))
    return out


def signals(tallies: dict, n_photons: int) -> np.ndarray:
    sym = 0.5 * (tallies["hw_native"] + tallies["hw_mirror"]).astype(np.float64)
    return np.log10((sym[list(CHANNELS)] + 0.5) / float(n_photons))


@dataclass
class Dataset:
    x: np.ndarray          # [n][6] features
    y: np.ndarray          # [n][3] log10 signals
    hits: np.ndarray       # [n][3] symmetric scores (counts) behind y
    photons: np.ndarray    # [n]
    mc_seconds: float      # device time of the Monte Carlo that made the labels (builds + traces)
    scenarios: list = field(default_factory=list)


def monte_carlo(ctx: L.Context, scs: list, chunk: int = 512, rng: str = "philox", seed_base: int = 0,
                tables: int = abi.TABLES_FAST) -> Dataset:
    """Monte Carlo labels of the scenarios, `chunk` scenarios per sweep build + trace (fast phase tables by
    default: equal to the reference-order ones to rounding, a third of the build time)."""
    mode = abi.RNG_PHILOX if rng == "philox" else abi.RNG_REFERENCE_XORSHIFT
    ys, hs, secs = [], [], 0.0
    for c0 in range(0, len(scs), chunk):
        part = scs[c0:c0 + chunk]
        scenes, parts, seds = S.sweep_specs(part, table_arithmetic=tables)
        ctx.sweep_build(scenes, parts, seds)
        secs += ctx.last_kernel_ms() * 1e-3
        runs = [S.run_params(sc.n_photons, seed=seed_base + sc.seed, rng_mode=mode, scenario_id=i)
                for i, sc in enumerate(part)]
        T = ctx.sweep_trace(runs)
        secs += ctx.last_kernel_ms() * 1e-3
        for sc, t in zip(part, T):
            ys.append(signals(t, sc.n_photons))
            sym = 0.5 * (t["hw_native"] + t["hw_mirror"]).astype(np.float64)
            hs.append(sym[list(CHANNELS)])
    return Dataset(features(scs), np.array(ys), np.array(hs), np.array([sc.n_photons for sc in scs]), secs, scs)


def make_dataset(ctx: L.Context, n_scenarios: int, photons: int, sampler_seed: int, seed_base: int = 0,
                 chunk: int = 512) -> Dataset:
    """n_scenarios scenarios of the sweep sampler, each traced with `photons` photons."""
    scs = S.sweep_workload(n_scenarios, sampler_seed=sampler_seed, photons=(photons, photons))
    return monte_carlo(ctx, scs, seed_base=seed_base, chunk=chunk)


# relative error floor of the optional label weights: below it a label's Monte Carlo noise no longer
# dominates what the network can fit, so counts beyond ~200 gain no extra weight (a tighter floor starves the
# low-count scenarios of the transmitted channel: 32768 training scenarios, floors 0.005 / 0.02 / 0.05 gave
# 2.4 / 2.1 / 1.3 % RMS error there against 1.3 % unweighted). Training is unweighted by default: weights
# taken from the observed counts correlate with the labels' noise (an upward fluctuation earns more weight),
# and at 262144 training scenarios they biased the 90-degree signal upward (+9.9 % against +3.6 %
# unweighted on the weak-signal scenarios of the precision judge, +1.2 % against +0.5 % at 1e8 photons).
WEIGHT_FLOOR_REL = 0.05


def label_weights(data: Dataset, y_std: np.ndarray, floor_rel: float = WEIGHT_FLOOR_REL) -> np.ndarray:
    """Per-label loss weights 1 / (noise variance + floor^2) in the standardised log10 units the network fits,
    normalised to mean 1. A label's noise is that of log10 of a Poisson count: (native + mirror) = 2 x the
    symmetric score, variance (1/ln 10)^2 / counts."""
    var = (1.0 / math.log(10.0)) ** 2 / np.maximum(2.0 * data.hits, 1.0)
    var = var + (floor_rel / math.log(10.0)) ** 2
    w = 1.0 / (var / (y_std[None, :] ** 2))
    return (w / w.mean(axis=0, keepdims=True)).astype(np.float32)


class Surrogate:
    """The trained network plus its input/output standardisation."""

    def __init__(self, device: int = 0, max_batch: int = 65536, seed: int = 0):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.net = L.Network(device, max_batch=max_batch, seed=seed)
        self.x_mean = np.zeros(6)
        self.x_std = np.ones(6)
        self.y_mean = np.zeros(3)
        self.y_std = np.ones(3)
        self.history: list = []

    def fit(self, data: Dataset, epochs: int = 400, batch: int = 2048, lr: float = 2e-3, lr_min: float = 5e-5,
            seed: int = 0, weight_floor: Optional[float] = None, val_frac: float = 0.05,
            eval_every: int = 10) -> list:
        """Adam on the tensor-core network; unless weight_floor is None each label's squared error is weighted
        by the inverse of its Monte Carlo noise variance plus weight_floor^2 (label_weights). With val_frac > 0
        that share of the scenarios is held out and the parameters with the lowest (weighted) validation loss,
        checked every eval_every epochs, are kept: with labels this noisy longer training fits the noise
        (32768 scenarios: 800 epochs doubled the error of 400)."""
        torch = self.torch
        self.x_mean, self.x_std = data.x.mean(0), data.x.std(0) + 1e-12
        self.y_mean, self.y_std = data.y.mean(0), data.y.std(0) + 1e-12
        x = torch.from_numpy(((data.x - self.x_mean) / self.x_std).astype(np.float32)).to(self.dev)
        t = torch.from_numpy(((data.y - self.y_mean) / self.y_std).astype(np.float32)).to(self.dev)
        wh = label_weights(data, self.y_std, weight_floor) if weight_floor is not None else None
        w = torch.from_numpy(wh).to(self.dev) if wh is not None else None
        self.net.set_loss_weights(w.data_ptr() if w is not None else 0)
        n = x.shape[0]
        perm = np.random.default_rng(seed + 17).permutation(n)
        n_val = int(val_frac * n) if val_frac > 0 else 0
        val = torch.from_numpy(perm[:n_val].astype(np.int64)).to(self.dev)
        tr = torch.from_numpy(perm[n_val:].astype(np.int32)).to(self.dev)
        n_tr = n - n_val
        use = (n_tr // batch) * batch
        g = torch.Generator().manual_seed(seed)
        hist = []
        best = (float("inf"), -1, None)
        t0 = time.perf_counter()

        def val_loss() -> float:
            if n_val == 0:
                return float("nan")
            e = self.predict_device(x[val]) - t[val]
            v = (e * e) if w is None else (w[val] * e * e)
            return float(v.mean().item())
        for e in range(epochs):
            lr_e = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * e / max(epochs - 1, 1)))
            idx = tr[torch.randperm(n_tr, generator=g)[:use].to(self.dev)]
            loss = self.net.train(x.data_ptr(), t.data_ptr(), idx.data_ptr(), use, batch, lr_e)
            vl = val_loss() if n_val and ((e + 1) % eval_every == 0 or e == epochs - 1) else float("nan")
            if vl < best[0]:
                best = (vl, e, self.net.get_params())
            hist.append((e, lr_e, loss, self.net.last_ms(), vl))
        if best[2] is not None:
            self.net.set_params(best[2])
        self.best_epoch = best[1]
        self.train_seconds = time.perf_counter() - t0
        self.net.set_loss_weights(0)
        self.history = hist
        return hist

    def predict_device(self, x_std):
        """Standardised inputs (device tensor [n][6]) -> standardised outputs (device tensor [n][3])."""
        torch = self.torch
        y = torch.empty((x_std.shape[0], 3), dtype=torch.float32, device=self.dev)
        self.net.forward(x_std.data_ptr(), x_std.shape[0], y.data_ptr())
        return y

    def predict(self, x: np.ndarray) -> np.ndarray:
        torch = self.torch
        xs = torch.from_numpy(((x - self.x_mean) / self.x_std).astype(np.float32)).to(self.dev)
        y = self.predict_device(xs).cpu().numpy().astype(np.float64)
        return y * self.y_std + self.y_mean

    def state(self) -> dict:
        return {"params": self.net.get_params(), "x_mean": self.x_mean, "x_std": self.x_std, "y_mean": self.y_mean,
                "y_std": self.y_std}

    def load_state(self, st: dict):
        self.net.set_params(np.asarray(st["params"], dtype=np.float32))
        for k in ("x_mean", "x_std", "y_mean", "y_std"):
            setattr(self, k, np.asarray(st[k], dtype=np.float64))

    def close(self):
        self.net.close()


def mc_error(model: Surrogate, data: Dataset, min_hits: float = 2500.0) -> dict:
    """Relative error of the surrogate's signals against Monte Carlo labels (the reference), per channel, over
    scenarios whose Monte Carlo count is at least `min_hits` (relative standard error <= 1/sqrt(min_hits): 2 % at
    the default; the 90-degree aperture sees ~5e-5 of the photons, so 1e8 reference photons give ~5e3 counts)."""
    pred = model.predict(data.x)
    out = {}
    for k, name in enumerate(SIGNAL_NAMES):
        ok = data.hits[:, k] >= min_hits
        rel = np.abs(10.0 ** (pred[ok, k] - data.y[ok, k]) - 1.0)
        mc_se = 1.0 / np.sqrt(np.maximum(data.hits[ok, k], 1.0))
        out[name] = {"scenarios": int(ok.sum()), "median_rel_error": float(np.median(rel)) if ok.any() else None,
                     "p90_rel_error": float(np.quantile(rel, 0.9)) if ok.any() else None,
                     "within_1pct": float(np.mean(rel <= 0.01)) if ok.any() else None,
                     "mc_median_rel_se": float(np.median(mc_se)) if ok.any() else None}
    return out


def judged_error(model: Surrogate, judge: Dataset, min_hits: float = 2500.0, boot: int = 2000, seed: int = 0) -> dict:
    """The surrogate's relative error per channel with the judge's own noise removed: over scenarios with at
    least `min_hits` judge counts, d = prediction / MC - 1 has E[d^2] = s^2 + sigma^2 (surrogate error s, judge
    relative standard error sigma = 1/sqrt(native + mirror counts)), so s_rms^2 = mean(d^2) - mean(sigma^2).
    Standard errors of s_rms and of the mean bias come from a bootstrap over the scenarios."""
    pred = model.predict(judge.x)
    rng = np.random.default_rng(seed)
    out = {}
    for k, name in enumerate(SIGNAL_NAMES):
        ok = judge.hits[:, k] >= min_hits
        m = int(ok.sum())
        if m < 2:
            out[name] = {"scenarios": m}
            continue
        d = 10.0 ** (pred[ok, k] - judge.y[ok, k]) - 1.0
        sig2 = 1.0 / (2.0 * judge.hits[ok, k])

        def stats(ix):
            s2 = float(np.mean(d[ix] ** 2) - np.mean(sig2[ix]))
            return math.sqrt(max(s2, 0.0)), float(np.mean(d[ix]))
        s_rms, bias = stats(np.arange(m))
        bs = np.array([stats(rng.integers(0, m, m)) for _ in range(boot)])
        out[name] = {"scenarios": m, "rms_rel_error": s_rms, "rms_rel_error_se": float(bs[:, 0].std(ddof=1)),
                     "mean_bias": bias, "mean_bias_se": float(bs[:, 1].std(ddof=1)),
                     "judge_rel_se_median": float(np.median(np.sqrt(sig2))),
                     "raw_rms_rel_difference": float(np.sqrt(np.mean(d ** 2))),
                     "median_abs_rel_difference": float(np.median(np.abs(d)))}
    return out


def linear_baseline(train: Dataset, test: Dataset, min_hits: float = 2500.0) -> dict:
    """The method without the network: least squares on the same six features (plus their squares and a
    constant), same Monte Carlo reference and error measure."""
    def design(x):
        return np.hstack([np.ones((x.shape[0], 1)), x, x * x])
    coef, *_ = np.linalg.lstsq(design(train.x), train.y, rcond=None)
    pred = design(test.x) @ coef
    out = {}
    for k, name in enumerate(SIGNAL_NAMES):
        ok = test.hits[:, k] >= min_hits
        rel = np.abs(10.0 ** (pred[ok, k] - test.y[ok, k]) - 1.0)
        out[name] = {"median_rel_error": float(np.median(rel)) if ok.any() else None,
                     "p90_rel_error": float(np.quantile(rel, 0.9)) if ok.any() else None}
    return out


def query_speed(model: Surrogate, batch: int = 65536, reps: int = 20) -> dict:
    """Inference throughput on `batch`-query batches resident on the device (CUDA events around each call,
    inside the library), and end to end from host memory."""
    torch = model.torch
    x = torch.randn(batch, 6, generator=torch.Generator().manual_seed(1)).to(model.dev)
    for _ in range(3):
        model.predict_device(x)
    ms = []
    for _ in range(reps):
        model.predict_device(x)
        ms.append(model.net.last_ms())
    xh = torch.randn(batch, 6).pin_memory()
    yh = torch.empty(batch, 3).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        y = model.predict_device(xh.to(model.dev, non_blocking=True))
        yh.copy_(y)
    torch.cuda.synchronize()
    e2e = (time.perf_counter() - t0) / reps
    dev = float(np.median(ms)) * 1e-3
    return {"batch": batch, "device_s_per_batch": dev, "queries_per_s": batch / dev, "e2e_queries_per_s": batch / e2e}


# ---------------- surrogate-in-the-loop inversion (Monte Carlo as check and fallback) ----------------
def with_concentration(sc: S.SweepScenario, conc_mg_l: float) -> S.SweepScenario:
    """The scenario with another concentration (everything else, photons and seed included, unchanged)."""
    import dataclasses
    parts = dataclasses.replace(sc.particles, concentration_kg_m3=float(conc_mg_l) * 1e-3)
    params = dict(sc.params, concentration_mg_l=float(conc_mg_l))
    return dataclasses.replace(sc, particles=parts, params=params)


def _features_at(x: np.ndarray, log_c: np.ndarray) -> np.ndarray:
    """Feature rows with the concentration replaced: log10 C and the optical depth (proportional to C)."""
    out = x.copy()
    out[..., 5] = x[..., 5] + (log_c - x[..., 0])
    out[..., 0] = log_c
    return out


def surrogate_invert(model: Surrogate, x_known: np.ndarray, observed: np.ndarray, channels=(1,), lo: float = 0.0,
                     hi: float = 4.0, grid: int = 401) -> np.ndarray:
    """log10 concentration per scenario minimising the squared log-signal mismatch of the network over a grid
    of candidates (one inference call for all scenarios), refined by a parabola through the best three."""
    n = x_known.shape[0]
    cand = np.linspace(lo, hi, grid)
    xs = _features_at(np.repeat(x_known[:, None, :], grid, axis=1), np.broadcast_to(cand, (n, grid)))
    pred = model.predict(xs.reshape(n * grid, 6)).reshape(n, grid, 3)
    ch = list(channels)
    err = np.sum((pred[:, :, ch] - observed[:, None, ch]) ** 2, axis=-1)
    k = np.clip(np.argmin(err, axis=1), 1, grid - 2)
    e0, e1, e2 = err[np.arange(n), k - 1], err[np.arange(n), k], err[np.arange(n), k + 1]
    den = e0 - 2.0 * e1 + e2
    step = np.where(den > 0, 0.5 * (e0 - e2) / np.where(den > 0, den, 1.0), 0.0)
    return cand[k] + np.clip(step, -1.0, 1.0) * (cand[1] - cand[0])


def mc_signals(ctx: L.Context, scs: list, seed_base: int) -> np.ndarray:
    return monte_carlo(ctx, scs, seed_base=seed_base).y


def mc_secant_invert(ctx: L.Context, scs: list, observed: np.ndarray, start: np.ndarray, channel: int = 1,
                     tol: float = 0.005, max_iter: int = 8, seed_base: int = 5 * 10 ** 6, step: float = 0.1):
    """Monte Carlo inversion of log10 concentration for one signal: secant iterations in log C, every
    iteration one Monte Carlo run of all unfinished scenarios. Stops per scenario when the signal agrees
    within `tol` (relative). Returns (log10 C, Monte Carlo evaluations per scenario)."""
    n = len(scs)
    x0 = np.asarray(start, dtype=float).copy()
    f0 = mc_signals(ctx, [with_concentration(s, 10 ** c) for s, c in zip(scs, x0)], seed_base)[:, channel] \
        - observed[:, channel]
    evals = np.ones(n, dtype=int)
    done = np.abs(10 ** f0 - 1.0) <= tol
    # more particles lower the transmitted signal: step toward the observation
    x1 = x0 + np.where(f0 < 0, -step, step) if channel == 1 else x0 + step
    x = x0.copy()
    xa, fa = x0.copy(), f0.copy()
    xb = x1.copy()
    for it in range(max_iter):
        idx = np.nonzero(~done)[0]
        if idx.size == 0:
            break
        fb_part = mc_signals(ctx, [with_concentration(scs[i], 10 ** xb[i]) for i in idx],
                             seed_base + 100_000 * (it + 1))[:, channel] - observed[idx, channel]
        evals[idx] += 1
        fb = np.zeros(n)
        fb[idx] = fb_part
        for j, i in enumerate(idx):
            x[i] = xb[i]
            if abs(10 ** fb[i] - 1.0) <= tol:
                done[i] = True
                continue
            den = fb[i] - fa[i]
            nxt = xb[i] - fb[i] * (xb[i] - xa[i]) / den if abs(den) > 1e-12 else xb[i] + step
            xa[i], fa[i] = xb[i], fb[i]
            xb[i] = float(np.clip(nxt, -1.0, 5.0))
    return x, evals


def inversion_study(ctx: L.Context, model: Surrogate, n: int = 1024, photons: int = 4_000_000, tol: float = 0.01,
                    sampler_seed: int = 3000, mc_only: int = 0, min_tau: float = 0.1) -> dict:
    """Recover the concentration of n sweep scenarios from their transmitted signal (observed by Monte
    Carlo at the true concentration): the surrogate proposes, the Monte Carlo at the proposal checks it,
    and scenarios whose surrogate signal is off by more than `tol` fall back to Monte Carlo secant
    iterations from the surrogate's proposal. The first `mc_only` scenarios are also inverted by Monte
    Carlo alone from a mid-range start, for the cost of the method without the network."""
    import time
    # The transmitted signal carries the concentration only where the cell is not optically thin: scenarios
    # are drawn from the sweep sampler and kept when their geometric optical depth is at least min_tau.
    pool = S.sweep_workload(8 * n, sampler_seed=sampler_seed, photons=(photons, photons))
    scs = [sc for sc in pool if optical_depth(sc) >= min_tau][:n]
    n = len(scs)
    true_log_c = np.log10([sc.params["concentration_mg_l"] for sc in scs])
    t0 = time.perf_counter()
    obs = monte_carlo(ctx, scs, seed_base=7 * 10 ** 6)
    t_obs = time.perf_counter() - t0
    x = features(scs)
    t0 = time.perf_counter()
    est = surrogate_invert(model, x, obs.y)
    t_sur = time.perf_counter() - t0
    t0 = time.perf_counter()
    proposals = [with_concentration(s, 10 ** c) for s, c in zip(scs, est)]
    check_mc = monte_carlo(ctx, proposals, seed_base=8 * 10 ** 6)
    pred = model.predict(features(proposals))
    t_check = time.perf_counter() - t0
    sur_err = np.abs(10 ** (pred[:, 1] - check_mc.y[:, 1]) - 1.0)
    bad = np.nonzero(sur_err > tol)[0]
    final = est.copy()
    fb_evals = np.zeros(n, dtype=int)
    t0 = time.perf_counter()
    if bad.size:
        xb, ev = mc_secant_invert(ctx, [scs[i] for i in bad], obs.y[bad], est[bad], tol=0.5 * tol)
        final[bad] = xb
        fb_evals[bad] = ev
    t_fb = time.perf_counter() - t0
    rel_c = np.abs(10 ** (final - true_log_c) - 1.0)
    out = {"scenarios": n, "photons": photons, "tolerance": tol, "min_optical_depth": min_tau,
           "fallback_fraction": float(bad.size / n),
           "surrogate_signal_error_median": float(np.median(sur_err)),
           "concentration_rel_error_median": float(np.median(rel_c)),
           "concentration_rel_error_p90": float(np.quantile(rel_c, 0.9)),
           "mc_evaluations_per_scenario": float(1.0 + fb_evals.mean()),
           "seconds": {"observations_mc": t_obs, "surrogate_search": t_sur, "check_mc": t_check,
                       "fallback_mc": t_fb}}
    if mc_only > 0:
        m = min(mc_only, n)
        t0 = time.perf_counter()
        xm, ev = mc_secant_invert(ctx, scs[:m], obs.y[:m], np.full(m, 2.0), tol=0.5 * tol, max_iter=12)
        t_mc = time.perf_counter() - t0
        rel_m = np.abs(10 ** (xm - true_log_c[:m]) - 1.0)
        out["mc_only"] = {"scenarios": m, "mc_evaluations_per_scenario": float(ev.mean()),
                          "concentration_rel_error_median": float(np.median(rel_m)), "seconds": t_mc,
                          "seconds_per_scenario": t_mc / m}
        per_sur = (t_sur + t_check + t_fb) / n
        out["speedup_per_scenario_vs_mc_only"] = (t_mc / m) / per_sur if per_sur > 0 else None
    return out
