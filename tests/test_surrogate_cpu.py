"""CPU: the surrogate network's oracle (numpy) checked by finite differences, and its BF16 rounding."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import mlp_reference as M  # noqa: E402


def test_parameter_count_matches_the_abi():
    from tardiis_and_claritas_gb300 import lib
    assert M.N_PARAMS == lib.Network.N_PARAMS == 199939
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "claritas_gb.h")).read()
    assert "#define CLR_MLP_PARAMS 199939" in hdr


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0, 3.1415926], dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                     # halfway between 1 and 1 + 2^-7: ties to the even mantissa
    assert r[2] == 1.0                     # below halfway
    assert r[3] == 1.0 + 2 ** -7           # above halfway
    assert r[4] == -2.5 and r[5] == 0.0
    assert abs(r[6] - 3.140625) < 1e-12


@pytest.mark.parametrize("weighted", [False, True])
def test_oracle_gradient_matches_finite_differences(weighted):
    rng = np.random.default_rng(3)
    p = M.init_params(5).astype(np.float64)
    x = rng.normal(size=(16, 6))
    t = rng.normal(size=(16, 3))
    w = rng.uniform(0.0, 3.0, size=(16, 3)) if weighted else None
    loss, g = M.loss_and_grad(p, x, t, bf16_round=False, w=w)
    probe = np.concatenate([rng.choice(np.arange(0, 1536), 6), rng.choice(np.arange(1536, 1792), 3),
                            rng.choice(np.arange(1792, 67328), 8), rng.choice(np.arange(198912, M.N_PARAMS), 8)])
    eps = 1e-6
    for k in probe:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        fd = (M.loss_and_grad(pp, x, t, False, w)[0] - M.loss_and_grad(pm, x, t, False, w)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (k, fd, g[k])
    assert loss > 0


class _KnownErrorModel:
    """A stand-in surrogate whose prediction is the true signal times (1 + e), e ~ N(bias, s)."""

    def __init__(self, truth_log10, s, bias, seed):
        rng = np.random.default_rng(seed)
        self.pred = truth_log10 + np.log10(1.0 + bias + s * rng.standard_normal(truth_log10.shape))

    def predict(self, x):
        return self.pred


@pytest.mark.parametrize("s_true,hits", [(0.01, 2e4), (0.02, 5e3), (0.005, 1e5)])
def test_judged_error_removes_the_judge_noise(s_true, hits):
    """surrogate.judged_error: prediction/MC - 1 has variance s^2 + sigma_judge^2; the estimator recovers s
    (within a few bootstrap standard errors) although the judge's own noise is as large as s."""
    from tardiis_and_claritas_gb300 import surrogate as G
    rng = np.random.default_rng(1)
    m = 400
    rate = 10.0 ** rng.uniform(-5, -3, size=(m, 3))
    photons = np.full(m, 2.0 * hits / 1e-4)
    lam = rate * photons[:, None]
    counts = rng.poisson(2.0 * lam) / 2.0  # symmetric score: (native + mirror) / 2
    y = np.log10((counts + 0.5) / photons[:, None])
    judge = G.Dataset(x=np.zeros((m, 6)), y=y, hits=counts, photons=photons, mc_seconds=0.0)
    model = _KnownErrorModel(np.log10(rate), s_true, 0.0, seed=2)
    out = G.judged_error(model, judge, min_hits=100.0, boot=500)
    for name in G.SIGNAL_NAMES:
        r = out[name]
        assert r["scenarios"] > 100
        assert abs(r["rms_rel_error"] - s_true) < 4.0 * r["rms_rel_error_se"] + 0.15 * s_true, (name, r)
        assert abs(r["mean_bias"]) < 4.0 * r["mean_bias_se"] + 1e-4, (name, r)
        # the raw difference overstates the error by the judge's noise
        assert r["raw_rms_rel_difference"] > r["rms_rel_error"]
