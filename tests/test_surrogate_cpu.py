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
