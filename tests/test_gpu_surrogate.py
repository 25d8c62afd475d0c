"""GPU: the surrogate network's tensor-core kernels.

1. The tcgen05 GEMM (BF16 operands, FP32 accumulation in TMEM) against a plain PyTorch FP32 product of
   the same BF16 values, including partial row tiles.
2. The network's forward pass and its gradients (clr_mlp_gradients: forward, tensor-core backward-data
   and weight-gradient products, CUDA-core thin layers) against the numpy oracle that rounds to BF16 at
   the same places (oracle/mlp_reference.py).
3. Training (captured Adam steps) reduces the loss on a smooth function of the six inputs.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import mlp_reference as M  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    from tardiis_and_claritas_gb300.build_ext import build
    build()
    return torch


@pytest.mark.parametrize("M_rows,K", [(128, 64), (300, 256), (1000, 192)])
def test_tcgen05_gemm_matches_fp32(torch_cuda, M_rows, K):
    torch = torch_cuda
    from tardiis_and_claritas_gb300 import lib as L
    g = torch.Generator(device="cpu").manual_seed(M_rows + K)
    a = torch.randn(M_rows, K, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(256, K, generator=g).to(torch.bfloat16).cuda()
    c = torch.full((M_rows, 256), float("nan"), dtype=torch.float32, device="cuda")
    L.bf16_gemm_n256(a.data_ptr(), K, b.data_ptr(), K, M_rows, K, c.data_ptr(), 256)
    ref = a.float() @ b.float().T
    torch.cuda.synchronize()
    assert torch.isfinite(c).all()
    # FP32 accumulation of exact BF16 products: only the summation order differs
    assert torch.allclose(c, ref, rtol=1e-5, atol=1e-4 * K ** 0.5), float((c - ref).abs().max())


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 6)).astype(np.float32)
    t = np.stack([np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2], np.cos(x[:, 3]) * x[:, 4], 0.3 * x[:, 5] ** 2 - x[:, 0]],
                 axis=1).astype(np.float32)
    return x, t


def test_forward_and_gradients_match_the_oracle(torch_cuda):
    torch = torch_cuda
    from tardiis_and_claritas_gb300 import lib as L
    net = L.Network(0, max_batch=1024, seed=1)
    p = M.init_params(7)
    net.set_params(p)
    assert np.array_equal(net.get_params(), p)
    x, t = _data(512, 2)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    y = torch.zeros(512, 3, device="cuda")
    net.forward(xd.data_ptr(), 512, y.data_ptr())
    y_or, _ = M.forward(p, x)
    yg = y.cpu().numpy()
    assert np.abs(yg - y_or).max() < 2e-2 * max(1.0, np.abs(y_or).max()), np.abs(yg - y_or).max()
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), 512)
    loss_or, g_or = M.loss_and_grad(p, x, t)
    assert abs(loss - loss_or) < 1e-3 * loss_or
    k = 0
    for li, (o, i) in enumerate(M.LAYERS):
        for name, cnt in (("W", o * i), ("b", o)):
            a, b = g[k:k + cnt].astype(np.float64), g_or[k:k + cnt]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            cos = float(a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30))
            assert rel < 2e-2 and cos > 0.9998, (li + 1, name, rel, cos)
            k += cnt
    net.close()


def test_weighted_gradients_match_the_oracle(torch_cuda):
    """clr_mlp_set_loss_weights: the loss sum w (y-t)^2 / (3n) and its gradients, against the numpy oracle."""
    torch = torch_cuda
    from tardiis_and_claritas_gb300 import lib as L
    net = L.Network(0, max_batch=1024, seed=1)
    p = M.init_params(9)
    net.set_params(p)
    x, t = _data(512, 6)
    w = np.random.default_rng(3).uniform(0.0, 4.0, size=(512, 3)).astype(np.float32)
    w[::7] = 0.0  # rows that do not count
    xd, td, wd = (torch.from_numpy(a).cuda() for a in (x, t, w))
    net.set_loss_weights(wd.data_ptr())
    loss, g = net.gradients(xd.data_ptr(), td.data_ptr(), 512)
    loss_or, g_or = M.loss_and_grad(p, x, t, w=w)
    assert abs(loss - loss_or) < 1e-3 * loss_or
    a, b = g.astype(np.float64), g_or
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 2e-2
    assert float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b))) > 0.9998
    # unset: back to the unweighted loss
    net.set_loss_weights(0)
    loss_u, _ = net.gradients(xd.data_ptr(), td.data_ptr(), 512)
    assert abs(loss_u - M.loss_and_grad(p, x, t)[0]) < 1e-3 * loss_u
    net.close()


def test_training_reduces_the_loss(torch_cuda):
    torch = torch_cuda
    from tardiis_and_claritas_gb300 import lib as L
    net = L.Network(0, max_batch=1024, seed=3)
    x, t = _data(8192, 4)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = None
    for epoch in range(30):
        idx = torch.randperm(8192, generator=torch.Generator().manual_seed(epoch)).to(torch.int32).cuda()
        loss = net.train(xd.data_ptr(), td.data_ptr(), idx.data_ptr(), 8192, 512, 2e-3)
        first = loss if first is None else first
    assert loss < 0.05 * first, (first, loss)
    # the trained weights reproduce the oracle's loss on the same data
    p = net.get_params()
    loss_or, _ = M.loss_and_grad(p, x[:1024], t[:1024])
    y = torch.zeros(1024, 3, device="cuda")
    net.forward(xd.data_ptr(), 1024, y.data_ptr())
    mse = float(((y.cpu().numpy() - t[:1024]) ** 2).mean())
    assert abs(mse - loss_or) < 0.05 * loss_or + 1e-5
    net.close()


def test_surrogate_of_monte_carlo_beats_the_method_without_it(torch_cuda):
    """Trained on batched Monte Carlo of sweep scenarios, the network predicts held-out scenarios' signals
    (checked by Monte Carlo with 100x the photons) better than a least-squares fit on the same features,
    and answers queries far faster than the Monte Carlo."""
    from tardiis_and_claritas_gb300 import lib as L, surrogate as G
    ctx = L.Context(0)
    train = G.make_dataset(ctx, 2048, 1_000_000, sampler_seed=31)
    test = G.make_dataset(ctx, 128, 20_000_000, sampler_seed=32, seed_base=10 ** 6)
    ctx.close()
    model = G.Surrogate(0, max_batch=4096, seed=0)
    hist = model.fit(train, epochs=300, batch=1024)
    assert hist[-1][2] < 0.2 * hist[0][2]
    # the 90-degree aperture sees ~5e-5 of the photons: check scenarios with >= 400 counts there (5 % error)
    err = G.mc_error(model, test, min_hits=400.0)
    base = G.linear_baseline(train, test, min_hits=400.0)
    assert err["signal_transmitted"]["scenarios"] >= 100, err
    assert err["signal_transmitted"]["median_rel_error"] < 0.5 * base["signal_transmitted"]["median_rel_error"], \
        (err, base)
    for name in G.SIGNAL_NAMES:
        if err[name]["scenarios"] >= 10:
            assert err[name]["median_rel_error"] < base[name]["median_rel_error"], (name, err[name], base[name])
    speed = G.query_speed(model, batch=4096, reps=5)
    assert speed["queries_per_s"] > 1e3 * len(test.x) / test.mc_seconds
    model.close()


def test_surrogate_in_the_loop_inversion(torch_cuda):
    """Concentrations recovered from transmitted signals: the network proposes, the Monte Carlo checks and
    takes over where the network is off by more than 1 %; the result is as accurate as a Monte Carlo-only
    inversion and needs far fewer Monte Carlo runs."""
    from tardiis_and_claritas_gb300 import lib as L, surrogate as G
    ctx = L.Context(0)
    train = G.make_dataset(ctx, 4096, 1_000_000, sampler_seed=41)
    model = G.Surrogate(0, max_batch=8192, seed=1)
    model.fit(train, epochs=300, batch=2048)
    out = G.inversion_study(ctx, model, n=48, photons=2_000_000, mc_only=16, sampler_seed=43)
    ctx.close()
    model.close()
    assert out["scenarios"] == 48
    assert out["concentration_rel_error_median"] < 0.05, out
    assert out["mc_evaluations_per_scenario"] < out["mc_only"]["mc_evaluations_per_scenario"], out
