"""CPU oracle of the surrogate network (test infrastructure only).

The reference has no surrogate: it answers every scenario query with a full Monte Carlo run. The
network the library trains on the GPU (6 -> 256 x4 SiLU -> 3, BF16 weights and activations, FP32
accumulation, mean-squared-error loss) is restated here in numpy, with its forward and backward pass
written out by hand and the BF16 roundings placed where the GPU kernels round (inputs, weights,
hidden activations, and the gradients at the pre-activations). Arithmetic between roundings is FP64,
so GPU and oracle agree up to FP32 accumulation order (and the occasional BF16 rounding that order
flips). With `bf16=False` nothing is rounded: that is the exact function the finite-difference
checks of the CPU tests differentiate.

Only tests/ import this module.
"""
from __future__ import annotations

import numpy as np

N_IN, WIDTH, N_OUT = 6, 256, 3
LAYERS = [(WIDTH, N_IN), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (N_OUT, WIDTH)]
N_PARAMS = sum(o * i + o for o, i in LAYERS)


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray):
    """Flat parameter vector -> [(W, b)] per layer (W as [out][in])."""
    p = np.asarray(params, dtype=np.float64)
    out, k = [], 0
    for o, i in LAYERS:
        W = p[k:k + o * i].reshape(o, i)
        k += o * i
        b = p[k:k + o]
        k += o
        out.append((W, b))
    assert k == N_PARAMS
    return out


def pack(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([W.ravel(), b.ravel()]) for W, b in layers])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, x, bf16_round: bool = True):
    """Returns (y, cache) for inputs x [n][6]."""
    R = bf16 if bf16_round else (lambda a: np.asarray(a, dtype=np.float64))
    L = unpack(params)
    h = R(x)
    cache = {"h": [h], "z": [None]}
    for li, (W, b) in enumerate(L):
        z = h @ R(W).T + b
        if li == len(L) - 1:
            cache["y"] = z
            return z, cache
        h = R(silu(z))
        cache["z"].append(z)
        cache["h"].append(h)


def loss_and_grad(params, x, t, bf16_round: bool = True, w=None):
    """(Weighted) mean squared error over the n x 3 outputs, sum w e^2 / (3 n), and its gradient (flat, like
    the parameters); w = None is the unweighted loss."""
    R = bf16 if bf16_round else (lambda a: np.asarray(a, dtype=np.float64))
    L = unpack(params)
    y, c = forward(params, x, bf16_round)
    n = x.shape[0]
    e = y - t
    we = e if w is None else np.asarray(w, dtype=np.float64) * e
    loss = float(np.mean(we * e))
    d = 2.0 * we / (3.0 * n)  # dL/dy
    grads = [None] * len(L)
    for li in range(len(L) - 1, -1, -1):
        W, _ = L[li]
        h_in = c["h"][li]
        grads[li] = (d.T @ h_in, d.sum(axis=0))
        if li == 0:
            break
        dh = d @ R(W)
        d = R(dh * dsilu(c["z"][li]))
    return loss, pack(grads)


def init_params(seed: int = 0) -> np.ndarray:
    """Uniform +-1/sqrt(fan_in) weights and biases (numpy generator; any values serve the checks)."""
    rng = np.random.default_rng(seed)
    layers = []
    for o, i in LAYERS:
        a = 1.0 / np.sqrt(i)
        layers.append((rng.uniform(-a, a, (o, i)), rng.uniform(-a, a, o)))
    return pack(layers).astype(np.float32)
