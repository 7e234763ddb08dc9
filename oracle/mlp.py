"""CPU restatement of the wrench surrogate's network, for checking the GPU
training kernels (test infrastructure: only tests and the smoke check use it).

The surrogate has no counterpart in the reference, so there is nothing to
pin against there; this module pins the GPU kernels instead:

* ``forward``/``backward`` evaluate the MLP x -> silu(x W0 + b0) -> ... ->
  x W3 + b3 and the gradient of the mean-squared error in FP64;
* with ``bf16=True`` they round to bfloat16 at exactly the points where the
  GPU kernels store bfloat16 (inputs, weights, activations, output and
  hidden-layer gradients), so the only remaining difference from the GPU is
  the FP32 accumulation order of the tensor-core products;
* ``finite_difference`` checks ``backward`` itself (FP64, no rounding).
"""
from __future__ import annotations

import numpy as np


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def bf16_bits_to_f32(bits: np.ndarray) -> np.ndarray:
    """bfloat16 bit patterns (uint16/int16) -> float32."""
    return (np.asarray(bits).astype(np.uint16).astype(np.uint32) << 16).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s + z * s * (1.0 - s)


def forward(x, Ws, bs, bf16: bool = False):
    """Returns (pre-activations z_l, activations a_l) with a_0 = x."""
    q = bf16_round if bf16 else (lambda t: t)
    a = [np.asarray(q(x), dtype=np.float64)]
    zs = []
    L = len(Ws)
    for l in range(L):
        z = a[-1] @ np.asarray(q(Ws[l]), dtype=np.float64) + bs[l]
        if bf16:
            z = z.astype(np.float32).astype(np.float64)
        zs.append(z)
        if l + 1 < L:
            a.append(np.asarray(q(silu(z)), dtype=np.float64))
    return zs, a


def loss(zout, target, n_out):
    d = zout[:, :n_out] - target
    return float(np.mean(d * d))


def backward(x, Ws, bs, target, n_out, bf16: bool = False):
    """Gradients (dW_l, db_l) of the mean squared error over the first n_out
    output columns."""
    q = bf16_round if bf16 else (lambda t: t)
    zs, a = forward(x, Ws, bs, bf16)
    rows = x.shape[0]
    dz = np.zeros_like(zs[-1])
    dz[:, :n_out] = 2.0 * (zs[-1][:, :n_out] - target) / (rows * n_out)
    dz = np.asarray(q(dz), dtype=np.float64)
    dWs, dbs = [None] * len(Ws), [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        dWs[l] = a[l].T @ dz
        dbs[l] = dz.sum(axis=0)
        if l > 0:
            dz = (dz @ np.asarray(q(Ws[l]), dtype=np.float64).T) * silu_grad(zs[l - 1])
            dz = np.asarray(q(dz), dtype=np.float64)
    return dWs, dbs


def finite_difference(x, Ws, bs, target, n_out, n_probe: int = 20, eps: float = 1e-6, seed: int = 0):
    """Central differences of the loss for n_probe random weight entries per
    layer; returns a list of (layer, analytic, numeric) tuples."""
    rng = np.random.default_rng(seed)
    dWs, _ = backward(x, Ws, bs, target, n_out)
    out = []
    for l, W in enumerate(Ws):
        for _ in range(n_probe):
            i, j = rng.integers(W.shape[0]), rng.integers(W.shape[1])
            Wp = [w.copy() for w in Ws]
            Wm = [w.copy() for w in Ws]
            Wp[l][i, j] += eps
            Wm[l][i, j] -= eps
            lp = loss(forward(x, Wp, bs)[0][-1], target, n_out)
            lm = loss(forward(x, Wm, bs)[0][-1], target, n_out)
            out.append((l, dWs[l][i, j], (lp - lm) / (2 * eps)))
    return out
