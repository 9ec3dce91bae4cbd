"""ORACLE (test infrastructure only) -- CPU reference of the learned T2-guess network.

Forward and backward of the 4-layer MLP (8 -> 256 -> 256 -> 256 -> 1, SiLU)
used by the GPU engine's learned guess, in float64 numpy with the same
roundings the GPU kernels apply: weights of layers 2 and 3 and the
activations entering them are rounded to bfloat16 (round to nearest even),
and so are the loss gradients entering the backward products of those
layers; everything is accumulated in higher precision. The GPU gradients are
checked against ``grads``.

Parameter layout (one flat float32 vector, the blob the engine consumes):
  W1 [256 x 8], b1 [256], W2 [256 x 256], b2 [256], W3 [256 x 256], b3 [256],
  w4 [256], b4 [1], x_shift [8], x_scale [8], y_scale [1]
"""
from __future__ import annotations

import numpy as np

H = 256
F = 8
SIZES = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
         ("w4", (H,)), ("b4", (1,)), ("x_shift", (F,)), ("x_scale", (F,)), ("y_scale", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(blob):
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(blob[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def pack(p):
    return np.concatenate([np.asarray(p[name], dtype=np.float32).ravel() for name, _ in SIZES])


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X, rounding=True):
    """X: [M x 8] raw features -> (prediction [M], cache). rounding=False drops the
    bf16 roundings (the smooth network, for finite-difference checks of the backward pass)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    x = (np.asarray(X, dtype=np.float64) - p["x_shift"]) * p["x_scale"]
    z1 = x @ p["W1"].T + p["b1"]
    h1 = r(silu(z1))
    z2 = h1 @ r(p["W2"]).T + p["b2"]
    h2 = r(silu(z2))
    z3 = h2 @ r(p["W3"]).T + p["b3"]
    h3 = silu(z3)
    y = h3 @ p["w4"] + p["b4"][0]
    return y * p["y_scale"][0], (x, z1, h1, z2, h2, z3, h3)


def loss_and_grads(p, X, T, rounding=True):
    """Mean squared error of the scaled prediction against targets T, and its gradients
    (straight-through for the bf16 roundings, as the GPU training kernels)."""
    rnd = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    y, (x, z1, h1, z2, h2, z3, h3) = forward(p, X, rounding)
    M = X.shape[0]
    s = p["y_scale"][0]
    r = (y - np.asarray(T, dtype=np.float64)) / s           # residual in network units
    loss = float(np.mean(r * r))
    dy = 2.0 * r / M                                        # d loss / d (network output)
    g = {}
    g["w4"] = h3.T @ dy
    g["b4"] = np.array([dy.sum()])
    # the gradients entering the bf16 tensor-core products of layers 3 and 2 are
    # rounded to bf16 there (weight gradients and input gradients); the bias sums
    # and the first layer use them unrounded
    dz3 = np.outer(dy, p["w4"]) * dsilu(z3)
    g["W3"] = rnd(dz3).T @ h2
    g["b3"] = dz3.sum(0)
    dz2 = (rnd(dz3) @ rnd(p["W3"])) * dsilu(z2)
    g["W2"] = rnd(dz2).T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (rnd(dz2) @ rnd(p["W2"])) * dsilu(z1)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    return loss, g


def init(rng, x_shift, x_scale, y_scale):
    p = {}
    p["W1"] = rng.normal(size=(H, F)) * np.sqrt(2.0 / F)
    p["b1"] = np.zeros(H)
    p["W2"] = rng.normal(size=(H, H)) * np.sqrt(2.0 / H)
    p["b2"] = np.zeros(H)
    p["W3"] = rng.normal(size=(H, H)) * np.sqrt(2.0 / H)
    p["b3"] = np.zeros(H)
    p["w4"] = rng.normal(size=H) * np.sqrt(1.0 / H) * 0.1
    p["b4"] = np.zeros(1)
    p["x_shift"] = np.asarray(x_shift, dtype=np.float64)
    p["x_scale"] = np.asarray(x_scale, dtype=np.float64)
    p["y_scale"] = np.array([y_scale], dtype=np.float64)
    return p


def features(F, gov, o, rows):
    """Inputs of canonical amplitude pairs `rows` (index of (p, q), p <= q, row-major
    over the upper triangle of the (ia) x (jb) matrix, p = i*v + a).

    F: MO Fock matrix (N x N); gov: (ia|jb) as an (ov x ov) matrix. Returns
    (X [n x 8], guess [n]) with X = (guess, e_i, e_j, e_a, e_b, (ia|jb), (ib|ja), 8/N)
    and guess = (2(ia|jb) - (ib|ja)) / (e_i + e_j - e_a - e_b) (guessCC,
    src/methods/coupledCluster/mod_cc.f90:634-650)."""
    N = F.shape[0]
    v = N - o
    ov = o * v
    rows = np.asarray(rows, dtype=np.int64)
    # p = largest with p*ov - p*(p-1)/2 <= r
    start = np.array([p * ov - p * (p - 1) // 2 for p in range(ov + 1)], dtype=np.int64)
    p = np.searchsorted(start, rows, side="right") - 1
    q = p + (rows - start[p])
    i, a, j, b = p // v, p % v, q // v, q % v
    e = np.diag(F)
    g = gov[p, q]
    gx = gov[i * v + b, j * v + a]
    guess = (2.0 * g - gx) / (e[i] + e[j] - e[o + a] - e[o + b])
    X = np.stack([guess, e[i], e[j], e[o + a], e[o + b], g, gx, np.full(len(rows), 8.0 / N)], axis=1)
    return X, guess
