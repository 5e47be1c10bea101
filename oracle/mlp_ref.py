"""CPU oracle of the proposal network (test infrastructure only).

The network (n_in -> 128 x depth GELU -> 1, include/mepi_mlp.h) has no
counterpart in the reference; this module restates its arithmetic in numpy
so that the CUDA forward pass, its gradients and its training can be checked:

* ``emulate=True`` rounds to BF16 at exactly the points the CUDA kernels do
  (inputs, layer weights, post-GELU activations, pre-activation gradients that
  enter a GEMM) and accumulates every product in float64, so the CUDA results
  (FP32 accumulation) agree to FP32 rounding plus rare one-ulp BF16 flips;
* ``emulate=False`` is the same network in float64 without rounding, checked
  against central finite differences in the CPU tests.

Parameter layout (the C ABI's): for each layer W_l (128 x in_l, row-major)
then b_l (128); then w_o (128) and b_o.
"""
from __future__ import annotations

import math

import numpy as np

WIDTH = 128


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to BF16 (nearest, ties to even), returned as float64."""
    u = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def f32(x):
    return np.asarray(x, np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def param_count(n_in: int, depth: int) -> int:
    return (WIDTH * n_in + WIDTH) + (depth - 1) * (WIDTH * WIDTH + WIDTH) + WIDTH + 1


def unpack(p: np.ndarray, n_in: int, depth: int):
    p = np.asarray(p, np.float64)
    layers, off = [], 0
    for l in range(depth):
        ni = n_in if l == 0 else WIDTH
        W = p[off:off + WIDTH * ni].reshape(WIDTH, ni)
        off += WIDTH * ni
        b = p[off:off + WIDTH]
        off += WIDTH
        layers.append((W, b))
    wo = p[off:off + WIDTH]
    bo = p[off + WIDTH]
    return layers, wo, bo


def forward(p, x, n_in: int, depth: int, emulate: bool = True):
    """(f (rows,), cache) of the network on rows x (rows, n_in)."""
    layers, wo, bo = unpack(p, n_in, depth)
    rnd = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    h = rnd(f32(x) if emulate else x)
    cache = {"in": [h], "Z": []}
    for W, b in layers:
        Wq = rnd(W)
        Z = h @ Wq.T
        Z = f32(f32(Z) + f32(b)) if emulate else Z + b
        h = rnd(f32(gelu(Z)) if emulate else gelu(Z))
        cache["Z"].append(Z)
        cache["in"].append(h)
    f = h @ wo + bo
    return (f32(f) if emulate else f), cache


def loss_grad(p, x, y, n_in: int, depth: int, emulate: bool = True):
    """Mean squared error and its gradient (parameter layout)."""
    layers, wo, bo = unpack(p, n_in, depth)
    rnd = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    rows = x.shape[0]
    f, cache = forward(p, x, n_in, depth, emulate)
    e = f - (f32(y) if emulate else y)
    loss = float(np.mean(e * e))
    dout = 2.0 * e / rows
    hL = cache["in"][-1]
    g_wo = dout @ hL
    g_bo = dout.sum()
    dH = np.outer(dout, wo)
    grads = [None] * depth
    for l in range(depth - 1, -1, -1):
        Z = cache["Z"][l]
        g = dH * gelu_d(Z)
        if emulate:
            g = f32(g)
        gq = rnd(g)
        g_b = g.sum(axis=0)
        g_W = gq.T @ cache["in"][l]
        grads[l] = (g_W, g_b)
        if l > 0:
            dH = gq @ rnd(layers[l][0])
            if emulate:
                dH = f32(dH)
    out = []
    for g_W, g_b in grads:
        out += [g_W.ravel(), g_b]
    out += [g_wo, [g_bo]]
    return loss, np.concatenate([np.ravel(a) for a in out])


def init_params(n_in: int, depth: int, seed: int) -> np.ndarray:
    """Random parameters (N(0, 1/in) weights, small biases) for tests."""
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(depth):
        ni = n_in if l == 0 else WIDTH
        parts += [rng.normal(0.0, 1.0 / math.sqrt(ni), WIDTH * ni), rng.normal(0.0, 0.05, WIDTH)]
    parts += [rng.normal(0.0, 1.0 / math.sqrt(WIDTH), WIDTH), [0.1]]
    return np.concatenate(parts)
