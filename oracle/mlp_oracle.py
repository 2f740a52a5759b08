"""ORACLE — numpy restatement of the warm-start MLP, for testing only.

Test infrastructure: only tests/ may use it, as the checker of the CUDA
kernels in collocation-solver-cuda_gb300/csrc/cs_mlp.cu.

Same network and arithmetic model as the kernels: depth linear layers with
GELU (erf form) between them, inputs and outputs normalised with the given
means and standard deviations, mean-squared-error loss on the normalised
outputs; every GEMM rounds both operands to bfloat16 (round to nearest even)
and accumulates in high precision (float64 here, float32 on the GPU).
Parameter layout: per layer W[out][in] then b[out].
"""
import math

import numpy as np


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _erf(x):
    return np.vectorize(math.erf)(x)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def unpack(params, sizes):
    """sizes: [(in, out), ...] -> list of (W, b)."""
    out, o = [], 0
    for di, dd in sizes:
        W = params[o:o + di * dd].reshape(dd, di)
        o += di * dd
        b = params[o:o + dd]
        o += dd
        out.append((W.astype(np.float64), b.astype(np.float64)))
    return out


def loss_and_grad(params, sizes, X, Y, xm, xs, ym, ys):
    """MSE of the normalised outputs and its gradient (flat, same layout)."""
    layers = unpack(params, sizes)
    a = ((X - xm) / xs).astype(np.float32).astype(np.float64)
    t = ((Y - ym) / ys).astype(np.float32).astype(np.float64)
    acts, pres = [a], []
    for li, (W, b) in enumerate(layers):
        z = bf16(acts[-1]) @ bf16(W).T + b
        if li < len(layers) - 1:
            pres.append(z)
            acts.append(gelu(z))
        else:
            acts.append(z)
    P = acts[-1]
    n = P.size
    loss = float(np.sum((P - t) ** 2) / n)
    d = 2.0 * (P - t) / n
    grads = [None] * len(layers)
    for li in range(len(layers) - 1, -1, -1):
        W, b = layers[li]
        if li < len(layers) - 1:
            d = d * gelu_grad(pres[li])
        gW = bf16(d).T @ bf16(acts[li])
        gb = d.sum(axis=0)
        grads[li] = (gW, gb)
        if li > 0:
            d = bf16(d) @ bf16(W)
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def predict(params, sizes, X, xm, xs, ym, ys):
    layers = unpack(params, sizes)
    a = ((X - xm) / xs).astype(np.float32).astype(np.float64)
    for li, (W, b) in enumerate(layers):
        z = bf16(a) @ bf16(W).T + b
        a = gelu(z) if li < len(layers) - 1 else z
    return a * ys + ym
