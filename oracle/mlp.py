"""FP64 numpy oracle of the warm-start MLP (test infrastructure only).

Only tests/ import this module; it is the checker of the library's BF16
training and inference kernels, never the thing measured or shipped.  The
network has no counterpart in the reference: it is the learned warm start of
the Lambda iteration (n_in -> width (SiLU) x depth -> n_out, linear output,
mean squared error).

Two evaluations of the same function:
  * exact: every product in FP64 -- checked against central finite
    differences, which pins the analytic backward pass;
  * bf16: the library's rounding points restated -- every GEMM operand (the
    weights, the layer inputs, the output gradients dZ) rounded to BF16 with
    round-to-nearest-even, products and sums then exact (FP64 stands in for
    the tensor cores' FP32 accumulation), biases, pre-activations and the
    bias gradients unrounded.

Flat parameter layout (the library's): per layer the weights W (fan_out x
fan_in, row-major) and then the bias (fan_out).
"""
from __future__ import annotations

import numpy as np


def bf16_round(a) -> np.ndarray:
    """float32 -> bfloat16 (round to nearest, ties to even) -> float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(f)
    if nan.any():
        out[nan] = np.nan
    return out


def layer_shapes(n_in: int, width: int, depth: int, n_out: int):
    dims = [n_in] + [width] * depth + [n_out]
    return [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]


def unflatten(params, shapes):
    """[(W, b)] views of the flat parameter vector (as float64)."""
    p = np.asarray(params, dtype=np.float64)
    out, o = [], 0
    for fo, fi in shapes:
        W = p[o:o + fo * fi].reshape(fo, fi)
        o += fo * fi
        b = p[o:o + fo]
        o += fo
        out.append((W, b))
    if o != p.size:
        raise ValueError("parameter count does not match the layer shapes")
    return out


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, shapes, X, bf16: bool = True):
    """Outputs (B, n_out) and the per-layer (inputs, pre-activations)."""
    rnd = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    H = np.asarray(X, dtype=np.float64)
    cache = []
    layers = unflatten(params, shapes)
    for li, (W, b) in enumerate(layers):
        Z = rnd(H) @ rnd(W).T + b
        cache.append((H, Z))
        H = Z if li == len(layers) - 1 else _silu(Z)
        if bf16:
            # the library keeps activations in FP32
            H = H.astype(np.float32).astype(np.float64)
    return H, cache


def loss_and_grad(params, shapes, X, T, bf16: bool = True):
    """Mean squared error over all B*n_out outputs and its flat gradient."""
    rnd = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Y, cache = forward(params, shapes, X, bf16)
    T = np.asarray(T, dtype=np.float64)
    n = Y.size
    loss = float(np.sum((Y - T) ** 2) / n)
    dZ = 2.0 * (Y - T) / n
    layers = unflatten(params, shapes)
    grads = [None] * len(layers)
    for li in range(len(layers) - 1, -1, -1):
        W, _ = layers[li]
        Hin, _ = cache[li]
        if bf16:
            dZ = dZ.astype(np.float32).astype(np.float64)
        gW = rnd(dZ).T @ rnd(Hin)
        gb = dZ.sum(axis=0)
        grads[li] = (gW, gb)
        if li > 0:
            _, Zp = cache[li - 1]
            dZ = (rnd(dZ) @ rnd(W)) * _dsilu(Zp)
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def finite_difference(params, shapes, X, T, idx, h: float = 1e-6):
    """Central differences of the exact (FP64) loss at parameter indices idx."""
    p = np.asarray(params, dtype=np.float64).copy()
    out = np.zeros(len(idx))
    for k, i in enumerate(idx):
        old = p[i]
        p[i] = old + h
        lp, _ = loss_and_grad(p, shapes, X, T, bf16=False)
        p[i] = old - h
        lm, _ = loss_and_grad(p, shapes, X, T, bf16=False)
        p[i] = old
        out[k] = (lp - lm) / (2.0 * h)
    return out


def standardise(X, Y):
    """The statistics portal_mlp_train takes: mean and population standard
    deviation per column (floored at 1e-6), as float32."""
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    mx, my = X.mean(0), Y.mean(0)
    sx = np.sqrt(np.maximum((X * X).mean(0) - mx * mx, 1e-12))
    sy = np.sqrt(np.maximum((Y * Y).mean(0) - my * my, 1e-12))
    return np.concatenate([mx, sx, my, sy]).astype(np.float32)


def predict(params, stats, shapes, X, bf16: bool = True):
    """Raw-unit predictions with the model's standardisation statistics."""
    n_in, n_out = shapes[0][1], shapes[-1][0]
    st = np.asarray(stats, dtype=np.float32)
    mx, sx = st[:n_in], st[n_in:2 * n_in]
    my, sy = st[2 * n_in:2 * n_in + n_out], st[2 * n_in + n_out:]
    Xs = ((np.asarray(X, dtype=np.float32) - mx) / sx).astype(np.float64)
    Y, _ = forward(params, shapes, Xs, bf16)
    return Y * sy.astype(np.float64) + my.astype(np.float64)
