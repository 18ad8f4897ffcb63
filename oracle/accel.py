"""Numpy restatement of the Lambda iteration's Ng acceleration (test
infrastructure only; no counterpart in the reference, which makes a single
pass).

Ng (1974, J. Chem. Phys. 61, 2680), order 2, in the form of Olson, Auer &
Buchler (1986, JQSRT 35, 431): from four successive iterates x0..x3 of a
fixed-point map, with d0 = x3 - x2, d1 = x2 - x1, d2 = x1 - x0 and weights
w = 1/x3^2, (a, b) minimise sum w (d0 - a (d0 - d1) - b (d0 - d2))^2 and
the extrapolation is (1 - a - b) x3 + a x2 + b x1.
"""
from __future__ import annotations

import numpy as np


def ng_coefficients(x0, x1, x2, x3, mask=None):
    """(a, b) of the weighted least-squares problem; x* arrays (nodes, levels).
    mask selects the entries that take part (default: all non-zero x3)."""
    x0, x1, x2, x3 = (np.asarray(v, dtype=np.float64) for v in (x0, x1, x2, x3))
    if mask is None:
        mask = x3 != 0
    w = np.where(mask, 1.0 / np.where(mask, x3, 1.0) ** 2, 0.0)
    d0, d1, d2 = x3 - x2, x2 - x1, x1 - x0
    p, q = d0 - d1, d0 - d2
    A11, A12, A22 = (w * p * p).sum(), (w * p * q).sum(), (w * q * q).sum()
    C1, C2 = (w * d0 * p).sum(), (w * d0 * q).sum()
    det = A11 * A22 - A12 * A12
    return (C1 * A22 - A12 * C2) / det, (A11 * C2 - A12 * C1) / det


def ng_extrapolate(x0, x1, x2, x3, mask=None):
    a, b = ng_coefficients(x0, x1, x2, x3, mask)
    return (1.0 - a - b) * np.asarray(x3) + a * np.asarray(x2) + b * np.asarray(x1), (a, b)


def population_mask(x3, floor=1e-12):
    """The entries the library's Ng step weighs: per node, levels at or above
    floor times the node's largest rho^0_0."""
    x3 = np.asarray(x3, dtype=np.float64)
    big = np.abs(x3).max(axis=1, keepdims=True)
    return (np.abs(x3) >= floor * big) & (x3 != 0)


def ng_populations(x0, x1, x2, x3, sqrt_g):
    """The library's Ng step on rho^0_0 (nodes, levels): extrapolate, keep x3
    where the result is not positive, renormalise sum sqrt(2J+1) rho = 1."""
    x, (a, b) = ng_extrapolate(x0, x1, x2, x3, population_mask(x3))
    x = np.where(x > 0, x, x3)
    x = x / (x * np.asarray(sqrt_g)[None, :]).sum(axis=1, keepdims=True)
    return x, (a, b)
