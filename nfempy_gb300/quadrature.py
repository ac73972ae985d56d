"""Collapsed Gauss-Jacobi quadrature on reference simplices.

The rule the reference requests from basix
(`make_quadrature(cell, 2 * max(k) + 1, gauss_jacobi)`,
src/spaces/product_space.py:23-50): m = (order + 2) // 2 Gauss-Jacobi points
per collapsed direction with weights (1 - x)^a, a = 0, 1, 2, mapped to
basix's reference cells.  Gauss-Jacobi nodes come from the Golub-Welsch
eigenvalue method on the Jacobi three-term recurrence.
"""
import math

import numpy as np


def gauss_jacobi(m, a):
    """m-point Gauss rule for weight (1 - x)^a on [-1, 1] (beta = 0)."""
    b = 0.0
    n = np.arange(m, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        diag = (b * b - a * a) / ((2 * n + a + b) * (2 * n + a + b + 2))
    if a + b == 0.0:
        diag[0] = (b - a) / (a + b + 2)
    k = np.arange(1, m, dtype=np.float64)
    off = np.sqrt(4 * k * (k + a) * (k + b) * (k + a + b)
                  / ((2 * k + a + b) ** 2 * (2 * k + a + b + 1) * (2 * k + a + b - 1)))
    Jm = np.diag(diag) + np.diag(off, 1) + np.diag(off, -1)
    x, V = np.linalg.eigh(Jm)
    mu0 = 2.0 ** (a + b + 1) * math.gamma(a + 1) * math.gamma(b + 1) / math.gamma(a + b + 2)
    w = mu0 * V[0, :] ** 2
    return x, w


def make_quadrature(dim, order):
    if dim == 0:
        return np.array([1.0]), np.array([1.0])
    m = (int(order) + 2) // 2
    if dim == 1:
        x, w = gauss_jacobi(m, 0.0)
        return (0.5 + 0.5 * x).reshape(-1, 1), 0.5 * w
    px, wx = gauss_jacobi(m, 0.0)
    py, wy = gauss_jacobi(m, 1.0)
    if dim == 2:
        X = 0.25 * (1 + px[:, None]) * (1 - py[None, :])
        Y = 0.5 * (1 + py[None, :]) * np.ones_like(X)
        W = wx[:, None] * wy[None, :] * 0.125
        return np.stack([X.ravel(), Y.ravel()], axis=1), W.ravel()
    pz, wz = gauss_jacobi(m, 2.0)
    I = (1 + px)[:, None, None]
    Jy = py[None, :, None]
    Kz = pz[None, None, :]
    X = 0.125 * I * (1 - Jy) * (1 - Kz)
    Y = 0.25 * (1 + Jy) * (1 - Kz) * np.ones_like(X)
    Z = 0.5 * (1 + Kz) * np.ones_like(X)
    W = wx[:, None, None] * wy[None, :, None] * wz[None, None, :] * 0.125 * 0.125
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1), W.ravel()
