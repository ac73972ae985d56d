"""Collapsed Gauss-Jacobi quadrature on the reference simplices (oracle).

Restates the rule the reference asks basix for:
`basix.make_quadrature(cell_type, order, QuadratureType.gauss_jacobi)` with
`order = 2 * max(k) + 1` (src/spaces/product_space.py:23-50, order at :31).

The published construction (Karniadakis & Sherwin collapsed coordinates):
m = (order + 2) // 2 points per direction, Gauss-Jacobi points with weight
(1 - x)^a on [-1, 1], a = 0, 1, 2 for the successive collapsed directions.
Reference cells are basix's: interval [0, 1], triangle (0,0),(1,0),(0,1),
tetrahedron (0,0,0),(1,0,0),(0,1,0),(0,0,1).
"""
import numpy as np
from scipy.special import roots_jacobi


def _gj(a, m):
    x, w = roots_jacobi(m, a, 0.0)
    return np.asarray(x, dtype=np.float64), np.asarray(w, dtype=np.float64)


def points_per_direction(order):
    return (int(order) + 2) // 2


def make_quadrature(dim, order):
    """Return (points [Q, dim], weights [Q]) for the reference cell of `dim`.

    dim 0 gives ([1], [1]) as in product_space.py:36-37.
    """
    if dim == 0:
        return np.array([1.0]), np.array([1.0])
    m = points_per_direction(order)
    if dim == 1:
        x, w = _gj(0.0, m)
        return (0.5 + 0.5 * x).reshape(-1, 1), 0.5 * w
    if dim == 2:
        px, wx = _gj(0.0, m)
        py, wy = _gj(1.0, m)
        pts, wts = [], []
        for i in range(m):
            for j in range(m):
                pts.append([0.25 * (1.0 + px[i]) * (1.0 - py[j]), 0.5 * (1.0 + py[j])])
                wts.append(wx[i] * wy[j] * 0.125)
        return np.array(pts), np.array(wts)
    if dim == 3:
        px, wx = _gj(0.0, m)
        py, wy = _gj(1.0, m)
        pz, wz = _gj(2.0, m)
        pts, wts = [], []
        for i in range(m):
            for j in range(m):
                for k in range(m):
                    pts.append([
                        0.125 * (1.0 + px[i]) * (1.0 - py[j]) * (1.0 - pz[k]),
                        0.25 * (1.0 + py[j]) * (1.0 - pz[k]),
                        0.5 * (1.0 + pz[k]),
                    ])
                    wts.append(wx[i] * wy[j] * wz[k] * 0.125 * 0.125)
        return np.array(pts), np.array(wts)
    raise ValueError(f"no quadrature for dim {dim}")
