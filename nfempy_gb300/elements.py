"""Small reference-element tables the host side needs.

Only the P1 Lagrange values (barycentric coordinates) used to place
quadrature points on physical cells (src/geometry/mapping.py:39-48); the
element integrals themselves are evaluated on the device.
"""
import numpy as np


def lagrange_p1_values(dim, pts):
    """[Q, dim + 1] barycentric coordinates of reference points (basix P1 order)."""
    pts = np.atleast_2d(np.asarray(pts, dtype=np.float64))
    lam = np.empty((pts.shape[0], dim + 1))
    lam[:, 0] = 1.0 - pts.sum(axis=1)
    lam[:, 1:] = pts
    return lam
