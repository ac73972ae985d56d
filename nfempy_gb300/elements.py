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


# P2 Lagrange on the reference simplex (gll_centroid = vertices and edge
# midpoints for degree 2), basix local order: vertices, then edges in basix's
# sub-entity order (src/mesh/mesh.py:187-193 for tetrahedra).
P2_EDGES = {2: ((1, 2), (0, 2), (0, 1)), 3: ((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))}


def lagrange_p2(dim, pts):
    """(values [Q, n], reference gradients [Q, n, dim]) of P2 at points [Q, dim]."""
    lam = lagrange_p1_values(dim, pts)
    dlam = np.zeros((dim, dim + 1))
    dlam[:, 0] = -1.0
    dlam[:, 1:] = np.eye(dim)
    edges = P2_EDGES[dim]
    n = dim + 1 + len(edges)
    Q = lam.shape[0]
    val = np.zeros((Q, n))
    grad = np.zeros((Q, n, dim))
    for v in range(dim + 1):
        val[:, v] = lam[:, v] * (2.0 * lam[:, v] - 1.0)
        grad[:, v, :] = (4.0 * lam[:, v] - 1.0)[:, None] * dlam[:, v][None, :]
    for e, (a, b) in enumerate(edges):
        val[:, dim + 1 + e] = 4.0 * lam[:, a] * lam[:, b]
        grad[:, dim + 1 + e, :] = 4.0 * (lam[:, b][:, None] * dlam[:, a][None, :] + lam[:, a][:, None] * dlam[:, b][None, :])
    return val, grad


def p2_reference_tables(dim):
    """Exact reference integrals of P2 (order-5 rule is exact for them):
    S[a, b, k, l] = int d_k phi_a d_l phi_b, m[a] = int phi_a,
    Mf[a, b] = int phi_a phi_b on the (dim-1) facet simplex (P2 there)."""
    from .quadrature import make_quadrature
    pts, w = make_quadrature(dim, 5)
    val, grad = lagrange_p2(dim, pts)
    S = np.einsum("q,qak,qbl->abkl", w, grad, grad)
    m = np.einsum("q,qa->a", w, val)
    fpts, fw = make_quadrature(dim - 1, 5)
    fval, _ = lagrange_p2(dim - 1, fpts)
    Mf = np.einsum("q,qa,qb->ab", fw, fval, fval)
    return S, m, Mf


# RT1 on the reference tetrahedron: psi_i = sigma_i * 2 * (x - v_i), with
# sigma_i = +1 when basix's facet normal (v1 - v0) x (v2 - v0) of face i
# points out of the cell, -1 otherwise (faces opposite v0..v3).
RT1_SIGMA_TET = np.array([1.0, -1.0, 1.0, -1.0])
TET_VERTS = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def rt1_tet_tables():
    """Exact reference integrals of RT1 on the tetrahedron (order-3 rule):
    Psi[i, j] = int psihat_i psihat_j^T (3 x 3), mhat[i] = int psihat_i,
    divhat[i] = int div psihat_i."""
    from .quadrature import make_quadrature
    pts, w = make_quadrature(3, 3)
    psi = 2.0 * RT1_SIGMA_TET[None, :, None] * (pts[:, None, :] - TET_VERTS[None, :, :])  # [Q, 4, 3]
    Psi = np.einsum("q,qik,qjl->ijkl", w, psi, psi)
    mhat = np.einsum("q,qik->ik", w, psi)
    divhat = RT1_SIGMA_TET * 6.0 * w.sum()
    return Psi, mhat, divhat
