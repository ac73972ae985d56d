"""Affine geometric map of a simplex (oracle restatement of src/geometry/mapping.py).

  * x_q = sum_v phi_v(q) X_v and J_q[:, k] = d x / d xhat_k from P1 shapes
    (mapping.py:9-20, :39-48); J is [gdim=3, tdim].
  * det and pseudo-inverse through a QR of J with the rows of R sign-normalised
    so diag(R) > 0: det = det(R) > 0 and J+ = R^-1 Q^T (mapping.py:23-36).
"""
import numpy as np

from . import elements as el


def det_and_pinv(J):
    """J [3, d] -> (|det|, J+ [d, 3]) as mapping.py:23-36 computes them."""
    q, r = np.linalg.qr(J)
    s = np.diag(np.sign(np.diag(r)))
    q = q @ s
    r = s @ r
    return np.linalg.det(r), np.linalg.inv(r) @ q.T


def evaluate_mapping(dim, points, X):
    """points [Q, dim] on the reference cell, X [dim+1, 3] vertex coordinates."""
    p1 = el.create_element("P", dim, 1)
    phi = p1.tabulate(1, points)
    x = phi[0, :, :, 0] @ X
    jac = np.transpose(np.moveaxis(phi[1:dim + 1, :, :, 0], 1, 0) @ X, (0, 2, 1))
    dets, invs = zip(*[det_and_pinv(j) for j in jac])
    return x, jac, np.array(dets), np.array(invs)


def cell_jacobians(X):
    """Vectorised affine Jacobians: X [T, d+1, 3] -> J [T, 3, d], |det| [T], J+ [T, d, 3].

    Same quantities as evaluate_mapping (constant over the cell for affine
    simplices), formed as stably as the QR forms above: for tetrahedra
    |det| = |det J| (LU) and J+ = J^-1; for triangles in R^3 |det| =
    |J[:, 0] x J[:, 1]| and J+ = (J^T J)^-1 J^T.  (|det| = sqrt(det(J^T J))
    would lose a relative eps / q^2 on cells of shape quality q, the QR form
    and these eps / q.)
    """
    J = np.transpose(X[:, 1:, :] - X[:, :1, :], (0, 2, 1))
    if J.shape[2] == 3:
        det = np.abs(np.linalg.det(J))
        pinv = np.linalg.inv(J)
    else:
        G = np.einsum("tgi,tgj->tij", J, J)
        det = np.linalg.norm(np.cross(J[:, :, 0], J[:, :, 1]), axis=1) if J.shape[2] == 2 else np.sqrt(
            np.linalg.det(G))
        pinv = np.linalg.solve(G, np.transpose(J, (0, 2, 1)))
    return J, det, pinv
