"""Direct solve and L2 error norms (oracle).

  * solve_newton_step: the linear problems are one Newton step from alpha = 0,
    b = -r(0), x = A^-1 b (examples/cauchy_elasticity/cg_elasticity_example_1.py:161-171);
    scipy SuperLU stands in for MUMPS.
  * l2_error_darcy: sqrt(sum detJ w |u - u_h|^2) per field
    (src/postprocess/l2_error_post_processor.py:7-63; Lagrange branch :35-40,
    vector branch :41-59).
"""
import numpy as np
import scipy.sparse.linalg as spla

from . import elements as el
from .geometry import cell_jacobians


def solve_newton_step(A, r):
    return spla.spsolve(A.tocsc(), -r)


def relative_residual(A, x, b):
    return float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))


def l2_error_darcy(X, signs, dim, quad, cell_dofs, alpha, u_exact, p_exact):
    """[||u - u_h||, ||p - p_h||] for RT1 x P0 on affine cells."""
    pts, wts = quad
    J, det, _ = cell_jacobians(X)
    p1 = el.create_element("P", dim, 1).tabulate(0, pts)[0, :, :, 0]  # [Q, d+1]
    xq = np.einsum("qv,tvg->tqg", p1, X)
    ref = el.create_element("RT", dim, 1).tabulate(0, pts)[0]  # [Q, n_u, d]
    psi = np.einsum("tgd,qid->tqig", J, ref) / det[:, None, None, None]
    psi = psi * np.asarray(signs)[:, None, :, None]
    n_u = dim + 1
    a = np.asarray(alpha)[cell_dofs]
    uh = np.einsum("tqig,ti->tqg", psi, a[:, :n_u])[..., :dim]
    ph = a[:, n_u][:, None] * np.ones(len(wts))[None, :]
    T = X.shape[0]
    ue = np.zeros((T, len(wts), dim))
    pe = np.zeros((T, len(wts)))
    for q in range(len(wts)):
        uv = np.asarray(u_exact(xq[:, q, 0], xq[:, q, 1], xq[:, q, 2]))
        ue[:, q, :] = np.stack([uv[k] for k in range(dim)], axis=1)
        pe[:, q] = np.ravel(p_exact(xq[:, q, 0], xq[:, q, 1], xq[:, q, 2]))
    wdet = det[:, None] * wts[None, :]
    eu = np.sqrt(np.sum(wdet * np.sum((ue - uh) ** 2, axis=2)))
    ep = np.sqrt(np.sum(wdet * (pe - ph) ** 2))
    return [eu, ep]
