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


def cell_block_jacobi(A, cell_dofs):
    """The plain preconditioner restated on the host: weighted additive
    Schwarz over the element cliques, z_r = (1/m_r) sum over the cells c that
    hold r of (A_cc^-1 v_c)_r, A_cc the cell's dense block of A, m_r the
    number of such cells.  Returns z = M(v) as a function."""
    A = A.tocsr()
    cd = np.asarray(cell_dofs, dtype=np.int64)
    T, n = cd.shape
    rows = np.repeat(cd, n, axis=1).ravel()
    cols = np.tile(cd, (1, n)).ravel()
    blocks = np.asarray(A[rows, cols]).reshape(T, n, n)
    inv = np.linalg.inv(blocks)
    mult = np.bincount(cd.ravel(), minlength=A.shape[0]).astype(np.float64)
    mult[mult == 0] = 1.0

    def apply(v):
        y = np.einsum("tij,tj->ti", inv, np.asarray(v).ravel()[cd])
        return np.bincount(cd.ravel(), weights=y.ravel(), minlength=A.shape[0]) / mult

    return apply


def gmres_block_jacobi(A, b, cell_dofs, rtol=1e-8, restart=50, maxiter=20000):
    """Host GMRES(restart) (scipy) with the cell-block Jacobi preconditioner:
    the plain method on the CPU.  Restarts until the true relative residual
    ||b - A x|| / ||b|| <= rtol or maxiter iterations.  Returns
    (x, iterations, relres)."""
    A = A.tocsr()
    op = spla.LinearOperator(A.shape, matvec=cell_block_jacobi(A, cell_dofs))
    x = np.zeros_like(b)
    its = [0]

    def cb(_):
        its[0] += 1

    nb = np.linalg.norm(b)
    rel = 1.0
    while its[0] < maxiter:
        before = its[0]
        x, info = spla.gmres(A, b, x0=x, M=op, rtol=rtol * 0.1, atol=0.0, restart=restart,
                             maxiter=max(1, (maxiter - its[0]) // restart), callback=cb, callback_type="pr_norm")
        rel = float(np.linalg.norm(b - A @ x) / nb)
        if rel <= rtol or its[0] == before:
            break
    return x, its[0], rel
