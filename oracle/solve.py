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


def field_error(family, dim, quad, X, signs, dest, n_comp, degree, alpha, exact, quantity="value",
                scale=None, grad_scale=None):
    """One field's error norm, restating the reference's per-cell loops:
      value, Lagrange   l2_error Lagrange branch (l2_error_post_processor.py:35-40),
                        components 0..dim-1, exact vectorised over the points;
      value, RT         vector branch (:41-59), exact called point by point,
                        [n_comp, 3] per point, its first dim columns compared;
      "div"             div_error (:185-238): trace of the oriented reference
                        gradients / det J, exact per point [n_comp];
      "div_scaled"      div_scaled_error (:240-306): grad l . psi + l div psi.
    X [T, d+1, 3], signs [T, d+1] (RT), dest [T, n_phi * n_comp] the field's
    DoFs of each cell, alpha the global solution (None: the exact norm, as in
    solution_norms_post_processor.py:7-78)."""
    from .forms import tabulate_oriented
    from .geometry import evaluate_mapping
    pts, wts = quad
    total = 0.0
    fam = "P" if family == "Lagrange" else family
    for c in range(X.shape[0]):
        x, J, det, pinv = evaluate_mapping(dim, pts, X[c])
        tab = tabulate_oriented(fam, dim, degree, pts, J, det, pinv, signs[c] if fam == "RT" else None,
                                discontinuous=(fam == "P" and degree == 0))
        n_phi = tab.shape[2]
        a = np.zeros(len(dest[c])) if alpha is None else np.asarray(alpha)[dest[c]]
        a_star = np.array(np.split(a, n_phi))  # [n_phi, n_comp]
        if quantity == "value" and fam == "P":
            fe = np.asarray(exact(x[:, 0], x[:, 1], x[:, 2]), dtype=np.float64).reshape(-1, len(wts))[0:dim, :]
            fh = (tab[0, :, :, 0] @ a_star[:, 0:dim]).T
            total += np.sum(det * wts * (fe - fh) * (fe - fh))
        elif quantity == "value":
            fe = np.array([np.asarray(exact(xv[0], xv[1], xv[2]), dtype=np.float64).reshape(n_comp, -1)
                           for xv in x])[:, :, 0:dim]
            fh = np.array([np.vstack([tab[0, k, :, 0:dim].T @ a_star[:, cc] for cc in range(n_comp)])
                           for k in range(len(pts))])
            d = fe - fh
            total += np.sum(det * wts * np.array([np.trace(e.T @ e) for e in d]))
        else:
            grad = tab[1:dim + 1, :, :, 0:dim]
            div = np.trace(grad, axis1=0, axis2=3).T * (1.0 / det)  # [n_phi, Q]
            if quantity == "div_scaled":
                gam = np.ravel(scale(x[:, 0], x[:, 1], x[:, 2])) * np.ones(len(wts))
                ggam = np.asarray(grad_scale(x[:, 0], x[:, 1], x[:, 2]), dtype=np.float64).reshape(-1, len(wts))
                div = np.array([[np.trace(np.outer(ggam[:dim, i], tab[0, i, j, 0:dim])) for i in range(len(pts))]
                                for j in range(n_phi)]) + div * gam[None, :]
            fe = np.array([np.asarray(exact(xv[0], xv[1], xv[2]), dtype=np.float64).reshape(n_comp) for xv in x])
            fh = div.T @ a_star
            total += np.sum(((fe - fh) * (fe - fh)).T @ (det * wts))
    return float(np.sqrt(total))
