"""Weak-form element matrices (oracle restatement, FP64).

Each form returns (r_el, j_el) like WeakForm.evaluate_form
(src/weak_forms/weak_from.py:6-29): the residual at the local coefficients
alpha and its (constant) Jacobian, local order = fields in ProductSpace order,
basis-major / component-minor inside a field.

  * darcy_element      LaplaceDualWeakForm        laplace_dual_weak_form.py:10-86
  * elasticity_element LEPrimalWeakForm           le_primal_weak_form.py:10-129
  * projector_element  L2ProjectorWeakForm        l2_projector_weak_form.py:8-93

The *_batch functions compute the same matrices for many cells at once with
numpy (the vectorised CPU baseline); they are checked against the per-cell
loops in tests/.
"""
import numpy as np

from . import elements as el
from .geometry import cell_jacobians, evaluate_mapping


def tabulate_oriented(family, dim, degree, points, J, det, pinv, signs=None,
                      discontinuous=False):
    """FiniteElement.evaluate_basis (finite_element.py:156-186) for one cell:
    tabulate, push forward the values only, pad 2-D vector fields to three
    components, then apply the RT1 orientation signs to every slice
    (permute_and_transform.py:22-35, :110-140)."""
    e = el.create_element(family, dim, degree, discontinuous)
    tab = e.tabulate(1, points)
    mapped = e.push_forward(tab[0], J, det, pinv)
    if mapped.shape != tab[0].shape:
        tab = np.insert(tab, 2, 0.0, axis=3)
    tab[0] = mapped
    if signs is not None and family == "RT":
        tab = tab * np.asarray(signs)[None, None, :, None]
    return tab


def _as_callable(v):
    if callable(v):
        return v
    return lambda x, y, z: np.full((1, np.size(x)), float(v))


def darcy_element(X, signs, dim, quad, kappa, rhs, alpha=None):
    """Mixed Darcy RT1 x P0 element (laplace_dual_weak_form.py:10-86)."""
    pts, wts = quad
    x, J, det, pinv = evaluate_mapping(dim, pts, X)
    u_tab = tabulate_oriented("RT", dim, 1, pts, J, det, pinv, signs)
    p_tab = tabulate_oriented("P", dim, 0, pts, J, det, pinv, discontinuous=True)
    n_u = u_tab.shape[2]
    n_p = p_tab.shape[2]
    n = n_u + n_p
    kappa = _as_callable(kappa)
    rhs = _as_callable(rhs)
    j = np.zeros((n, n))
    r = np.zeros(n)
    f_val = np.atleast_2d(rhs(x[:, 0], x[:, 1], x[:, 2]))
    phi_s = det * wts * p_tab[0, :, :, 0].T
    r[n_u:] -= phi_s @ f_val[0]
    for q, w in enumerate(wts):
        psi = u_tab[0, q, :, 0:dim]
        wh = p_tab[0, q, :, 0]
        grad = u_tab[1:, q, :, 0:dim]
        div = np.trace(grad, axis1=0, axis2=2) / det[q]
        k = float(np.ravel(kappa(x[q, 0], x[q, 1], x[q, 2]))[0])
        j[:n_u, :n_u] += det[q] * w * (psi @ psi.T) / k
        j[:n_u, n_u:] -= det[q] * w * np.outer(div, wh)
        j[n_u:, :n_u] += det[q] * w * np.outer(wh, div)
    if alpha is not None:
        r = r + j @ np.asarray(alpha)
    return r, j


def darcy_batch(X, signs, dim, quad, kappa_q, f_q):
    """All cells at once.  X [T, d+1, 3]; signs [T, d+1]; kappa_q, f_q [T, Q]
    (coefficients sampled at the quadrature points).  Returns r [T, n], j [T, n, n]
    at alpha = 0."""
    pts, wts = quad
    T = X.shape[0]
    J, det, pinv = cell_jacobians(X)
    rt = el.create_element("RT", dim, 1)
    ref = rt.tabulate(1, pts)  # [1+d, Q, n_u, d]
    n_u = dim + 1
    psi_hat = ref[0]  # [Q, n_u, d]
    divhat = np.einsum("kqik->qi", ref[1:])  # [Q, n_u]
    s = np.asarray(signs, dtype=np.float64)
    psi = np.einsum("tgd,qid->tqig", J, psi_hat) / det[:, None, None, None]
    psi = psi * s[:, None, :, None]
    wdet = det[:, None] * wts[None, :]  # [T, Q]
    n = n_u + 1
    j = np.zeros((T, n, n))
    j[:, :n_u, :n_u] = np.einsum("tq,tqig,tqjg->tij", wdet / kappa_q, psi, psi)
    div = divhat[None, :, :] * s[:, None, :] / det[:, None, None]  # [T, Q, n_u]
    b = np.einsum("tq,tqi->ti", wdet, div)
    j[:, :n_u, n_u] = -b
    j[:, n_u, :n_u] = b
    r = np.zeros((T, n))
    r[:, n_u] = -np.einsum("tq,tq->t", wdet, f_q)
    return r, j


def elasticity_element(X, dim, quad, lam, mu, rhs, alpha=None):
    """Vector P2 linear elasticity (le_primal_weak_form.py:10-129)."""
    pts, wts = quad
    x, J, det, pinv = evaluate_mapping(dim, pts, X)
    tab = tabulate_oriented("P", dim, 2, pts, J, det, pinv)
    n_phi = tab.shape[2]
    nc = dim
    n = n_phi * nc
    lam = _as_callable(lam)
    mu = _as_callable(mu)
    f = np.atleast_2d(rhs(x[:, 0], x[:, 1], x[:, 2]))
    lam_q = np.ravel(lam(x[:, 0], x[:, 1], x[:, 2])) * np.ones(len(wts))
    mu_q = np.ravel(mu(x[:, 0], x[:, 1], x[:, 2])) * np.ones(len(wts))
    r = np.zeros(n)
    for c in range(nc):
        r[c::nc] += (det * wts * tab[0, :, :, 0].T) @ f[c]
    j = np.zeros((n, n))
    for q, w in enumerate(wts):
        G = (pinv[q].T[:dim, :dim] @ tab[1:dim + 1, q, :, 0]).T if dim == 3 else \
            (np.vstack([pinv[q][:, 0], pinv[q][:, 1]]) @ tab[1:dim + 1, q, :, 0]).T
        # G [n_phi, dim]: physical gradients
        gg = G @ G.T
        blk = np.zeros((n_phi, nc, n_phi, nc))
        for c in range(nc):
            blk[:, c, :, c] += mu_q[q] * gg
        blk += mu_q[q] * np.einsum("ae,bc->acbe", G, G)
        blk += lam_q[q] * np.einsum("ac,be->acbe", G, G)
        j += det[q] * w * blk.reshape(n, n)
    if alpha is not None:
        r = r + j @ np.asarray(alpha)
    return r, j


def elasticity_batch(X, dim, quad, lam_c, mu_c, f_q):
    """All cells, per-cell lambda/mu [T], body force at quadrature points f_q [T, Q, dim]."""
    pts, wts = quad
    J, det, pinv = cell_jacobians(X)
    p2 = el.create_element("P", dim, 2)
    ref = p2.tabulate(1, pts)  # [1+d, Q, n_phi, 1]
    dref = ref[1:dim + 1, :, :, 0]  # [d, Q, n_phi]
    # physical gradient: grad_i phi = sum_k pinv[k, i] d_k phi
    G = np.einsum("tki,kqa->tqai", pinv[:, :, :dim], dref)  # [T, Q, n_phi, d]
    wdet = det[:, None] * wts[None, :]
    gg = np.einsum("tq,tqai,tqbi->tab", wdet, G, G)
    outer = np.einsum("tq,tqai,tqbj->taibj", wdet, G, G)  # [T, a, i, b, j]
    T = X.shape[0]
    n_phi = dref.shape[2]
    nc = dim
    blk = np.zeros((T, n_phi, nc, n_phi, nc))
    for c in range(nc):
        blk[:, :, c, :, c] += mu_c[:, None, None] * gg
    blk += mu_c[:, None, None, None, None] * np.transpose(outer, (0, 1, 4, 3, 2))
    blk += lam_c[:, None, None, None, None] * outer
    j = blk.reshape(T, n_phi * nc, n_phi * nc)
    phi = ref[0, :, :, 0]  # [Q, n_phi]
    r = np.einsum("tq,qa,tqc->tac", wdet, phi, f_q).reshape(T, n_phi * nc)
    return r, j


def projector_element(fields, X, dim, quad, functions, signs=None):
    """L2 projection mass matrix and load (l2_projector_weak_form.py:8-93).

    fields: list of (name, family, degree, n_comp, discontinuous)."""
    pts, wts = quad
    x, J, det, pinv = evaluate_mapping(dim, pts, X)
    r_els, j_els = [], []
    for name, family, degree, nc, disc in fields:
        tab = tabulate_oriented(family, dim, degree, pts, J, det, pinv,
                                signs if family == "RT" else None, disc)
        n_phi = tab.shape[2]
        n = n_phi * nc
        r = np.zeros(n)
        j = np.zeros((n, n))
        fv = np.asarray(functions[name](x[:, 0], x[:, 1], x[:, 2]))
        for c in range(nc):
            if family == "P":
                r[c::nc] -= (det * wts * tab[0, :, :, 0].T) @ fv[c]
            else:
                for q in range(len(wts)):
                    r[c::nc] -= det[q] * wts[q] * tab[0, q, :, 0:dim] @ fv[c, 0:dim, q]
            for q, w in enumerate(wts):
                if family == "P":
                    ph = tab[0, q, :, 0]
                    j[c::nc, c::nc] += det[q] * w * np.outer(ph, ph)
                else:
                    for d in range(dim):
                        ph = tab[0, q, :, d]
                        j[c::nc, c::nc] += det[q] * w * np.outer(ph, ph)
        r_els.append(r)
        j_els.append(j)
    n = sum(len(r) for r in r_els)
    r = np.zeros(n)
    j = np.zeros((n, n))
    o = 0
    for rr, jj in zip(r_els, j_els):
        m = len(rr)
        r[o:o + m] += rr
        j[o:o + m, o:o + m] += jj
        o += m
    return r, j
