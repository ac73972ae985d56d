"""Weak-form element matrices (oracle restatement, FP64).

Each form returns (r_el, j_el) like WeakForm.evaluate_form
(src/weak_forms/weak_from.py:6-29): the residual at the local coefficients
alpha and its (constant) Jacobian, local order = fields in ProductSpace order,
basis-major / component-minor inside a field.

  * darcy_element      LaplaceDualWeakForm        laplace_dual_weak_form.py:10-86
  * elasticity_element LEPrimalWeakForm           le_primal_weak_form.py:10-129
  * projector_element  L2ProjectorWeakForm        l2_projector_weak_form.py:8-93
  * cosserat_element   LCEDualWeakForm            lce_dual_weak_form.py:410-648

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


def cosserat_element(X, signs, quad, par, f_u, f_t):
    """Mixed Cosserat element, 3-D (lce_dual_weak_form.py:410-648,
    evaluate_form_vectorized).  Fields s (RT1, 3 rows), m (RT1, 3 rows),
    u (P0^3), t (P0^3); local order s, m, u, t, basis-major / component-minor.
    par: dict lambda_s, mu_s, kappa_s, lambda_o, mu_o, kappa_o, l (constants
    on the cell).  f_u, f_t: body force and couple (3-vectors, constant), or
    f_u a callable f(x, y, z) -> [6, Q] (f_u then f_t, evaluated at the
    physical quadrature points like the reference's f_rhs, :472, :490-502)
    and f_t None."""
    dim = 3
    pts, wts = quad
    x, J, det, pinv = evaluate_mapping(dim, pts, X)
    s_tab = tabulate_oriented("RT", dim, 1, pts, J, det, pinv, signs)
    p_tab = tabulate_oriented("P", dim, 0, pts, J, det, pinv, discontinuous=True)
    ns, nm, nu, nt = 12, 12, 3, 3
    n = ns + nm + nu + nt
    j = np.zeros((n, n))
    r = np.zeros(n)
    Q = len(wts)
    wdet = det * wts
    w0 = p_tab[0, :, 0, 0]  # P0 value (1)
    # rhs_u, rhs_t
    if callable(f_u):
        fq = np.asarray(f_u(x[:, 0], x[:, 1], x[:, 2]), dtype=np.float64).reshape(6, Q)
        for c in range(3):
            r[ns + nm + c] += -np.sum(wdet * w0 * fq[c])
            r[ns + nm + nu + c] += -np.sum(wdet * w0 * fq[3 + c])
    else:
        for c in range(3):
            r[ns + nm + c] += -np.sum(wdet * w0) * f_u[c]
            r[ns + nm + nu + c] += -np.sum(wdet * w0) * f_t[c]

    def block(psi, mu_v, kappa_v, lam_v, scale):
        # psi [Q, 4, 3]
        out = np.zeros((12, 12))
        vol = (1.0 / (2.0 * mu_v)) * (lam_v / (2.0 * mu_v + dim * lam_v))
        for q in range(Q):
            P = psi[q]
            inner = np.zeros((12, 12))
            outer = np.zeros((12, 12))
            tro = np.outer(P.ravel(), P.ravel())
            for i in range(4):
                for jj in range(4):
                    inner[i * 3:(i + 1) * 3, jj * 3:(jj + 1) * 3] = 0.5 * np.dot(P[i], P[jj]) * np.eye(3)
                    outer[i * 3:(i + 1) * 3, jj * 3:(jj + 1) * 3] = 0.5 * np.outer(P[jj], P[i])
            symm = inner + outer
            skew = inner - outer
            out += wdet[q] * scale * (symm / (2.0 * mu_v) + skew / (2.0 * kappa_v) - vol * tro)
        return out

    s_psi = s_tab[0, :, :, 0:dim]
    j[0:ns, 0:ns] += block(s_psi, par["mu_s"], par["kappa_s"], par["lambda_s"], 1.0)
    j[ns:ns + nm, ns:ns + nm] += block(s_psi, par["mu_o"], par["kappa_o"], par["lambda_o"], 1.0 / par["l"])
    # (t,s) / (s,t): asymmetry coupling
    A = [np.einsum("q,q,qi->i", wdet, w0, s_psi[:, :, k]) for k in range(3)]  # [3][4]
    tmap = {0: ((2, A[1]), (1, -A[2])), 1: ((0, A[2]), (2, -A[0])), 2: ((1, A[0]), (0, -A[1]))}
    for c in range(3):
        tb = ns + nm + nu + c
        for cs, op in tmap[c]:
            for i in range(4):
                j[tb, i * 3 + cs] += -op[i]
                j[i * 3 + cs, tb] += -op[i]
    # (u,s) and (t,m): divergence coupling, int w div psi
    grad = s_tab[1:dim + 1, :, :, 0:dim]  # [d, Q, 4, d]
    div = np.einsum("kqik->qi", grad)  # reference divergence (det cancels)
    ub = np.einsum("q,q,qi->i", wts, w0, div)
    for c in range(3):
        for i in range(4):
            j[ns + nm + c, i * 3 + c] += ub[i]
            j[i * 3 + c, ns + nm + c] += ub[i]
            j[ns + nm + nu + c, ns + i * 3 + c] += ub[i]
            j[ns + i * 3 + c, ns + nm + nu + c] += ub[i]
    return r, j


def cosserat_batch(X, signs, quad, par, f_q):
    """cosserat_element for many cells at once (numpy, FP64).  X [T, 4, 3],
    signs [T, 4], par the seven constants, f_q [T, Q, 6] the load (f_u, f_t)
    at the quadrature points.  Returns r [T, 30], j [T, 30, 30]; checked
    against the per-cell restatement in tests/."""
    pts, wts = quad
    T = X.shape[0]
    J, det, pinv = cell_jacobians(X)
    ref = el.create_element("RT", 3, 1).tabulate(1, pts)  # [4, Q, 4, 3]
    sg = np.asarray(signs, dtype=np.float64)
    psi = np.einsum("tgd,qid->tqig", J, ref[0]) / det[:, None, None, None] * sg[:, None, :, None]
    wdet = det[:, None] * wts[None, :]
    Phi = np.einsum("tq,tqia,tqjb->tijab", wdet, psi, psi)  # [T, 4, 4, 3, 3]
    eye = np.eye(3)
    tr = np.einsum("tijaa->tij", Phi)
    inner = 0.5 * np.einsum("tij,cd->ticjd", tr, eye)
    outer = 0.5 * np.einsum("tijdc->ticjd", Phi)
    tro = np.einsum("tijcd->ticjd", Phi)

    def block(mu_v, kappa_v, lam_v, scale):
        vol = (1.0 / (2.0 * mu_v)) * (lam_v / (2.0 * mu_v + 3 * lam_v))
        b = scale * ((inner + outer) / (2.0 * mu_v) + (inner - outer) / (2.0 * kappa_v) - vol * tro)
        return b.reshape(T, 12, 12)

    n = 30
    j = np.zeros((T, n, n))
    j[:, 0:12, 0:12] = block(par["mu_s"], par["kappa_s"], par["lambda_s"], 1.0)
    j[:, 12:24, 12:24] = block(par["mu_o"], par["kappa_o"], par["lambda_o"], 1.0 / par["l"])
    v = np.einsum("tq,tqik->tki", wdet, psi)  # [T, 3 (component k), 4]
    tmap = {0: ((2, v[:, 1]), (1, -v[:, 2])), 1: ((0, v[:, 2]), (2, -v[:, 0])), 2: ((1, v[:, 0]), (0, -v[:, 1]))}
    for c in range(3):
        tb = 27 + c
        for cs, op in tmap[c]:
            for i in range(4):
                j[:, tb, i * 3 + cs] += -op[:, i]
                j[:, i * 3 + cs, tb] += -op[:, i]
    divhat = np.einsum("kqik->qi", ref[1:4])  # [Q, 4]
    ub = np.einsum("q,qi->i", wts, divhat)[None, :] * sg  # [T, 4]
    for c in range(3):
        for i in range(4):
            j[:, 24 + c, i * 3 + c] += ub[:, i]
            j[:, i * 3 + c, 24 + c] += ub[:, i]
            j[:, 27 + c, 12 + i * 3 + c] += ub[:, i]
            j[:, 12 + i * 3 + c, 27 + c] += ub[:, i]
    r = np.zeros((T, n))
    r[:, 24:27] = -np.einsum("tq,tqk->tk", wdet, f_q[:, :, 0:3])
    r[:, 27:30] = -np.einsum("tq,tqk->tk", wdet, f_q[:, :, 3:6])
    return r, j


def cosserat_riesz_element(X, signs, quad, par, l_fn, grad_l_fn):
    """LCEScaledRieszMapWeakForm.evaluate_form_vectorized
    (lce_scaled_riesz_map_weak_form.py:415-598), 3-D: block-diagonal by
    field; (s,s) the stress compliance plus sum over the rows of
    (div tau_i, div tau_j); (m,m) the couple-stress compliance (no 1/l) plus
    the rows' (div(l v_i), div(l v_j)) with div(l v) = grad l . v + l div v;
    (u,u) and (t,t) the P0 mass.  l_fn(x, y, z) -> [Q], grad_l_fn -> [3, Q]."""
    dim = 3
    pts, wts = quad
    x, J, det, pinv = evaluate_mapping(dim, pts, X)
    s_tab = tabulate_oriented("RT", dim, 1, pts, J, det, pinv, signs)
    Q = len(wts)
    wdet = det * wts
    n = 30
    j = np.zeros((n, n))

    def compliance(psi, mu_v, kappa_v, lam_v):
        out = np.zeros((12, 12))
        vol = (1.0 / (2.0 * mu_v)) * (lam_v / (2.0 * mu_v + dim * lam_v))
        for q in range(Q):
            P = psi[q]
            inner = np.zeros((12, 12))
            outer = np.zeros((12, 12))
            tro = np.outer(P.ravel(), P.ravel())
            for i in range(4):
                for jj in range(4):
                    inner[i * 3:(i + 1) * 3, jj * 3:(jj + 1) * 3] = 0.5 * np.dot(P[i], P[jj]) * np.eye(3)
                    outer[i * 3:(i + 1) * 3, jj * 3:(jj + 1) * 3] = 0.5 * np.outer(P[jj], P[i])
            out += wdet[q] * ((inner + outer) / (2.0 * mu_v) + (inner - outer) / (2.0 * kappa_v) - vol * tro)
        return out

    psi = s_tab[0, :, :, 0:dim]
    j[0:12, 0:12] += compliance(psi, par["mu_s"], par["kappa_s"], par["lambda_s"])
    j[12:24, 12:24] += compliance(psi, par["mu_o"], par["kappa_o"], par["lambda_o"])
    grad = s_tab[1:dim + 1, :, :, 0:dim]
    div = np.trace(grad, axis1=0, axis2=3).T / det  # [4, Q]
    lv = np.ravel(l_fn(x[:, 0], x[:, 1], x[:, 2])) * np.ones(Q)
    gl = np.asarray(grad_l_fn(x[:, 0], x[:, 1], x[:, 2]), dtype=np.float64).reshape(-1, Q)[:dim]
    sdiv = (div * wdet) @ div.T
    ldiv = np.einsum("dq,qid->iq", gl, psi) + div * lv[None, :]
    mdiv = (ldiv * wdet) @ ldiv.T
    for c in range(3):
        idx = np.arange(4) * 3 + c
        j[np.ix_(idx, idx)] += sdiv
        j[np.ix_(12 + idx, 12 + idx)] += mdiv
    for k in range(24, 30):
        j[k, k] += np.sum(wdet)
    return np.zeros(n), j


LE_OF_COSSERAT = np.r_[0:12, 24:30]  # s, u, t inside the Cosserat layout s, m, u, t


def le_dual_element(X, signs, quad, lam, mu, f_fn):
    """LEDualWeakForm.evaluate_form_vectorized (le_dual_weak_form.py:354-515),
    3-D, fields s (RT1 x 3), u, t (P0 x 3), 18 local DoFs: the mixed Cosserat
    element with kappa = mu (the compliance 1/(2 mu) on the symmetric and the
    skew part alike) restricted to the s, u and t DoFs.  The reference's
    blocks are the same operators: (s, s) 1/(2 mu) psi_i . psi_j minus the
    volumetric term, (t, s) the skew moments of the stress basis, (u, s)
    int div psi_j per component, r = -int f.  lam, mu constants; f_fn(x, y,
    z) -> [6, Q] (f_u then f_t)."""
    par = dict(lambda_s=lam, mu_s=mu, kappa_s=mu, lambda_o=lam, mu_o=mu, kappa_o=mu, l=1.0)
    r, j = cosserat_element(X, signs, quad, par, f_fn, None)
    idx = LE_OF_COSSERAT
    return r[idx], j[np.ix_(idx, idx)]


def le_riesz_element(X, signs, quad, lam_fn, mu_fn):
    """LERieszMapWeakForm.evaluate_form_vectorized
    (le_riesz_map_weak_form.py:245-360), 3-D, fields s (RT1 x 3), u, t
    (P0 x 3), 18 local DoFs, s DoF (i, c) at 3 i + c: per stress row c the
    (1/(2 mu)) psi_i . psi_j mass and the (div psi_i, div psi_j) term; across
    the rows -(1/(2 mu)) lambda / (2 mu + 3 lambda) psi_i[c] psi_j[d]; the P0
    mass on u and t.  lam_fn, mu_fn(x, y, z) -> [Q] at the quadrature
    points."""
    dim = 3
    pts, wts = quad
    x, J, det, pinv = evaluate_mapping(dim, pts, X)
    s_tab = tabulate_oriented("RT", dim, 1, pts, J, det, pinv, signs)
    Q = len(wts)
    wdet = det * wts
    lam = np.ravel(lam_fn(x[:, 0], x[:, 1], x[:, 2])) * np.ones(Q)
    mu = np.ravel(mu_fn(x[:, 0], x[:, 1], x[:, 2])) * np.ones(Q)
    psi = s_tab[0, :, :, 0:dim]  # [Q, 4, 3]
    j = np.zeros((18, 18))
    mass = np.einsum("q,qid,qjd->ij", wdet / (2.0 * mu), psi, psi)
    div = np.trace(s_tab[1:dim + 1, :, :, 0:dim], axis1=0, axis2=3).T / det  # [4, Q]
    ddiv = (div * wdet) @ div.T
    for c in range(3):
        idx = np.arange(4) * 3 + c
        j[np.ix_(idx, idx)] += mass + ddiv
    vf = (1.0 / (2.0 * mu)) * (lam / (2.0 * mu + dim * lam))
    flat = psi.reshape(Q, 12)
    j[:12, :12] -= np.einsum("q,qa,qb->ab", vf * wdet, flat, flat)
    for k in range(12, 18):
        j[k, k] += np.sum(wdet)
    return np.zeros(18), j


def darcy_dirichlet_facet(Xc, signs_c, local_face, Xf, dim, quad_f, p_D):
    """LaplaceDualWeakFormBCDirichlet.evaluate_form (laplace_dual_weak_form.py:90-154)
    for one boundary facet: r = sum_q |det J_F| w_q p_D(x_q) (psi_f . n), with
    psi_f the neighbour cell's oriented RT1 function of that face and n the
    outward unit normal of compute_normal.py:7-24.  Xc [d+1, 3] cell
    vertices, Xf [d, 3] facet vertices (file order).  Returns the scalar
    residual entry of the face's flux DoF."""
    from .geometry import evaluate_mapping as emap
    pts, wts = quad_f
    xf, Jf, detf, _ = emap(dim - 1, pts, Xf)
    # outward normal (compute_normal.py): from the cell centroid to the facet centroid
    xc1 = Xf.mean(axis=0)
    xc0 = Xc.mean(axis=0)
    out = (xc1 - xc0) / np.linalg.norm(xc1 - xc0)
    if dim == 3:
        v = Xf[0] - xc1
        w = Xf[1] - xc1
        nrm = np.cross(v, w)
        nrm /= np.linalg.norm(nrm)
    else:
        v = (Xf[1] - Xf[0]) / np.linalg.norm(Xf[1] - Xf[0])
        w = np.cross(v, out)
        w /= np.linalg.norm(w)
        nrm = np.cross(v, w)
    if nrm @ out < 0:
        nrm = -nrm
    # psi_f at the facet points, through the neighbour cell's mapping
    Jc = (Xc[1:] - Xc[0]).T  # [3, d]
    xhat = np.linalg.lstsq(Jc, (xf - Xc[0]).T, rcond=None)[0].T  # reference coordinates
    x, J, det, pinv = emap(dim, xhat, Xc)
    tab = tabulate_oriented("RT", dim, 1, xhat, J, det, pinv, signs_c)
    psi = tab[0, :, local_face, :]  # [Q, 3]
    pd = np.ravel(np.asarray(p_D(xf[:, 0], xf[:, 1], xf[:, 2]))[0]) * np.ones(len(wts))
    return float(np.sum(detf * wts * pd * (psi @ nrm)))
