"""Known-answer and convergence checks of the oracle (CPU)."""
import numpy as np
import pytest

from oracle import assembly, elements, forms, mesh_gen, quadrature, solve, topology

PI = np.pi


def darcy_problem(dim, n):
    m = mesh_gen.square(n) if dim == 2 else mesh_gen.cube(n)
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "RT", 1), topology.FieldSpec("p", "P", 0, 1, True)])
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(dim, 3)
    pts, _ = quad
    lam = elements.create_element("P", dim, 1).tabulate(0, pts)[0, :, :, 0]
    xq = np.einsum("qv,tvg->tqg", lam, X)
    return m, topo, cd, nd, X, s, quad, xq


def f2(x, y, z):
    return np.array([2 * PI ** 2 * np.sin(PI * x) * np.sin(PI * y)])


def test_darcy_loop_equals_batch_2d_3d():
    for dim, n in ((2, 4), (3, 2)):
        m, topo, cd, nd, X, s, quad, xq = darcy_problem(dim, n)
        fq = np.sin(3 * xq[..., 0]) + xq[..., 1]
        kap = 1.0 + np.arange(topo.n_cells) % 3
        r, j = forms.darcy_batch(X, s, dim, quad, np.repeat(kap[:, None], len(quad[1]), 1), fq)
        for c in range(topo.n_cells):
            r1, j1 = forms.darcy_element(
                X[c], s[c], dim, quad, kap[c], lambda x, y, z, c=c: np.array([np.sin(3 * x) + y]))
            np.testing.assert_allclose(j1, j[c], rtol=1e-12, atol=1e-14)
            np.testing.assert_allclose(r1, r[c], rtol=1e-12, atol=1e-14)


def test_darcy_first_order_convergence_2d():
    errs = []
    for n in (8, 16, 32):
        m, topo, cd, nd, X, s, quad, xq = darcy_problem(2, n)
        fq = f2(xq[..., 0], xq[..., 1], xq[..., 2])[0]
        r, j = forms.darcy_batch(X, s, 2, quad, np.ones_like(fq), fq)
        A, res = assembly.assemble_csr(cd, j, r, nd)
        x = solve.solve_newton_step(A, res)
        ue = lambda x, y, z: np.array([-PI * np.cos(PI * x) * np.sin(PI * y), -PI * np.sin(PI * x) * np.cos(PI * y)])
        pe = lambda x, y, z: np.sin(PI * x) * np.sin(PI * y)
        errs.append(solve.l2_error_darcy(X, s, 2, quad, cd, x, ue, pe))
    errs = np.array(errs)
    rates = np.log2(errs[:-1] / errs[1:])
    assert np.all(rates > 0.95), rates


@pytest.mark.parametrize("dim", [2, 3])
def test_projector_reproduces_polynomials(dim):
    """Known-answer test of tests/test_projectors/test_projectors.py:86-216 logic:
    L2-projecting a polynomial the space contains reproduces it (1e-13)."""
    n = 2
    m = mesh_gen.square(n) if dim == 2 else mesh_gen.cube(n)
    topo = topology.Topology(m)
    X = m["points"][topo.cells]
    for family, k, disc, func, nc in (
            ("P", 2, False, lambda x, y, z: np.array([x * x + 2 * y - 0.5 * x * y + (z if dim == 3 else 0)]), 1),
            ("P", 1, True, lambda x, y, z: np.array([1 + x - y]), 1),
            ("RT", 1, False, None, 1)):
        quad = quadrature.make_quadrature(dim, 2 * k + 1)
        cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("f", family, k, nc, disc)])
        s = topo.rt1_signs()
        if family == "RT":
            a, b = 0.3, -0.7
            def func(x, y, z):
                v = [a + 2 * x, b + 2 * y] + ([0.1 + 2 * z] if dim == 3 else [])
                return np.array([np.stack(v)])
        r_l, j_l = [], []
        for c in range(topo.n_cells):
            r, j = forms.projector_element([("f", family, k, nc, disc)], X[c], dim, quad, {"f": func}, s[c])
            r_l.append(r)
            j_l.append(j)
        A, res = assembly.assemble_csr(cd, np.array(j_l), np.array(r_l), nd)
        x = solve.solve_newton_step(A, res)
        # evaluate at quadrature points and compare
        pts, wts = quad
        err = 0.0
        for c in range(topo.n_cells):
            from oracle.geometry import evaluate_mapping
            xq, J, det, pinv = evaluate_mapping(dim, pts, X[c])
            tab = forms.tabulate_oriented(family, dim, k, pts, J, det, pinv, s[c] if family == "RT" else None, disc)
            a_l = x[cd[c]]
            fe = func(xq[:, 0], xq[:, 1], xq[:, 2])
            if family == "P":
                fh = tab[0, :, :, 0] @ a_l
                err += np.sum(det * wts * (fe[0] - fh) ** 2)
            else:
                fh = np.einsum("qnd,n->qd", tab[0, :, :, :dim], a_l)
                err += np.sum(det * wts * np.sum((fe[0, :dim].T - fh) ** 2, axis=1))
        assert np.sqrt(err) < 1e-13, (family, k, np.sqrt(err))


def test_elasticity_loop_equals_batch():
    for dim, mk in ((3, lambda: mesh_gen.cube(1)), (2, lambda: mesh_gen.square(2))):
        m = mk()
        topo = topology.Topology(m)
        X = m["points"][topo.cells]
        quad = quadrature.make_quadrature(dim, 5)
        lam = 1.0 + 0.1 * np.arange(topo.n_cells)
        mu = 2.0 - 0.05 * np.arange(topo.n_cells)
        fq = np.ones((topo.n_cells, len(quad[1]), dim))
        r, j = forms.elasticity_batch(X, dim, quad, lam, mu, fq)
        for c in range(topo.n_cells):
            rhs = lambda x, y, z: np.ones((dim, np.size(x)))
            r1, j1 = forms.elasticity_element(X[c], dim, quad, lam[c], mu[c], rhs)
            np.testing.assert_allclose(j1, j[c], rtol=1e-12, atol=1e-13)
            np.testing.assert_allclose(r1, r[c], rtol=1e-12, atol=1e-14)
            # rigid translations are in the kernel
            t = np.tile(np.eye(dim)[0], j1.shape[0] // dim)
            assert np.abs(j1 @ t).max() < 1e-12


def test_cosserat_batch_equals_element():
    """The vectorised Cosserat oracle against the per-cell restatement that the
    reference's own form pins (load varying inside the cells)."""
    from oracle import forms, mesh_gen, quadrature, topology
    from tests.cases import COSSERAT_PARAMS, cosserat_rhs
    m = mesh_gen.cube(2)
    topo = topology.Topology(m)
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(3, 3)
    from oracle.elements import create_element
    lam = create_element("P", 3, 1).tabulate(0, quad[0])[0, :, :, 0]
    xq = np.einsum("qv,tvg->tqg", lam, X)
    fq = np.moveaxis(cosserat_rhs(xq[..., 0], xq[..., 1], xq[..., 2]), 0, -1)
    rb, jb = forms.cosserat_batch(X, s, quad, COSSERAT_PARAMS, fq)
    for c in range(topo.n_cells):
        r, j = forms.cosserat_element(X[c], s[c], quad, COSSERAT_PARAMS, cosserat_rhs, None)
        np.testing.assert_allclose(jb[c], j, rtol=0, atol=1e-14 * np.abs(j).max())
        np.testing.assert_allclose(rb[c], r, rtol=0, atol=1e-14 * np.abs(r).max())


def test_field_error_matches_darcy_l2():
    """The per-field restatement of l2_error equals the Darcy-specific one."""
    m, topo, cd, nd, X, s, quad, xq = darcy_problem(2, 6)
    rng = np.random.default_rng(2)
    alpha = rng.normal(size=nd)

    def u_ex(x, y, z):
        return np.array([np.sin(x) + y, x * y, 0.0 * x])

    def p_ex(x, y, z):
        return np.array([np.cos(x + y)])

    want = solve.l2_error_darcy(X, s, 2, quad, cd, alpha, u_ex, p_ex)
    eu = solve.field_error("RT", 2, quad, X, s, cd[:, :3], 1, 1, alpha, u_ex)
    ep = solve.field_error("Lagrange", 2, quad, X, s, cd[:, 3:], 1, 0, alpha, p_ex)
    np.testing.assert_allclose([eu, ep], want, rtol=1e-13)
