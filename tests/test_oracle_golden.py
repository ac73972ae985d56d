"""The oracle against the fixtures produced by the reference's own code."""
import numpy as np
import pytest

from oracle import assembly, forms, geometry, quadrature, topology
from tests.cases import CASES, golden


@pytest.mark.parametrize("name", sorted(CASES))
def test_dof_map_and_pattern(name):
    mk, fields = CASES[name]
    m = mk()
    g = golden(name)
    topo = topology.Topology(m, physical_tags=[1])
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in fields])
    assert nd == int(g["n_dof"])
    np.testing.assert_array_equal(cd, g["cell_dofs"])
    np.testing.assert_array_equal(topo.cells, g["cell_vertices"])
    ip, ix = assembly.pattern_csr(cd, nd)
    rows = np.repeat(np.arange(nd), np.diff(ip))
    np.testing.assert_array_equal(rows, g["pattern_rows"])
    np.testing.assert_array_equal(ix, g["pattern_cols"])
    n = cd.shape[1]
    A, _ = assembly.assemble_csr(cd, np.ones((topo.n_cells, n, n)), np.zeros(cd.shape), nd)
    np.testing.assert_array_equal(A.data, g["multiplicity"])


@pytest.mark.parametrize("name", [n for n in sorted(CASES) if "darcy" in n or "cosserat" in n])
def test_orientation_mapping_basis(name):
    mk, fields = CASES[name]
    m = mk()
    g = golden(name)
    dim = m["dim"]
    topo = topology.Topology(m, physical_tags=[1])
    if dim == 2:
        np.testing.assert_array_equal(~topo.facet_reflected, g["edge_oriented"])
    else:
        np.testing.assert_array_equal(topo.facet_tagged, g["bc_entities"])
        np.testing.assert_array_equal(topo.rt1_signs() < 0, g["face_reflections"] % 2 == 1)
    pts, wts = g["quad_points"], g["quad_weights"]
    qp, qw = quadrature.make_quadrature(dim, 3)
    np.testing.assert_allclose(qp, pts, atol=1e-15)
    np.testing.assert_allclose(qw, wts, atol=1e-15)
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    for c in range(topo.n_cells):
        x, J, det, pinv = geometry.evaluate_mapping(dim, pts, X[c])
        np.testing.assert_array_equal(det, g["det_jac"][c])
        np.testing.assert_array_equal(pinv, g["inv_jac"][c])
        tab = forms.tabulate_oriented("RT", dim, 1, pts, J, det, pinv, s[c])
        np.testing.assert_array_equal(tab, g["rt_basis"][c])
    _, detb, pinvb = geometry.cell_jacobians(X)
    np.testing.assert_allclose(np.broadcast_to(detb[:, None], g["det_jac"].shape), g["det_jac"], rtol=1e-14)
    np.testing.assert_allclose(np.broadcast_to(pinvb[:, None], g["inv_jac"].shape), g["inv_jac"], atol=1e-13)


def test_pattern_b_filter():
    """Driver filter: drops |v| <= 1e-8, keeps row <= col, adds zero diagonals."""
    cd = np.array([[0, 1, 2]])
    j = np.array([[[1.0, 1e-9, 2.0], [1e-9, 0.0, 3.0], [2.0, 3.0, 4.0]]])
    ip, ix = assembly.pattern_b(cd, j, 3)
    rows = np.repeat(np.arange(3), np.diff(ip))
    assert list(zip(rows.tolist(), ix.tolist())) == [(0, 0), (0, 2), (1, 1), (1, 2), (2, 2)]


@pytest.mark.parametrize("name", sorted(CASES))
def test_element_forms_match_reference(name):
    """The oracle's element residuals and Jacobians against the ones the
    reference's own weak forms computed (LaplaceDualWeakForm, LEPrimalWeakForm
    through a forward-mode auto_diff stand-in; LCEDualWeakForm.
    evaluate_form_vectorized), cell by cell, with the same coefficient
    functions.  Bar: 1e-13 of the largest entry of the cell."""
    from tests.cases import COSSERAT_PARAMS, FORM_FUNCTIONS
    mk, fields = CASES[name]
    m = mk()
    g = golden(name)
    dim = m["dim"]
    topo = topology.Topology(m, physical_tags=[1])
    X = m["points"][topo.cells]
    kmax = max(f[2] for f in fields)
    quad = quadrature.make_quadrature(dim, 2 * kmax + 1)
    kind = name.split("_")[0].rstrip("23d")
    F = FORM_FUNCTIONS[kind]
    signs = topo.rt1_signs() if kind != "elast" else None
    assert g["j_el"].shape[0] == topo.n_cells
    for c in range(topo.n_cells):
        if kind == "darcy":
            r, j = forms.darcy_element(X[c], signs[c], dim, quad, F["kappa"], F["rhs"])
        elif kind == "elast":
            r, j = forms.elasticity_element(X[c], dim, quad, F["lambda"], F["mu"], F["rhs"])
        elif kind == "le":
            r, j = forms.le_dual_element(X[c], signs[c], quad, 1.3, 0.7, F["rhs"])
        else:
            r, j = forms.cosserat_element(X[c], signs[c], quad, COSSERAT_PARAMS, F["rhs"], None)
        jr, rr = g["j_el"][c], g["r_el"][c]
        assert j.shape == jr.shape and r.shape == rr.shape
        scale = np.abs(jr).max()
        np.testing.assert_allclose(j, jr, rtol=0, atol=1e-13 * scale, err_msg=f"{name} cell {c} j_el")
        np.testing.assert_allclose(r, rr, rtol=0, atol=1e-13 * max(np.abs(rr).max(), 1e-300),
                                   err_msg=f"{name} cell {c} r_el")


def test_cosserat_riesz_map_matches_reference():
    """oracle.forms.cosserat_riesz_element against the reference's own
    LCEScaledRieszMapWeakForm.evaluate_form_vectorized (varying l, so the
    grad l . v part of the scaled divergence is pinned too), 1e-13 of the
    cell's largest entry."""
    from tests.cases import COSSERAT_PARAMS, RIESZ_FUNCTIONS
    mk, fields = CASES["cosserat3d_n1"]
    m = mk()
    g = golden("cosserat3d_n1")
    topo = topology.Topology(m, physical_tags=[1])
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(3, 3)
    for c in range(topo.n_cells):
        _, j = forms.cosserat_riesz_element(X[c], s[c], quad, COSSERAT_PARAMS, RIESZ_FUNCTIONS["l"],
                                            RIESZ_FUNCTIONS["grad_l"])
        jr = g["j_riesz"][c]
        np.testing.assert_allclose(j, jr, rtol=0, atol=1e-13 * np.abs(jr).max(), err_msg=f"cell {c}")


@pytest.mark.parametrize("name", ["le3d_n1", "le3d_msh0"])
def test_le_riesz_map_matches_reference(name):
    """oracle.forms.le_riesz_element against the reference's own
    LERieszMapWeakForm.evaluate_form_vectorized on the mixed linear-elastic
    space (s RT1^3, u P0^3, t P0^3), 1e-13 of the cell's largest entry."""
    from tests.cases import LE_RIESZ_FUNCTIONS
    mk, fields = CASES[name]
    m = mk()
    g = golden(name)
    topo = topology.Topology(m, physical_tags=[1])
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(3, 3)
    assert g["j_riesz"].shape == (topo.n_cells, 18, 18)
    for c in range(topo.n_cells):
        _, j = forms.le_riesz_element(X[c], s[c], quad, LE_RIESZ_FUNCTIONS["lambda"], LE_RIESZ_FUNCTIONS["mu"])
        jr = g["j_riesz"][c]
        np.testing.assert_allclose(j, jr, rtol=0, atol=1e-13 * np.abs(jr).max(), err_msg=f"{name} cell {c}")
