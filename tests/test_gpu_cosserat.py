"""Mixed Cosserat assembly on the GPU vs the FP64 oracle (oracle/forms.cosserat_element).

Tolerances: FP64 within 1e-12, FP32 within 1e-5, relative to each row's
largest entry; the pattern and DoF map are checked bit-exact."""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from nfempy_gb300.assembly import LCEDualWeakForm
from oracle import assembly, forms, mesh_gen, quadrature, solve, topology
from tests.cases import golden
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu
FIELDS = [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False), ("u", "P", 0, 3, True), ("t", "P", 0, 3, True)]
PAR = dict(lambda_s=1.0, mu_s=1.0, kappa_s=0.5, lambda_o=1.0, mu_o=1.0, kappa_o=0.5, l=0.7)


def row_scaled_err(Ag, Ao):
    d = (Ag - Ao).tocsr()
    scale = np.maximum(abs(Ao).max(axis=1).toarray().ravel(), 1e-300)
    return (abs(d).max(axis=1).toarray().ravel() / scale).max()


@pytest.mark.parametrize("rows", [0, 2])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("n", [1, 3])
def test_cosserat_matches_oracle(cuda_lib, dtype, tol, n, rows):
    """rows: the node-row kernel (2 register accumulation, 0 the default
    shared-memory row images), the NFEM_KNOB_ELAS_ROWS launch knob."""
    from nfempy_gb300 import autotune
    autotune.set_knobs({"elas_rows": rows})
    try:
        _check_cosserat(dtype, tol, n)
    finally:
        autotune.reset_knobs()


def _check_cosserat(dtype, tol, n, mesh=None):
    m = mesh_gen.cube(n) if mesh is None else mesh
    sp = product_space(m, FIELDS)
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in FIELDS])
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
    if n == 1:
        np.testing.assert_array_equal(cd, golden("cosserat3d_n1")["cell_dofs"])
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = LCEDualWeakForm(sp)
    f6 = [1.0, -2.0, 0.5, 0.3, 0.0, -1.0]
    wf.functions = dict(PAR, rhs=f6)
    wf.assemble(A, res)
    torch.cuda.synchronize()
    A.check_status("cosserat")
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(3, 3)
    rs, js = [], []
    for c in range(topo.n_cells):
        r, j = forms.cosserat_element(X[c], s[c], quad, PAR, f6[:3], f6[3:])
        rs.append(r)
        js.append(j)
    Ao, ro = assembly.assemble_csr(cd, np.array(js), np.array(rs), nd)
    Ag = A.to_scipy()
    np.testing.assert_array_equal(Ag.indptr, Ao.indptr)
    np.testing.assert_array_equal(Ag.indices, Ao.indices)
    assert row_scaled_err(Ag, Ao) <= tol
    rg = res.double().cpu().numpy()
    assert np.abs(rg - ro).max() <= tol * np.abs(ro).max()


@pytest.mark.parametrize("flat", [1 / 512, 1 / 4096])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_cosserat_badly_shaped_cells(cuda_lib, flat, dtype, tol):
    """Flat tetrahedra in general orientation (shape quality ~ flat): the
    FP32 geometry pass takes J and det J of such cells in FP64 from the
    points.  Against the FP64 oracle at the usual tolerance, except that FP64
    is held to max(1e-12, 10 ulp / q_min): the oracle's own det J is only
    that accurate there."""
    from tests.test_gpu_darcy import _badly_shaped
    m = _badly_shaped("cube", 2, flat)
    E = m["points"][m["blocks"][-1][1]]
    E = E[:, 1:] - E[:, :1]
    q = np.abs(np.linalg.det(E)) / np.prod(np.linalg.norm(E, axis=2), axis=1)
    if dtype == torch.float64:
        tol = max(tol, 10 * 2.0 ** -53 / q.min())
    _check_cosserat(dtype, tol, 2, mesh=m)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_riesz_map_matches_oracle(cuda_lib, dtype, tol):
    """LCEScaledRieszMapWeakForm on the device against the oracle restatement
    that the reference's own form pins (constant l here: the device form
    takes one length scale), in the dual form's CSR pattern."""
    from nfempy_gb300.assembly import LCEScaledRieszMapWeakForm
    m = mesh_gen.cube(3)
    sp = product_space(m, FIELDS)
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in FIELDS])
    A = nf.CSRMatrix(sp, dtype=dtype)
    par = dict(PAR)
    wf = LCEScaledRieszMapWeakForm(sp)
    wf.functions = dict(par, l=lambda x, y, z: 0.7 + 0 * x, grad_l=lambda x, y, z: np.zeros((3,) + np.shape(x)))
    wf.assemble(A)
    torch.cuda.synchronize()
    A.check_status("riesz")
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(3, 3)
    js = [forms.cosserat_riesz_element(X[c], s[c], quad, par, lambda x, y, z: 0.7 + 0 * x,
                                       lambda x, y, z: np.zeros((3,) + np.shape(x)))[1] for c in range(topo.n_cells)]
    Po, _ = assembly.assemble_csr(cd, np.array(js), np.zeros((topo.n_cells, 30)), nd)
    Pg = A.to_scipy()
    np.testing.assert_array_equal(Pg.indptr, Po.indptr)
    np.testing.assert_array_equal(Pg.indices, Po.indices)
    assert row_scaled_err(Pg, Po) <= tol


def test_cosserat_solve_matches_superlu_and_converges(cuda_lib):
    """The mixed Cosserat system (manufactured solution's load) solved on the
    device to 1e-8 FP64 relative residual by FGMRES with the cell-block
    Jacobi preconditioner (30 x 30 blocks): equal to SuperLU's solution of
    the oracle's system to 1e-6, and the P0 displacement / rotation errors
    against the exact fields fall by about 2x per mesh halving."""
    from nfempy_gb300 import workloads as wl
    from nfempy_gb300.solvers import KrylovSolver
    rhs, exact = wl.cosserat_manufactured()
    errs = []
    for n in (2, 4):
        m = mesh_gen.cube(n)
        sp = product_space(m, FIELDS)
        fn = dict(wl.COSSERAT_MATERIAL, rhs=rhs)
        A64 = nf.CSRMatrix(sp, dtype=torch.float64)
        r64 = torch.empty(A64.n_rows, dtype=torch.float64, device="cuda")
        wf = LCEDualWeakForm(sp)
        wf.functions = fn
        wf.assemble(A64, r64)
        A32 = A64.with_dtype(torch.float32)
        r32 = torch.empty(A64.n_rows, dtype=torch.float32, device="cuda")
        wf.assemble(A32, r32)
        ksp = KrylovSolver(A64, pc="cell_block", A32_values=A32.values, restart=30)
        x, info = ksp.solve(-r64, rtol=1e-8)
        assert info.final_relres <= 1e-8
        xg = x.cpu().numpy()
        Ag = A64.to_scipy()
        xo = solve.solve_newton_step(Ag, r64.cpu().numpy())
        assert np.linalg.norm(xg - xo) <= 1e-6 * np.linalg.norm(xo)
        e = nf.l2_error(3, sp, exact, xg, skip_fields=["s", "m"])
        errs.append(e)
    errs = np.array(errs)
    rates = errs[0] / errs[1]
    assert np.all(rates > 1.6), (errs, rates)


def test_cosserat_dirichlet_matches_oracle(cuda_lib):
    """LCEDualWeakFormBCDirichlet: -int_F u_D[c] (tau . n) on the stress rows
    and -int_F t_D[c] (v . n) on the couple-stress rows of every boundary
    facet's flux DoF, against the oracle's facet restatement (normal from
    compute_normal, basis traced from the neighbour cell), FP64 1e-12."""
    from nfempy_gb300.assembly import LCEDualWeakFormBCDirichlet
    m = mesh_gen.cube(2)
    sp = product_space(m, FIELDS)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    uD = lambda x, y, z: np.array([1 + x, y * z, np.sin(z) + 0 * x])
    tD = lambda x, y, z: np.array([0.5 + 0 * x, x * x, y - z])
    bc = LCEDualWeakFormBCDirichlet(sp)
    bc.functions = {"u": uD, "t": tD}
    bc.assemble(A, res)
    torch.cuda.synchronize()
    rg = res.cpu().numpy()
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in FIELDS])
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    qf = quadrature.make_quadrature(2, 3)
    ro = np.zeros(nd)
    occ, fverts = bc.facets()
    assert len(occ) == 6 * 2 * 2 * 2
    for o, fv in zip(occ, fverts):
        c, i = divmod(int(o), 4)
        for off, fn in ((0, uD), (12, tD)):
            for comp in range(3):
                val = forms.darcy_dirichlet_facet(X[c], s[c], i, m["points"][fv], 3, qf,
                                                  lambda x, y, z: np.array([fn(x, y, z)[comp]]))
                ro[cd[c, off + i * 3 + comp]] -= val
    np.testing.assert_allclose(rg, ro, rtol=1e-12, atol=1e-13 * np.abs(ro).max())


def test_le_dual_dirichlet_matches_oracle(cuda_lib):
    """LEDualWeakFormBCDirichlet (le_dual_weak_form.py:518-595): -int_F u_D[c]
    (tau . n) on the stress rows of every boundary facet's flux DoF of the
    mixed linear-elastic space (s, u, t), against the oracle's facet
    restatement, FP64 1e-12."""
    from nfempy_gb300.assembly import LEDualWeakFormBCDirichlet
    from tests.cases import LE_FIELDS
    m = mesh_gen.cube(2)
    sp = product_space(m, LE_FIELDS)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    uD = lambda x, y, z: np.array([1 + x, y * z, np.sin(z) + 0 * x])
    bc = LEDualWeakFormBCDirichlet(sp)
    bc.functions = {"u": uD}
    bc.assemble(A, res)
    torch.cuda.synchronize()
    rg = res.cpu().numpy()
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in LE_FIELDS])
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    qf = quadrature.make_quadrature(2, 3)
    ro = np.zeros(nd)
    occ, fverts = bc.facets()
    for o, fv in zip(occ, fverts):
        c, i = divmod(int(o), 4)
        for comp in range(3):
            val = forms.darcy_dirichlet_facet(X[c], s[c], i, m["points"][fv], 3, qf,
                                              lambda x, y, z: np.array([uD(x, y, z)[comp]]))
            ro[cd[c, i * 3 + comp]] -= val
    np.testing.assert_allclose(rg, ro, rtol=1e-12, atol=1e-13 * np.abs(ro).max())
