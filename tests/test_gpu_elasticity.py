"""Vector P2 elasticity assembly on the GPU vs the FP64 oracle.

Tolerances: FP64 entries within 1e-12 and FP32 within 1e-5, relative to the
largest entry of each row; residual likewise.  The boundary penalty (beta =
1e12) is checked separately against an oracle facet mass."""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from nfempy_gb300.assembly import LEPrimalWeakForm, LEPrimalWeakFormBCDirichlet
from oracle import assembly, elements, forms, mesh_gen, quadrature, topology
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu
FIELD = [("u", "P", 2, 3, False)]


def oracle_system(m, lam, mu, f):
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*FIELD[0])])
    X = m["points"][topo.cells]
    quad = quadrature.make_quadrature(3, 5)
    fq = np.repeat(np.asarray(f)[:, None, :], len(quad[1]), 1)
    r, j = forms.elasticity_batch(X, 3, quad, lam, mu, fq)
    A, res = assembly.assemble_csr(cd, j, r, nd)
    return A, res, cd, topo


def row_scaled_err(Ag, Ao):
    d = (Ag - Ao).tocsr()
    scale = np.maximum(abs(Ao).max(axis=1).toarray().ravel(), 1e-300)
    return (abs(d).max(axis=1).toarray().ravel() / scale).max()


@pytest.mark.parametrize("rows", [1, 2, 3])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("n", [1, 2, 4])
def test_elasticity_matches_oracle(cuda_lib, dtype, tol, n, rows):
    """rows: the node-row kernel (2 register accumulation, 1 shared-memory
    row images), chosen by the NFEM_KNOB_ELAS_ROWS launch knob."""
    from nfempy_gb300 import autotune
    autotune.set_knobs({"elas_rows": rows})
    try:
        _check_elasticity(dtype, tol, n)
    finally:
        autotune.reset_knobs()


def _check_elasticity(dtype, tol, n, mesh=None):
    m = mesh_gen.cube(n) if mesh is None else mesh
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(n)
    lam = np.exp(rng.normal(0, 0.5, T))
    mu = np.exp(rng.normal(0, 0.5, T))
    f = np.stack([np.ones(T), 2 * np.ones(T), np.linspace(-1, 1, T)], 1)
    sp = product_space(m, FIELD)
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = LEPrimalWeakForm(sp)
    wf.functions = {"lambda": lam, "mu": mu, "rhs": f}
    wf.assemble(A, res)
    torch.cuda.synchronize()
    A.check_status("elasticity")
    Ao, ro, cd, topo = oracle_system(m, lam, mu, f)
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
    Ag = A.to_scipy()
    np.testing.assert_array_equal(Ag.indptr, Ao.indptr)
    np.testing.assert_array_equal(Ag.indices, Ao.indices)
    assert row_scaled_err(Ag, Ao) <= tol
    rg = res.double().cpu().numpy()
    assert np.abs(rg - ro).max() <= tol * np.abs(ro).max()


@pytest.mark.parametrize("flat", [1 / 512, 1 / 4096])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_elasticity_badly_shaped_cells(cuda_lib, flat, dtype, tol):
    """Flat tetrahedra in general orientation (shape quality ~ flat): the
    FP32 geometry pass takes J^-1 and det J of such cells in FP64 from the
    points.  Against the FP64 oracle at the usual tolerance."""
    from tests.test_gpu_darcy import _badly_shaped
    _check_elasticity(dtype, tol, 2, mesh=_badly_shaped("cube", 2, flat))


def test_elasticity_penalty_matches_oracle(cuda_lib):
    m = mesh_gen.cube(2)
    T = m["blocks"][-1][1].shape[0]
    sp = product_space(m, FIELD)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    wf = LEPrimalWeakForm(sp)
    wf.functions = {"lambda": 1.0, "mu": 1.0, "rhs": None}
    wf.assemble(A, res)
    bc = LEPrimalWeakFormBCDirichlet(sp)
    bc.functions = {"u": None}
    bc.assemble(A)
    torch.cuda.synchronize()
    A.check_status("penalty")
    Ao, _, cd, topo = oracle_system(m, np.ones(T), np.ones(T), np.zeros((T, 3)))
    # oracle facet penalty: beta int phi_a phi_b on each boundary triangle
    fd = bc.facet_dofs()[0].cpu().numpy().astype(np.int64)
    fv = bc.facet_dofs()[1].cpu().numpy().astype(np.int64)
    quad = quadrature.make_quadrature(2, 5)
    phi = elements.create_element("P", 2, 2).tabulate(0, quad[0])[0, :, :, 0]
    Mref = np.einsum("q,qa,qb->ab", quad[1], phi, phi)
    P = m["points"]
    rows, cols, vals = [], [], []
    for k in range(fd.shape[0]):
        e1 = P[fv[k, 1]] - P[fv[k, 0]]
        e2 = P[fv[k, 2]] - P[fv[k, 0]]
        det = np.linalg.norm(np.cross(e1, e2))
        for a in range(6):
            for b in range(6):
                for i in range(3):
                    rows.append(fd[k, 3 * a + i]); cols.append(fd[k, 3 * b + i])
                    vals.append(1e12 * det * Mref[a, b])
    import scipy.sparse as sps
    Pen = sps.coo_matrix((vals, (rows, cols)), shape=Ao.shape).tocsr()
    Ag = A.to_scipy()
    assert row_scaled_err(Ag, Ao + Pen) <= 1e-12
    # every boundary facet vertex DoF is penalised
    bnd_nodes = np.unique(fd)
    assert np.all(Ag.diagonal()[bnd_nodes] > 1e9)


def test_elasticity_clamped_solve(cuda_lib):
    """The elasticity driver's step (cg_elasticity_example_1.py:147-181): the
    penalised system A u = -r solved on the device (FGMRES with point Jacobi
    inside FP64 refinement) to 1e-8 FP64 relative residual, and equal to
    SuperLU's solution of the same system."""
    from nfempy_gb300.solvers import KrylovSolver
    from oracle import solve
    m = mesh_gen.cube(3)
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(5)
    sp = product_space(m, FIELD)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    wf = LEPrimalWeakForm(sp)
    wf.functions = {"lambda": np.exp(rng.normal(0, 0.5, T)), "mu": np.exp(rng.normal(0, 0.5, T)),
                    "rhs": np.array([1.0, 1.0, 1.0])}
    wf.assemble(A, res)
    bc = LEPrimalWeakFormBCDirichlet(sp)
    bc.functions = {"u": None}
    bc.assemble(A)
    torch.cuda.synchronize()
    ksp = KrylovSolver(A, pc="jacobi", restart=60)
    x, info = ksp.solve(-res, rtol=1e-8, max_inner=20000)
    assert info.status == 0 and info.final_relres <= 1e-8
    Ag = A.to_scipy()
    xo = solve.solve_newton_step(Ag, res.cpu().numpy())
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xo) <= 1e-5 * np.linalg.norm(xo)


@pytest.mark.parametrize("pc", ["jacobi", "node_block"])
def test_elasticity_clamped_solve_cg(cuda_lib, pc):
    """The driver's own solver family (cg_elasticity_example_1.py:159-170:
    CG on the SPD penalised system): CGSolver with point Jacobi or 3 x 3 node
    blocks in place of ICC, FP32 CG inside FP64 refinement, to 1e-8 FP64
    relative residual; equal to SuperLU's solution; twice the same solve
    gives bitwise the same iterate (fixed-order reductions)."""
    from nfempy_gb300.solvers import CGSolver
    from oracle import solve
    m = mesh_gen.cube(3)
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(5)
    sp = product_space(m, FIELD)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    wf = LEPrimalWeakForm(sp)
    wf.functions = {"lambda": np.exp(rng.normal(0, 0.5, T)), "mu": np.exp(rng.normal(0, 0.5, T)),
                    "rhs": np.array([1.0, 1.0, 1.0])}
    wf.assemble(A, res)
    bc = LEPrimalWeakFormBCDirichlet(sp)
    bc.functions = {"u": None}
    bc.assemble(A)
    torch.cuda.synchronize()
    cg = CGSolver(A, pc=pc)
    x, info = cg.solve(-res, rtol=1e-8)
    assert info.status == 0 and info.final_relres <= 1e-8, info.as_dict()
    rel = float(cg.residual(x, -res).norm() / res.norm())
    assert rel <= 1e-8
    x2, info2 = cg.solve(-res, rtol=1e-8)
    assert torch.equal(x, x2) and info2.inner_iterations == info.inner_iterations
    Ag = A.to_scipy()
    xo = solve.solve_newton_step(Ag, res.cpu().numpy())
    assert np.linalg.norm(x.cpu().numpy() - xo) <= 1e-5 * np.linalg.norm(xo)


def test_cg_refuses_a_zero_diagonal(cuda_lib):
    """The mixed Darcy saddle point (zero pressure block) is not a CG system:
    its point-Jacobi setup finds the zero diagonal and reports
    NFEM_ERR_DEGENERATE instead of dividing by it."""
    from nfempy_gb300 import _lib
    from nfempy_gb300.solvers import CGSolver
    from tests.cases import DARCY
    m = mesh_gen.cube(2)
    sp = product_space(m, DARCY)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": 1.0, "rhs": 1.0}
    wf.assemble(A, res)
    cg = CGSolver(A, pc="jacobi")
    with pytest.raises(_lib.NfemError) as e:
        cg.setup()
    assert _lib.STATUS_NAMES[e.value.status] == "NFEM_ERR_DEGENERATE"
