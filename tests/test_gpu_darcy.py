"""Mixed Darcy RT1 x P0 assembly on the GPU vs the FP64 oracle.

Tolerances (from the path's accuracy contract): FP64 entries within 1e-12
relative, FP32 entries within 1e-5 relative; "relative" is measured against
the largest entry of the same row (entries that cancel to round-off are
compared at that scale).
"""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from oracle import mesh_gen, solve
from tests.gpu_helpers import darcy_oracle, product_space

pytestmark = pytest.mark.gpu
PI = np.pi
DARCY = [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)]


def f2d(x, y, z):
    return np.array([2 * PI ** 2 * np.sin(PI * x) * np.sin(PI * y)])


def assemble_gpu(m, kappa, rhs, dtype):
    sp = product_space(m, DARCY)
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": rhs}
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"darcy": ["form", range(sp.n_cells), wf, None]}
    asm.scatter_forms()
    A.assemble()
    torch.cuda.synchronize()
    return sp, A, res


def row_scaled_err(Ag, Ao):
    d = (Ag - Ao).tocsr()
    scale = np.maximum(abs(Ao).max(axis=1).toarray().ravel(), 1e-300)
    return (abs(d).max(axis=1).toarray().ravel() / scale).max()


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("gen,n", [("square", 4), ("square", 32), ("cube", 2), ("cube", 6)])
def test_darcy_matrix_matches_oracle(cuda_lib, dtype, tol, gen, n):
    m = getattr(mesh_gen, gen)(n)
    T = m["blocks"][-1][1].shape[0]
    kappa = np.exp(np.sin(np.arange(T) * 0.37))
    f_cell = np.cos(np.arange(T) * 0.11)
    sp, A, res = assemble_gpu(m, kappa, f_cell, dtype)
    Ao, ro, cd, nd, topo = darcy_oracle(m, kappa, f_cell=f_cell)
    Ag = A.to_scipy()
    np.testing.assert_array_equal(Ag.indptr, Ao.indptr)
    np.testing.assert_array_equal(Ag.indices, Ao.indices)
    assert row_scaled_err(Ag, Ao) <= tol
    rg = res.double().cpu().numpy()
    assert np.abs(rg - ro).max() <= tol * np.abs(ro).max()


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_darcy_cfg1_manufactured_rhs_and_solve(cuda_lib, dtype, tol):
    """2-D mixed Darcy, 32x32 squares -> 2048 triangles, K = 1, f from
    p = sin(pi x) sin(pi y), sampled at the quadrature points; FP64 solve."""
    m = mesh_gen.square(32)
    sp, A, res = assemble_gpu(m, 1.0, f2d, dtype)
    assert sp.n_dof == 5184 and A.nnz == 29760
    Ao, ro, cd, nd, topo = darcy_oracle(m, np.ones(2048), f_callable=f2d)
    Ag = A.to_scipy()
    assert row_scaled_err(Ag, Ao) <= tol
    rg = res.double().cpu().numpy()
    assert np.abs(rg - ro).max() <= tol * np.abs(ro).max()
    xo = solve.solve_newton_step(Ao, ro)
    xg = solve.solve_newton_step(Ag, rg)
    rel = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    assert rel <= (1e-10 if dtype == torch.float64 else 1e-4), rel


def test_darcy_accumulate_and_callable_kappa(cuda_lib):
    m = mesh_gen.cube(3)
    sp, A, res = assemble_gpu(m, lambda x, y, z: 2.0 * np.ones_like(x), 1.0, torch.float64)
    Ao, ro, *_ = darcy_oracle(m, 2.0 * np.ones(m["blocks"][-1][1].shape[0]), f_cell=np.ones(162))
    assert row_scaled_err(A.to_scipy(), Ao) <= 1e-12
    # a second form in the same pass accumulates
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": 2.0, "rhs": 1.0}
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"a": ["form", range(sp.n_cells), wf, None], "b": ["form", range(sp.n_cells), wf, None]}
    A.zeroEntries()
    asm.scatter_forms()
    torch.cuda.synchronize()
    assert row_scaled_err(A.to_scipy(), 2 * Ao) <= 1e-12
    np.testing.assert_allclose(res.cpu().numpy(), 2 * ro, rtol=1e-12, atol=1e-15)


def test_darcy_host_residual_and_deterministic(cuda_lib):
    m = mesh_gen.cube(4)
    sp = product_space(m, DARCY)
    A = nf.CSRMatrix(sp, dtype=torch.float32)
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": np.linspace(0.5, 2.0, sp.n_cells), "rhs": 3.0}
    host = np.zeros(A.n_rows)
    asm = nf.SequentialAssembler(sp, A, host)
    asm.form_to_input_list = {"d": ["form", range(sp.n_cells), wf, None]}
    asm.scatter_forms()
    v1 = A.values.clone()
    A.zeroEntries()
    host2 = np.zeros(A.n_rows)
    asm.residual = host2
    asm.scatter_forms()
    assert torch.equal(v1, A.values)  # bitwise reproducible
    np.testing.assert_array_equal(host, host2)
    assert np.abs(host).max() > 0
