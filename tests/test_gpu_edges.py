"""Edge cases of the newer entry points: empty batches, zero right-hand
sides, DoFs outside the matrix (reported in the status word, no fault)."""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from nfempy_gb300 import _lib
from tests.cases import CASES, FORM_FUNCTIONS_DEVICE
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu


def darcy_case():
    mk, fields = CASES["darcy3d_n2"]
    sp = product_space(mk(), fields)
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = FORM_FUNCTIONS_DEVICE["darcy"]
    return sp, wf


def test_empty_batches(cuda_lib):
    sp, wf = darcy_case()
    r, j = wf.evaluate_forms([])
    assert r.shape == (0, sp.n_loc) and j.shape == (0, sp.n_loc, sp.n_loc)
    A = nf.CSRMatrix(sp)
    res = A.createVecLeft()
    z = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert _lib.lib().nfem_scatter_elements(_lib.NFEM_F64, 0, sp.n_loc, _lib.ptr(z), None, None, _lib.ptr(A.row_ptr),
                                            _lib.ptr(A.col_idx), A.n_rows, _lib.ptr(A.values), _lib.ptr(res),
                                            _lib.ptr(A.status), None) == 0
    assert _lib.lib().nfem_csr_add_entries(_lib.NFEM_F64, 0, None, None, None, _lib.ptr(A.row_ptr),
                                           _lib.ptr(A.col_idx), A.n_rows, _lib.ptr(A.values), _lib.ptr(A.status),
                                           None) == 0
    A.assemble()  # nothing buffered: a no-op
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"none": ["bc_form", [], object(), None]}
    asm.scatter_forms()
    assert float(A.values.abs().max().item()) == 0.0


def test_scatter_rejects_dofs_outside_the_matrix(cuda_lib):
    sp, _ = darcy_case()
    A = nf.CSRMatrix(sp)
    res = A.createVecLeft()
    dofs = torch.tensor([[0, A.n_rows]], dtype=torch.int32, device="cuda")  # the second is one past the end
    jel = torch.ones((1, 2, 2), dtype=torch.float64, device="cuda")
    _lib.call("nfem_scatter_elements", _lib.NFEM_F64, 1, 2, _lib.ptr(dofs), _lib.ptr(jel), None,
              _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), A.n_rows, _lib.ptr(A.values), _lib.ptr(res),
              _lib.ptr(A.status), None)
    with pytest.raises(_lib.NfemError) as e:
        A.check_status("scatter")
    assert _lib.STATUS_NAMES[e.value.status] == "NFEM_ERR_INVALID_ARG"


def test_cg_zero_rhs_and_tc_empty_batch(cuda_lib):
    from nfempy_gb300.solvers import CGSolver
    from oracle import mesh_gen
    sp = product_space(mesh_gen.cube(2), [("u", "P", 2, 3, False)])
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LEPrimalWeakForm(sp)
    wf.functions = {"lambda": 1.0, "mu": 1.0, "rhs": None}
    wf.assemble(A, res)
    x, info = CGSolver(A).solve(torch.zeros(A.n_rows, dtype=torch.float64, device="cuda"))
    assert info.status == 0 and info.inner_iterations == 0 and float(x.abs().max().item()) == 0.0
    d = torch.tensor([8, 256, 256, 1], dtype=torch.int32)
    P = torch.zeros(10, device="cuda")
    assert _lib.lib().nfem_mlp_infer_tc(_lib.C.c_void_p(d.data_ptr()), _lib.ptr(P), _lib.ptr(P), 0, None, None, None,
                                        None) == 0
