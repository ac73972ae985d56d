"""Element matrices from the device forms (evaluate_forms / evaluate_form)
against the reference's own weak forms on the same cells: the fixtures hold
LaplaceDualWeakForm / LEPrimalWeakForm / LCEDualWeakForm output of the
reference itself (tests/golden/make_golden.py).  Tolerance: FP64 within
1e-12 of the largest entry of each fixture."""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from oracle import assembly
from tests.cases import CASES, FORM_FUNCTIONS, FORM_FUNCTIONS_DEVICE, golden
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu

FORMS = {"darcy": nf.LaplaceDualWeakForm, "elast": nf.LEPrimalWeakForm, "cosserat": nf.LCEDualWeakForm,
         "le": nf.LEDualWeakForm}


def kind_of(name):
    return name.split("_")[0].rstrip("23d")


def reference_arrays(name):
    g = golden(name)
    kind = kind_of(name)
    if kind in ("cosserat", "le"):
        return g["r_el"], g["j_el"], FORM_FUNCTIONS[kind]
    return g["r_el_dev"], g["j_el_dev"], FORM_FUNCTIONS_DEVICE[kind]


CELL_CASES = ["darcy2d_n4", "darcy3d_n2", "darcy3d_msh0", "elast3d_n2", "cosserat3d_n1", "cosserat3d_msh0",
              "le3d_n1", "le3d_msh0"]


@pytest.mark.parametrize("name", CELL_CASES)
def test_element_matrices_equal_reference(cuda_lib, name):
    mk, fields = CASES[name]
    sp = product_space(mk(), fields)
    r_ref, j_ref, fn = reference_arrays(name)
    wf = FORMS[kind_of(name)](sp)
    wf.functions = fn
    r, j = wf.evaluate_forms(np.arange(sp.n_cells))
    torch.cuda.synchronize()
    scale = np.abs(j_ref).max()
    np.testing.assert_allclose(j.cpu().numpy(), j_ref, rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(r.cpu().numpy(), r_ref, rtol=0, atol=1e-12 * max(np.abs(r_ref).max(), 1e-300))
    # one cell through the reference's per-element signature, at alpha != 0:
    # r(alpha) = r(0) + j alpha_l for these linear forms
    i = sp.n_cells // 2
    a = np.linspace(-1.0, 1.0, sp.n_loc)
    r1, j1 = wf.evaluate_form(i, a)
    np.testing.assert_allclose(j1, j_ref[i], rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(r1, r_ref[i] + j_ref[i] @ a, rtol=0, atol=1e-11 * scale)


@pytest.mark.parametrize("name", ["darcy3d_n2", "elast3d_n2"])
def test_device_form_on_a_cell_subset_at_nonzero_alpha(cuda_lib, name):
    """SequentialAssembler with a device form, part of the cells and alpha
    != 0: the element data of those cells at alpha, scattered."""
    mk, fields = CASES[name]
    g = golden(name)
    sp = product_space(mk(), fields)
    r_ref, j_ref, fn = reference_arrays(name)
    wf = FORMS[kind_of(name)](sp)
    wf.functions = fn
    A = nf.CSRMatrix(sp)
    res = A.createVecLeft()
    rng = np.random.default_rng(2)
    alpha = rng.standard_normal(sp.n_dof)
    seq = np.sort(rng.choice(sp.n_cells, sp.n_cells // 3, replace=False))
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"w": ["form", seq, wf, alpha]}
    asm.scatter_forms()
    A.assemble()
    cd = g["cell_dofs"]
    r_a = np.array([r_ref[i] + j_ref[i] @ alpha[cd[i]] for i in seq])
    O, ro = assembly.assemble_csr(cd[seq], j_ref[seq], r_a, int(g["n_dof"]))
    got = A.to_scipy().toarray()
    scale = np.abs(j_ref).max()
    np.testing.assert_allclose(got, O.toarray(), rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(res.cpu().numpy(), ro, rtol=0, atol=1e-11 * max(scale, np.abs(ro).max()))


@pytest.mark.parametrize("name", ["le3d_n1", "le3d_msh0"])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_le_riesz_map_equals_reference(cuda_lib, name, dtype, tol):
    """LERieszMapWeakForm on the device (the Cosserat node-row kernel over
    the 18-DoF layout) against the reference's own
    LERieszMapWeakForm.evaluate_form_vectorized; the assembled operator
    against the oracle's."""
    from tests.cases import LE_RIESZ_FUNCTIONS
    mk, fields = CASES[name]
    g = golden(name)
    sp = product_space(mk(), fields)
    wf = nf.LERieszMapWeakForm(sp)
    wf.functions = LE_RIESZ_FUNCTIONS
    r, j = wf.evaluate_forms(np.arange(sp.n_cells), dtype=dtype)
    scale = np.abs(g["j_riesz"]).max()
    np.testing.assert_allclose(j.double().cpu().numpy(), g["j_riesz"], rtol=0, atol=tol * scale)
    assert float(r.abs().max().item()) == 0.0
    A = nf.CSRMatrix(sp, dtype=dtype)
    wf.assemble(A)
    A.assemble()
    O, _ = assembly.assemble_csr(g["cell_dofs"], g["j_riesz"], np.zeros(g["cell_dofs"].shape), int(g["n_dof"]))
    Ag = A.to_scipy()
    np.testing.assert_array_equal(Ag.indptr, O.indptr)
    np.testing.assert_allclose(Ag.toarray(), O.toarray(), rtol=0, atol=tol * scale)
