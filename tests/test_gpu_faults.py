"""Bad inputs fed from the host, and the GPU serving the next call.

Each case passes data whose VALUES are wrong (a degenerate tetrahedron, a
NaN or non-positive coefficient) while every index array stays in range, so
nothing can fault: the kernels record the condition in the status word
(first code wins) and the host raises NfemError with that code.  After each
bad call a good assembly on the same device must still match the oracle.
"""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from nfempy_gb300 import _lib
from nfempy_gb300.assembly import LCEDualWeakForm, LEPrimalWeakForm
from oracle import mesh_gen
from tests.gpu_helpers import darcy_oracle, product_space

pytestmark = pytest.mark.gpu
DARCY = [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)]
NONFINITE, DEGENERATE, DOMAIN = 10, 11, 12


def _darcy(m, kappa, dtype):
    sp = product_space(m, DARCY)
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": 1.0}
    wf.assemble(A, res)
    torch.cuda.synchronize()
    return sp, A, res


def _degenerate_cube(n):
    """cube(n) with vertex 1 moved onto vertex 0: every cell holding both has
    |det J| = 0 exactly (FP64 and the FP32 fixed-point records alike); ids are
    untouched."""
    m = mesh_gen.cube(n)
    pts = m["points"].copy()
    pts[1] = pts[0]
    return dict(m, points=pts)


def _good_darcy_matches_oracle(dtype, tol):
    m = mesh_gen.cube(3)
    T = m["blocks"][-1][1].shape[0]
    kappa = np.exp(np.sin(np.arange(T)))
    sp, A, res = _darcy(m, kappa, dtype)
    A.check_status("good assembly")
    Ao, ro, *_ = darcy_oracle(m, kappa, f_cell=np.ones(T))
    Ag = A.to_scipy()
    d = abs(Ag - Ao).max() / abs(Ao).max()
    assert d <= tol, d


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("case,code", [("degenerate", DEGENERATE), ("nan_kappa", NONFINITE),
                                       ("inf_kappa", NONFINITE), ("negative_kappa", DOMAIN),
                                       ("zero_kappa", DOMAIN)])
def test_darcy_bad_input_sets_status(cuda_lib, dtype, tol, case, code):
    m = _degenerate_cube(2) if case == "degenerate" else mesh_gen.cube(2)
    T = m["blocks"][-1][1].shape[0]
    kappa = np.ones(T)
    bad = {"nan_kappa": np.nan, "inf_kappa": np.inf, "negative_kappa": -1.0, "zero_kappa": 0.0}
    if case in bad:
        kappa[T // 2] = bad[case]
    sp, A, res = _darcy(m, kappa, dtype)
    with pytest.raises(_lib.NfemError) as err:
        A.check_status(case)
    assert err.value.status == code
    assert int(A.status.item()) == 0  # check_status clears the word
    _good_darcy_matches_oracle(dtype, tol)


@pytest.mark.parametrize("case,code", [("degenerate", DEGENERATE), ("nan_lambda", NONFINITE),
                                       ("negative_mu", DOMAIN)])
def test_elasticity_bad_input_sets_status(cuda_lib, case, code):
    m = _degenerate_cube(2) if case == "degenerate" else mesh_gen.cube(2)
    T = m["blocks"][-1][1].shape[0]
    lam, mu = np.ones(T), np.ones(T)
    if case == "nan_lambda":
        lam[3] = np.nan
    if case == "negative_mu":
        mu[7] = -0.5
    sp = product_space(m, [("u", "P", 2, 3, False)])
    A = nf.CSRMatrix(sp, dtype=torch.float32)
    res = torch.empty(A.n_rows, dtype=torch.float32, device="cuda")
    wf = LEPrimalWeakForm(sp)
    wf.functions = {"lambda": lam, "mu": mu, "rhs": [1.0, 1.0, 1.0]}
    wf.assemble(A, res)
    torch.cuda.synchronize()
    with pytest.raises(_lib.NfemError) as err:
        A.check_status(case)
    assert err.value.status == code
    _good_darcy_matches_oracle(torch.float32, 1e-5)


def test_cosserat_bad_material_rejected_on_host(cuda_lib):
    """The Cosserat material is one set of constants, checked before launch."""
    m = mesh_gen.cube(1)
    sp = product_space(m, [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False), ("u", "P", 0, 3, True),
                           ("t", "P", 0, 3, True)])
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.empty(A.n_rows, dtype=torch.float64, device="cuda")
    base = dict(lambda_s=1.0, mu_s=1.0, kappa_s=0.5, lambda_o=1.0, mu_o=1.0, kappa_o=0.5, l=1.0, rhs=None)
    for key, val, code in (("mu_s", 0.0, DOMAIN), ("l", -1.0, DOMAIN), ("kappa_o", np.nan, NONFINITE)):
        wf = LCEDualWeakForm(sp)
        wf.functions = dict(base, **{key: val})
        with pytest.raises(_lib.NfemError) as err:
            wf.assemble(A, res)
        assert err.value.status == code
    wf = LCEDualWeakForm(sp)
    wf.functions = base
    wf.assemble(A, res)
    torch.cuda.synchronize()
    A.check_status("good cosserat")
