"""Mixed Cosserat assembly on the GPU vs the FP64 oracle (oracle/forms.cosserat_element).

Tolerances: FP64 within 1e-12, FP32 within 1e-5, relative to each row's
largest entry; the pattern and DoF map are checked bit-exact."""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from nfempy_gb300.assembly import LCEDualWeakForm
from oracle import assembly, forms, mesh_gen, quadrature, topology
from tests.cases import golden
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu
FIELDS = [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False), ("u", "P", 0, 3, True), ("t", "P", 0, 3, True)]
PAR = dict(lambda_s=1.0, mu_s=1.0, kappa_s=0.5, lambda_o=1.0, mu_o=1.0, kappa_o=0.5, l=0.7)


def row_scaled_err(Ag, Ao):
    d = (Ag - Ao).tocsr()
    scale = np.maximum(abs(Ao).max(axis=1).toarray().ravel(), 1e-300)
    return (abs(d).max(axis=1).toarray().ravel() / scale).max()


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("n", [1, 3])
def test_cosserat_matches_oracle(cuda_lib, dtype, tol, n):
    m = mesh_gen.cube(n)
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
