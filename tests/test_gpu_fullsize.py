"""Parity at the benchmarked sizes: every workload that bench.py times is
assembled here at its full size through the public API and checked against
the FP64 oracle.

  * the DoF map of every cell bit-exact against the oracle's own numbering
    (oracle/topology.py, an independent restatement of the reference's mesh
    and DoF-map code);
  * a seeded sample of >= 10,000 rows (plus the first and last rows of each
    field): their pattern bit-exact and their values within 1e-12 (FP64) or
    1e-5 (FP32) of the row's largest oracle entry, the oracle rows summed from
    the element matrices of the incident cells only;
  * the residual entries of the same rows, within the same bars of the
    largest residual entry.

The FP32 kernels form edge vectors from 16-byte fixed-point point records;
their error bound grows with the cells across the mesh, which these tests
cover at the sizes the bench runs.
"""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from nfempy_gb300 import workloads as wl
from oracle import forms, mesh_gen, quadrature, topology
from tests.gpu_helpers import compare_rows, gpu_rows, oracle_rows, quadrature_xq, sample_rows

pytestmark = pytest.mark.gpu
N_SAMPLE = 10000
DARCY_FIELDS = [topology.FieldSpec("u", "RT", 1), topology.FieldSpec("p", "P", 0, 1, True)]


def _same_mesh(m_product, m_oracle):
    np.testing.assert_array_equal(m_product["points"], m_oracle["points"])
    assert len(m_product["blocks"]) == len(m_oracle["blocks"])
    for (t1, c1, p1), (t2, c2, p2) in zip(m_product["blocks"], m_oracle["blocks"]):
        assert t1 == t2
        np.testing.assert_array_equal(c1, c2)
        np.testing.assert_array_equal(p1, p2)


def _residual_check(rg, ro, tol, scale):
    assert np.abs(rg - ro).max() <= tol * scale, (np.abs(rg - ro).max(), scale)


@pytest.fixture(scope="module")
def darcy64():
    m, sp, kappa, f = wl.darcy3d(64)
    mo = mesh_gen.cube(64)
    _same_mesh(m, mo)
    topo = topology.Topology(mo)
    cd, nd = topology.cell_dofs(topo, DARCY_FIELDS)
    return m, sp, kappa, f, topo, cd, nd


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_darcy_cube64_full_size(cuda_lib, darcy64, dtype, tol):
    """64^3 x 6 tets (1,572,864 cells, 4,743,168 DoF), the headline workload:
    lognormal GRF kappa (sigma 2), f = 1."""
    m, sp, kappa, f, topo, cd, nd = darcy64
    assert nd == sp.n_dof == 4743168
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
    A = nf.CSRMatrix(sp, dtype=dtype)
    assert A.nnz == 36200448
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": f}
    wf.assemble(A, res)
    torch.cuda.synchronize()
    A.check_status("darcy 64^3")
    p_base = sp.field_offsets["p"]
    rows = sample_rows(nd, N_SAMPLE, 64, extra=[0, p_base - 1, p_base, nd - 1])
    X = mo_points = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(3, 3)
    Q = len(quad[1])

    def elem(cells):
        kq = np.repeat(kappa[cells, None], Q, 1)
        fq = np.repeat(f[cells, None], Q, 1)
        return forms.darcy_batch(X[cells], s[cells], 3, quad, kq, fq)

    O, ro = oracle_rows(cd, nd, rows, elem)
    compare_rows(gpu_rows(A, rows), O, tol)
    rg = res[torch.as_tensor(rows, device="cuda")].double().cpu().numpy()
    # largest residual entry: a pressure row, -|det J| |T| f
    scale = np.abs(np.abs(np.linalg.det(mo_points[:, 1:] - mo_points[:, :1])) / 6.0).max()
    _residual_check(rg, ro, tol, scale)


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_elasticity_cube40_full_size(cuda_lib, dtype, tol):
    """40^3 x 6 tets (384,000 cells, 1,594,323 DoF, nnz 134,475,849), vector
    P2, per-cell lognormal Lame parameters, body force (1, 1, 1)."""
    m, sp, fn = wl.elasticity3d(40)
    mo = mesh_gen.cube(40)
    _same_mesh(m, mo)
    topo = topology.Topology(mo)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "P", 2, 3)])
    assert nd == sp.n_dof == 1594323
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
    A = nf.CSRMatrix(sp, dtype=dtype)
    assert A.nnz == 134475849
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.assembly.LEPrimalWeakForm(sp)
    wf.functions = fn
    wf.assemble(A, res)
    torch.cuda.synchronize()
    A.check_status("elasticity 40^3")
    rows = sample_rows(nd, N_SAMPLE, 40, extra=[0, 1, 2, nd - 1])
    X = m["points"][topo.cells]
    quad = quadrature.make_quadrature(3, 5)
    Q = len(quad[1])
    lam, mu = fn["lambda"], fn["mu"]

    def elem(cells):
        fq = np.ones((len(cells), Q, 3))
        return forms.elasticity_batch(X[cells], 3, quad, lam[cells], mu[cells], fq)

    O, ro = oracle_rows(cd, nd, rows, elem, chunk=8000)
    compare_rows(gpu_rows(A, rows), O, tol)
    rg = res[torch.as_tensor(rows, device="cuda")].double().cpu().numpy()
    _residual_check(rg, ro, tol, np.abs(ro).max())


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_cosserat_cube24_full_size(cuda_lib, dtype, tol):
    """24^3 x 6 tets (82,944 cells, 1,513,728 DoF, nnz 68,802,048), the
    manufactured-solution load and the material as callables (the driver's
    form of the functions dict)."""
    m, sp, fn, exact = wl.cosserat3d(24)
    mo = mesh_gen.cube(24)
    _same_mesh(m, mo)
    topo = topology.Topology(mo)
    fields = [topology.FieldSpec("s", "RT", 1, 3), topology.FieldSpec("m", "RT", 1, 3),
              topology.FieldSpec("u", "P", 0, 3, True), topology.FieldSpec("t", "P", 0, 3, True)]
    cd, nd = topology.cell_dofs(topo, fields)
    assert nd == sp.n_dof == 1513728
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
    A = nf.CSRMatrix(sp, dtype=dtype)
    assert A.nnz == 68802048
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.assembly.LCEDualWeakForm(sp)
    wf.functions = fn
    wf.assemble(A, res)
    torch.cuda.synchronize()
    A.check_status("cosserat 24^3")
    offs = [sp.field_offsets[k] for k in "smut"]
    rows = sample_rows(nd, N_SAMPLE, 24, extra=offs + [o - 1 for o in offs[1:]] + [nd - 1])
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(3, 3)
    par = wl.COSSERAT_MATERIAL

    def elem(cells):
        xq = quadrature_xq(X[cells], 3, quad[0])
        fq = np.moveaxis(fn["rhs"](xq[..., 0], xq[..., 1], xq[..., 2]), 0, -1)
        return forms.cosserat_batch(X[cells], s[cells], quad, par, fq)

    O, ro = oracle_rows(cd, nd, rows, elem, chunk=5000)
    compare_rows(gpu_rows(A, rows), O, tol)
    rg = res[torch.as_tensor(rows, device="cuda")].double().cpu().numpy()
    # residual rows: the u and t rows carry the load; bar against the largest
    _, r_all = elem(np.arange(0, topo.n_cells, 97))
    _residual_check(rg, ro, tol, np.abs(r_all).max())


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_darcy_batch512_full_size(cuda_lib, dtype, tol):
    """The 512-problem 2-D batch (n_i ~ U{8..128}, 5,835,418 triangles,
    14,656,783 DoF) assembled in one launch over the disjoint union: the
    union's DoF map bit-exact against the oracle's numbering of the union
    mesh, and sampled rows against the oracle."""
    from nfempy_gb300 import meshes
    u, sp, kappa, f, sides = wl.darcy2d_batch(512)
    mo = meshes.union([mesh_gen.square(int(n)) for n in sides])
    _same_mesh(u, mo)
    topo = topology.Topology(mo)
    cd, nd = topology.cell_dofs(topo, DARCY_FIELDS)
    assert nd == sp.n_dof
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": f}
    wf.assemble(A, res)
    torch.cuda.synchronize()
    A.check_status("batch 512")
    p_base = sp.field_offsets["p"]
    rows = sample_rows(nd, 2 * N_SAMPLE, 512, extra=[0, p_base - 1, p_base, nd - 1])
    X = u["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(2, 3)
    Q = len(quad[1])

    def elem(cells):
        kq = np.repeat(kappa[cells, None], Q, 1)
        fq = np.repeat(f[cells, None], Q, 1)
        return forms.darcy_batch(X[cells], s[cells], 2, quad, kq, fq)

    O, ro = oracle_rows(cd, nd, rows, elem)
    compare_rows(gpu_rows(A, rows), O, tol)
    rg = res[torch.as_tensor(rows, device="cuda")].double().cpu().numpy()
    area = 0.5 * np.abs(np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0])[:, 2])
    _residual_check(rg, ro, tol, area.max())
