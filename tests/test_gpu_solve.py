"""Device Krylov solve (FP32 FGMRES inside FP64 iterative refinement) vs scipy's direct solve."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla
import torch

import nfempy_gb300 as nf
from nfempy_gb300.solvers import KrylovSolver
from oracle import mesh_gen
from tests.gpu_helpers import darcy_oracle, product_space

pytestmark = pytest.mark.gpu
PI = np.pi
DARCY = [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)]


def assembled(m, kappa, rhs):
    sp = product_space(m, DARCY)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.empty(A.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": rhs}
    wf.assemble(A, res)
    torch.cuda.synchronize()
    return sp, A, res


def test_spmv_matches_scipy(cuda_lib):
    m = mesh_gen.cube(6)
    sp, A, res = assembled(m, 1.0, 1.0)
    As = A.to_scipy()
    x = torch.randn(A.n_rows, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    nf._lib.call("nfem_spmv", 0, A.n_rows, nf._lib.ptr(A.row_ptr), nf._lib.ptr(A.col_idx), nf._lib.ptr(A.values),
                 nf._lib.ptr(x), nf._lib.ptr(y), nf._lib.stream_ptr())
    np.testing.assert_allclose(y.cpu().numpy(), As @ x.cpu().numpy(), rtol=1e-12, atol=1e-12)
    v32 = A.values.float()
    x32 = x.float()
    y32 = torch.empty_like(x32)
    nf._lib.call("nfem_spmv", 1, A.n_rows, nf._lib.ptr(A.row_ptr), nf._lib.ptr(A.col_idx), nf._lib.ptr(v32),
                 nf._lib.ptr(x32), nf._lib.ptr(y32), nf._lib.stream_ptr())
    ref = As @ x32.double().cpu().numpy()
    assert np.abs(y32.double().cpu().numpy() - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("pc", ["cell_block", "jacobi_fails", "none_fails"])
def test_darcy_2d_solve_matches_direct(cuda_lib, pc):
    """cfg1: 2-D mixed Darcy 32x32, K = 1, manufactured f; the solution of the
    device solve matches SuperLU's to the residual tolerance."""
    f = lambda x, y, z: np.array([2 * PI ** 2 * np.sin(PI * x) * np.sin(PI * y)])
    m = mesh_gen.square(32)
    sp, A, res = assembled(m, 1.0, f)
    b = -res
    kind = pc if pc == "cell_block" else pc.split("_")[0]
    if pc != "cell_block":
        # the saddle-point matrix has a zero pressure diagonal: point Jacobi is undefined
        if kind == "jacobi":
            with pytest.raises(nf._lib.NfemError):
                KrylovSolver(A, pc="jacobi").setup()
        return
    ksp = KrylovSolver(A, pc=kind, restart=30)
    x, info = ksp.solve(b, rtol=1e-10)
    assert info.final_relres <= 1e-10 and info.status == 0
    As = A.to_scipy()
    xd = spla.spsolve(As.tocsc(), b.cpu().numpy())
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xd) / np.linalg.norm(xd) < 1e-7
    r = ksp.residual(x, b)
    assert float(r.norm() / b.norm()) <= 1e-10


def test_darcy_3d_lognormal_solve(cuda_lib):
    m = mesh_gen.cube(8)
    T = m["blocks"][-1][1].shape[0]
    from nfempy_gb300 import meshes
    cent = m["points"][m["blocks"][-1][1]].mean(axis=1)
    kappa = np.exp(meshes.grf_log_field(cent, 0.05, 2.0, 5))
    sp, A, res = assembled(m, kappa, 1.0)
    b = -res
    ksp = KrylovSolver(A, pc="cell_block", restart=30)
    x, info = ksp.solve(b, rtol=1e-8)
    assert info.final_relres <= 1e-8
    As = A.to_scipy()
    xg = x.cpu().numpy()
    bb = b.cpu().numpy()
    assert np.linalg.norm(bb - As @ xg) / np.linalg.norm(bb) <= 1e-8
    # deterministic: a second solve from zero repeats the iteration count and bits
    x2, info2 = ksp.solve(b, rtol=1e-8)
    assert info2.inner_iterations == info.inner_iterations
    assert torch.equal(x, x2)


def test_not_converged_reports_status(cuda_lib):
    m = mesh_gen.cube(4)
    sp, A, res = assembled(m, 1.0, 1.0)
    ksp = KrylovSolver(A, pc="cell_block", restart=5)
    x, info = ksp.solve(-res, rtol=1e-12, max_inner=3, raise_on_failure=False)
    assert info.status == 8  # NFEM_ERR_NOT_CONVERGED
    assert info.inner_iterations <= 5


@pytest.mark.parametrize("blocks", [False, True])
def test_batched_union_two_level_solve(cuda_lib, blocks):
    """A batch of independent 2-D problems solved at once: two-level FGMRES on
    their disjoint union with aggregates inside each problem reaches 1e-8 in
    FP64, and every problem's part equals SuperLU's solve of that problem
    alone.  blocks=True stores and inverts the coarse matrix per problem."""
    import numpy as np
    from nfempy_gb300 import meshes, workloads
    from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse
    from oracle import mesh_gen, solve
    from tests.gpu_helpers import darcy_oracle, product_space
    sides = [6, 9, 12, 8]
    ms = [mesh_gen.square(n) for n in sides]
    u = meshes.union(ms)
    rng = np.random.default_rng(2)
    kap = np.exp(rng.normal(0.0, 1.0, sum(2 * n * n for n in sides)))
    sp = product_space(u, [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)])
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.empty(A.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kap, "rhs": 1.0}
    wf.assemble(A, res)
    agg, bp = workloads.batch_aggregates(sides, 3, blocks=True)
    tl = TwoLevelCoarse(A, None, cell_agg=agg, blocks=bp if blocks else None)
    assert tl.n_agg == 4 * 9 and tl.n_blocks == (4 if blocks else 0)
    ksp = KrylovSolver(A, pc="two_level", two_level=tl)
    x, info = ksp.solve(-res, rtol=1e-8, max_inner=5000)
    assert info.status == 0 and info.final_relres <= 1e-8
    xg = x.cpu().numpy()
    _, _, cd, nd, _ = darcy_oracle(u, kap, f_cell=np.ones(len(kap)))
    c0 = 0
    for k, n in enumerate(sides):
        Ak, rk, cdk, ndk, _ = darcy_oracle(ms[k], kap[c0:c0 + 2 * n * n], f_cell=np.ones(2 * n * n))
        xk = solve.solve_newton_step(Ak, rk)
        loc = np.empty(ndk, dtype=np.int64)
        loc[cdk.ravel()] = cd[c0:c0 + 2 * n * n].ravel()
        assert np.linalg.norm(xg[loc] - xk) <= 1e-6 * np.linalg.norm(xk)
        c0 += 2 * n * n


def test_block_coarse_matches_dense(cuda_lib):
    """The block-diagonal coarse storage is the dense coarse matrix's diagonal
    blocks: on a batch union, the block inverse equals the dense inverse's
    blocks (FP32 round-off), the dense inverse is zero off the blocks, and
    both give the same iterations and solution."""
    import numpy as np
    from nfempy_gb300 import meshes, workloads
    from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse
    from oracle import mesh_gen
    from tests.gpu_helpers import product_space
    sides = [10, 7, 13]
    u = meshes.union([mesh_gen.square(n) for n in sides])
    rng = np.random.default_rng(5)
    kap = np.exp(rng.normal(0.0, 1.0, sum(2 * n * n for n in sides)))
    sp = product_space(u, [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)])
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.empty(A.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kap, "rhs": 1.0}
    wf.assemble(A, res)
    agg, bp = workloads.batch_aggregates(sides, size=3, blocks=True)
    out = {}
    for blk in (False, True):
        tl = TwoLevelCoarse(A, None, cell_agg=agg, blocks=bp if blk else None)
        ksp = KrylovSolver(A, pc="two_level", two_level=tl)
        x, info = ksp.solve(-res, rtol=1e-8, max_inner=5000)
        assert info.status == 0 and info.final_relres <= 1e-8
        out[blk] = (tl, x, info)
    dense, blockwise = out[False][0], out[True][0]
    inv_d = dense.ac_inv.cpu().numpy()
    inv_b = blockwise.ac_inv.cpu().numpy()
    off = blockwise.blk_off.cpu().numpy()
    mask = np.zeros_like(inv_d, dtype=bool)
    for b in range(len(bp) - 1):
        s0, s1 = bp[b], bp[b + 1]
        blk = inv_b[off[b]:off[b + 1]].reshape(s1 - s0, s1 - s0)
        ref = inv_d[s0:s1, s0:s1]
        assert np.abs(blk - ref).max() <= 1e-4 * np.abs(ref).max()
        mask[s0:s1, s0:s1] = True
    assert np.abs(inv_d[~mask]).max() <= 1e-5 * np.abs(inv_d).max()
    assert abs(out[False][2].inner_iterations - out[True][2].inner_iterations) <= 2
    xd, xb = out[False][1], out[True][1]
    assert torch.linalg.norm(xd - xb) <= 1e-6 * torch.linalg.norm(xd)


def test_two_level_ap_product_and_fused_solve(cuda_lib):
    """The product A P kept by the two-level preconditioner equals the FP32
    matrix times the prolongation (scipy, FP64 products of the same FP32
    operands) to FP32 rounding, and the solve that takes A z from the
    preconditioner (one SpMV fewer per iteration) reaches 1e-8 like the one
    that does its own SpMV."""
    import scipy.sparse as sps
    from nfempy_gb300 import meshes
    from nfempy_gb300.solvers import TwoLevelCoarse
    m = mesh_gen.cube(8)
    cent = m["points"][m["blocks"][-1][1]].mean(axis=1)
    kappa = np.exp(meshes.grf_log_field(cent, 0.05, 2.0, 5))
    sp, A, res = assembled(m, kappa, 1.0)
    b = -res
    out = {}
    for fuse in (True, False):
        tl = TwoLevelCoarse(A, 2, fuse_ap=fuse)
        ksp = KrylovSolver(A, pc="two_level", restart=15, two_level=tl)
        x, info = ksp.solve(b, rtol=1e-8)
        assert info.status == 0 and info.final_relres <= 1e-8
        out[fuse] = (tl, ksp, x, info)
    tl, ksp = out[True][0], out[True][1]
    n = A.n_rows
    a32 = sps.csr_matrix((ksp.values32.cpu().numpy().astype(np.float64), A.col_idx.cpu().numpy(),
                          A.row_ptr.cpu().numpy()), shape=(n, n))
    pa = tl.p_agg.cpu().numpy().reshape(n, 2)
    pv = tl.p_val.cpu().numpy().astype(np.float64).reshape(n, 2)
    keep = pa >= 0
    rows = np.repeat(np.arange(n), 2).reshape(n, 2)[keep]
    P = sps.csr_matrix((pv[keep], (rows, pa[keep])), shape=(n, tl.n_agg))
    ref = (a32 @ P).toarray()
    ap = sps.csr_matrix((tl.ap_val.cpu().numpy()[:tl.ap_nnz].astype(np.float64),
                         tl.ap_col.cpu().numpy()[:tl.ap_nnz], tl.ap_ptr.cpu().numpy()),
                        shape=(n, tl.n_agg)).toarray()
    assert np.abs(ap - ref).max() <= 1e-6 * np.abs(ref).max()
    # the pattern holds every structural entry of A P, columns ascending per row
    cols = tl.ap_col.cpu().numpy()[:tl.ap_nnz]
    ptr = tl.ap_ptr.cpu().numpy()
    assert all(np.all(np.diff(cols[ptr[i]:ptr[i + 1]]) > 0) for i in range(0, n, 97))
    assert abs(out[True][3].inner_iterations - out[False][3].inner_iterations) <= 3


@pytest.mark.parametrize("n_c,coarse_tc", [(4, 0), (7, 0), (7, 2), (8, 0), (8, 1), (9, 0)])
def test_dense_coarse_inverse(cuda_lib, n_c, coarse_tc):
    """The stored FP32 inverse of the Galerkin coarse matrix: 64 aggregates
    (one tile) and 343 (tiles clipped at the padded edge, 128-wide trailing
    tiles straddling the pivot block) both give ||X A_c - I|| within FP32
    round-off times the conditioning.  512 and 729 aggregates take the
    trailing updates on the tensor cores (3xTF32 tcgen05 MMAs, tiles of
    128 x 256 straddling the pivot block and the padded edge); the knob
    NFEM_KNOB_COARSE_TC forces them at 343 (2) or keeps the CUDA cores at 512
    (1), and both reach the same bound."""
    from nfempy_gb300 import autotune, meshes
    from nfempy_gb300.solvers import TwoLevelCoarse
    autotune.set_knobs({"coarse_tc": coarse_tc})
    try:
        _check_dense_coarse_inverse(n_c)
    finally:
        autotune.reset_knobs()


def _check_dense_coarse_inverse(n_c):
    from nfempy_gb300 import meshes
    from nfempy_gb300.solvers import TwoLevelCoarse
    m = mesh_gen.cube(max(14, 2 * n_c))
    cent = m["points"][m["blocks"][-1][1]].mean(axis=1)
    kappa = np.exp(meshes.grf_log_field(cent, 0.1, 1.0, 3))
    sp, A, res = assembled(m, kappa, 1.0)
    tl = TwoLevelCoarse(A, n_c)
    ksp = KrylovSolver(A, pc="two_level", restart=15, two_level=tl)
    ksp.setup()
    torch.cuda.synchronize()
    Ac = tl.ac.cpu().numpy()
    X = tl.ac_inv.cpu().numpy().astype(np.float64)
    na = tl.n_agg
    assert Ac.shape == (na, na) and np.allclose(Ac, Ac.T, rtol=1e-10, atol=1e-12 * np.abs(Ac).max())
    cond = np.linalg.cond(Ac)
    err = np.abs(X @ Ac - np.eye(na)).max()
    assert err <= max(1e-4, 64 * cond * 6e-8), (err, cond)


@pytest.mark.parametrize("pc", ["cell_block", "two_level"])
def test_smoother_matrix_matches_cell_blocks(cuda_lib, pc):
    """The cell-block smoother stored in A's pattern applies the same operator
    as the cell-by-cell form (FP32 rounding), and both solves reach 1e-8 in
    a similar number of iterations."""
    from nfempy_gb300 import _lib, meshes
    from nfempy_gb300.solvers import TwoLevelCoarse
    m = mesh_gen.cube(8)
    cent = m["points"][m["blocks"][-1][1]].mean(axis=1)
    kappa = np.exp(meshes.grf_log_field(cent, 0.05, 2.0, 5))
    sp, A, res = assembled(m, kappa, 1.0)
    b = -res
    out = {}
    v = torch.randn(A.n_rows, dtype=torch.float32, device="cuda")
    for mat in (False, True):
        tl = TwoLevelCoarse(A, 2) if pc == "two_level" else None
        ksp = KrylovSolver(A, pc=pc, restart=15, two_level=tl, smoother_matrix=mat)
        ksp.setup()
        z = torch.empty_like(v)
        _lib.call("nfem_precond_apply", _lib.C.byref(ksp.pc), A.n_rows, _lib.ptr(v), _lib.ptr(z), _lib.stream_ptr())
        x, info = ksp.solve(b, rtol=1e-8, max_inner=20000)
        assert info.status == 0 and info.final_relres <= 1e-8
        out[mat] = (z, info.inner_iterations)
    z0, z1 = out[False][0], out[True][0]
    assert (z0 - z1).abs().max().item() <= 1e-5 * z0.abs().max().item()
    # restarted block-Jacobi FGMRES is sensitive to round-off in its
    # iteration count (hundreds of iterations here); the two-level one is not
    slack = out[False][1] // 4 if pc == "cell_block" else max(3, out[False][1] // 20)
    assert abs(out[False][1] - out[True][1]) <= slack


def test_recorded_schedule_replays_in_a_graph(cuda_lib):
    """A two-level solve records its launch schedule; assembly + setup +
    the replayed solve are then captured as one CUDA graph.  Each replay
    reaches the same FP64 relative residual (below 1e-8) on the device and
    the same solution as the first solve, with new coefficients between
    replays picked up by the graph (same values -> same answer)."""
    import nfempy_gb300 as nf
    from nfempy_gb300 import workloads as wl
    from nfempy_gb300.solvers import KrylovSolver, TwoLevelCoarse
    m, sp, kappa, f = wl.darcy3d(12)
    A32 = nf.CSRMatrix(sp, dtype=torch.float32)
    A64 = A32.with_dtype(torch.float64)
    r32 = torch.empty(A32.n_rows, dtype=torch.float32, device="cuda")
    r64 = torch.empty(A32.n_rows, dtype=torch.float64, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": f}
    c32, c64 = wf.coefficients(torch.float32), wf.coefficients(torch.float64)
    wf.assemble(A32, r32, coefficients=c32)
    wf.assemble(A64, r64, coefficients=c64)
    b = -r64
    tl = TwoLevelCoarse(A64, 3)
    ksp = KrylovSolver(A64, pc="two_level", A32_values=A32.values, restart=15, two_level=tl)
    x0, info0 = ksp.solve(b.clone(), record_schedule=True)
    assert info0.final_relres <= 1e-8 and ksp.schedule[0] == info0.outer_iterations
    x = torch.zeros_like(b)
    rel = torch.zeros(1, dtype=torch.float64, device="cuda")

    def step():
        wf.assemble(A32, r32, coefficients=c32)
        wf.assemble(A64, r64, coefficients=c64)
        torch.neg(r64, out=b)
        x.zero_()
        ksp.refresh()
        ksp.solve(b, x, replay=True, relres_out=rel)

    step()  # eager once (allocations of the first call happen outside the capture)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    for _ in range(3):
        x.fill_(123.0)
        g.replay()
        torch.cuda.synchronize()
        assert float(rel.item()) <= 1e-8
        assert torch.allclose(x, x0, rtol=0, atol=1e-10 * x0.abs().max().item())
