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


def assemble_gpu(m, kappa, rhs, dtype, use_chunks=False, use_records=None, use_slices=True, slice_shift=17,
                 record_quarters=None, use_streams=0):
    sp = product_space(m, DARCY)
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = torch.empty(A.n_rows, dtype=dtype, device="cuda")
    wf = nf.LaplaceDualWeakForm(sp)
    wf.use_chunks = use_chunks
    wf.use_records = use_records
    wf.use_slices = use_slices
    wf.min_slice_shift = slice_shift
    wf.use_streams = use_streams
    if record_quarters is not None:
        wf.record_quarters = record_quarters
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


@pytest.mark.parametrize("kernel", ["cell_chunks", "row_records", "row_records_unsliced", "row_one_pass"])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
@pytest.mark.parametrize("gen,n", [("square", 4), ("square", 32), ("cube", 2), ("cube", 6), ("cube", 12)])
def test_darcy_matrix_matches_oracle(cuda_lib, dtype, tol, gen, n, kernel):
    """The Darcy kernels against the oracle; cube(12) has 10,368 cells, so the
    cell-chunk kernel runs several chunks and meets neighbours outside them."""
    m = getattr(mesh_gen, gen)(n)
    T = m["blocks"][-1][1].shape[0]
    kappa = np.exp(np.sin(np.arange(T) * 0.37))
    f_cell = np.cos(np.arange(T) * 0.11)
    sp, A, res = assemble_gpu(m, kappa, f_cell, dtype, kernel == "cell_chunks", kernel.startswith("row_records"),
                              use_slices=kernel != "row_records_unsliced", slice_shift=5)
    assert (A.chunk_rows is not None) == (sp.dof_shift == 0)
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


@pytest.mark.parametrize("gen,n", [("square", 6), ("cube", 3)])
def test_darcy_dirichlet_matches_oracle(cuda_lib, gen, n):
    """LaplaceDualWeakFormBCDirichlet: residual of the boundary flux DoFs for
    p_D = 1 + x + 2y + z^2, compared with the oracle's faithful restatement
    (normal from compute_normal, basis traced from the neighbour cell)."""
    from oracle import forms, quadrature, topology
    m = getattr(mesh_gen, gen)(n)
    dim = m["dim"]
    sp = product_space(m, DARCY)
    A = nf.CSRMatrix(sp, dtype=torch.float64)
    res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
    pD = lambda x, y, z: np.array([1 + x + 2 * y + z * z])
    bc = nf.assembly.LaplaceDualWeakFormBCDirichlet(sp)
    bc.functions = {"p": pD}
    bc.assemble(A, res)
    torch.cuda.synchronize()
    rg = res.cpu().numpy()
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in DARCY])
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    qf = quadrature.make_quadrature(dim - 1, 3)
    ro = np.zeros(nd)
    occ, fverts = bc.facets()
    for o, fv in zip(occ, fverts):
        c, i = divmod(int(o), dim + 1)
        ro[cd[c, i]] += forms.darcy_dirichlet_facet(X[c], s[c], i, m["points"][fv], dim, qf, pD)
    assert len(occ) == (4 * n if dim == 2 else 12 * n * n)
    np.testing.assert_allclose(rg, ro, rtol=1e-12, atol=1e-13)


def test_darcy_l2_error_matches_oracle(cuda_lib):
    """Device L2 errors of a solved 2-D / 3-D Darcy problem equal the oracle's
    (src/postprocess/l2_error_post_processor.py:7-63) to 1e-12 relative."""
    from oracle import quadrature

    def p_ex(x, y, z):
        return np.sin(PI * x) * np.sin(PI * y)

    def u_ex(x, y, z):
        return np.array([-PI * np.cos(PI * x) * np.sin(PI * y), -PI * np.sin(PI * x) * np.cos(PI * y),
                         np.zeros_like(x)])

    for m in (mesh_gen.square(16), mesh_gen.cube(4)):
        dim = m["dim"]
        sp, A, res = assemble_gpu(m, 1.0, f2d, torch.float64)
        Ao, ro, cd, nd, topo = darcy_oracle(m, np.ones(sp.n_cells), f_callable=f2d)
        x = solve.solve_newton_step(Ao, ro)
        got = nf.l2_error(dim, sp, {"u": u_ex, "p": p_ex}, x)
        quad = quadrature.make_quadrature(dim, 3)
        assert len(quad[1]) == len(sp.quadrature[dim][1])
        want = solve.l2_error_darcy(m["points"][topo.cells], topo.rt1_signs(), dim, quad, cd, x, u_ex, p_ex)
        np.testing.assert_allclose(got, want, rtol=1e-12)
        if dim == 2:
            assert want[1] < 0.05 and want[0] < 0.3


def test_darcy_batched_union_matches_oracle(cuda_lib):
    """A batch of independent 2-D problems assembled in one launch over their
    disjoint union: equal to the oracle's assembly of the union (FP64, 1e-12),
    block diagonal across problems, and each problem's solution equal to the
    oracle's solve of that problem alone."""
    from nfempy_gb300 import meshes
    rng = np.random.default_rng(3)
    sides = [3, 7, 4, 9, 5, 6]
    ms = [mesh_gen.square(n) for n in sides]
    u = meshes.union(ms)
    kap = np.exp(rng.normal(0.0, 1.0, sum(2 * n * n for n in sides)))
    sp, A, res = assemble_gpu(u, kap, 1.0, torch.float64)
    Ao, ro, cd, nd, topo = darcy_oracle(u, kap, f_cell=np.ones(len(kap)))
    Ag = A.to_scipy()
    assert row_scaled_err(Ag, Ao) <= 1e-12
    rg = res.double().cpu().numpy()
    assert np.abs(rg - ro).max() <= 1e-12 * np.abs(ro).max()
    # cells of problem k own only DoFs of problem k
    owner = np.full(nd, -1)
    c0 = 0
    for k, n in enumerate(sides):
        dofs = np.unique(cd[c0:c0 + 2 * n * n])
        assert (owner[dofs] == -1).all()
        owner[dofs] = k
        c0 += 2 * n * n
    coo = Ag.tocoo()
    assert (owner[coo.row] == owner[coo.col]).all()
    x = solve.solve_newton_step(Ag, rg)
    c0 = 0
    for k, n in enumerate(sides):
        Ak, rk, cdk, ndk, _ = darcy_oracle(ms[k], kap[c0:c0 + 2 * n * n], f_cell=np.ones(2 * n * n))
        xk = solve.solve_newton_step(Ak, rk)
        # the union numbers problem k's DoFs in the same relative order
        glob = np.unique(cd[c0:c0 + 2 * n * n])
        loc = np.empty(ndk, dtype=np.int64)
        loc[cdk.ravel()] = cd[c0:c0 + 2 * n * n].ravel()
        np.testing.assert_allclose(x[loc], xk, rtol=1e-9, atol=1e-12 * np.abs(xk).max())
        assert len(glob) == ndk
        c0 += 2 * n * n


def test_darcy_chunk_table_and_kernels_agree(cuda_lib):
    """The chunk row table against a host recomputation, and the two kernels'
    FP32 values against each other on a 16^3 x 6 mesh with a random field."""
    m = mesh_gen.cube(16)
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(11)
    kappa = np.exp(rng.normal(0.0, 2.0, T))
    f_cell = rng.normal(0.0, 1.0, T)
    sp, A, res = assemble_gpu(m, kappa, f_cell, torch.float32, True)
    pairs = A.pairs.cpu().numpy()
    p_base = sp.field_offsets["p"]
    first_cell = pairs[:p_base, 0] // sp.n_loc
    K = nf._lib.DARCY_CHUNK_CELLS
    want = np.searchsorted(first_cell, np.arange(0, -(-T // K) + 1) * K, side="left")
    np.testing.assert_array_equal(A.chunk_rows.cpu().numpy(), want)
    A_chunks = A.to_scipy()
    r_chunks = res.clone()
    wf = nf.LaplaceDualWeakForm(sp)
    wf.use_chunks = False
    wf.functions = {"kappa": kappa, "rhs": f_cell}
    wf.assemble(A, res)
    torch.cuda.synchronize()
    # entries that cancel to round-off are compared at the scale of their row
    assert row_scaled_err(A_chunks, A.to_scipy()) <= 2e-6
    assert ((r_chunks - res).abs().max() / res.abs().max()).item() <= 2e-6


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("gen,n,qpoint", [("square", 24, False), ("cube", 10, False), ("cube", 6, True)])
def test_darcy_records_equal_one_pass(cuda_lib, dtype, gen, n, qpoint):
    """The two-pass form (cell records, then rows) writes the single pass's
    values and residual up to the last bits: the FP32 records hold the same
    intermediate quantities and the row pass applies element_row's
    expressions (the compiler may still fuse a multiply-add differently).
    FP64 tetrahedra form their records in double-float arithmetic (about 48
    significant bits, df64.cuh) against the one pass's FP64: 1e-13."""
    m = getattr(mesh_gen, gen)(n)
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(4)
    kappa = np.exp(rng.normal(0.0, 2.0, T))
    rhs = f2d if qpoint else rng.normal(0.0, 1.0, T)
    sp, A1, r1 = assemble_gpu(m, kappa, rhs, dtype, use_records=False)
    _, A2, r2 = assemble_gpu(m, kappa, rhs, dtype, use_records=True)
    tol = 1e-6 if dtype == torch.float32 else (1e-13 if gen == "cube" else 1e-14)
    assert row_scaled_err(A1.to_scipy(), A2.to_scipy()) <= tol
    assert ((r1 - r2).abs().max() / r1.abs().max()).item() <= tol


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n,shift,quarters", [(12, 10, 1), (16, 11, 2), (16, 13, 3), (6, 17, 2)])
def test_darcy_sliced_equals_two_pass(cuda_lib, dtype, n, shift, quarters):
    """The overlapped assembly (cell slices of 2^shift cells, records in a
    ring of three slices, cell pass and row pass in the same launches) writes
    exactly the values and residual of the two-pass assembly: the same
    record and row arithmetic, only scheduled differently.  The sizes give
    1 to 15 slices, so the ring wraps several times."""
    m = mesh_gen.cube(n)
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(n + shift)
    kappa = np.exp(rng.normal(0.0, 2.0, T))
    f_cell = rng.normal(0.0, 1.0, T)
    sp, A1, r1 = assemble_gpu(m, kappa, f_cell, dtype, use_records=True, use_slices=False)
    _, A2, r2 = assemble_gpu(m, kappa, f_cell, dtype, use_records=True, use_slices=True, slice_shift=shift,
                             record_quarters=quarters)
    A2.check_status("sliced")
    assert A2.lookahead_cells < 2 ** shift
    assert torch.equal(A1.values, A2.values)
    assert torch.equal(r1, r2)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n,K", [(3, 1), (6, 4), (10, 7), (12, 16)])
def test_darcy_two_streams_equal_two_pass(cuda_lib, dtype, n, K):
    """The two passes over K cell slices on two streams (records of slice k
    on one stream, rows of slice k on the other once the records its rows
    need are done) write exactly the values and residual of the two passes
    in turn."""
    m = mesh_gen.cube(n)
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(n + K)
    kappa = np.exp(rng.normal(0.0, 2.0, T))
    f_cell = rng.normal(0.0, 1.0, T)
    sp, A1, r1 = assemble_gpu(m, kappa, f_cell, dtype, use_records=True, use_slices=False)
    _, A2, r2 = assemble_gpu(m, kappa, f_cell, dtype, use_records=True, use_slices=False, use_streams=K)
    A2.check_status("two streams")
    assert torch.equal(A1.values, A2.values)
    assert torch.equal(r1, r2)


def test_autotune_keeps_values(cuda_lib, tmp_path, monkeypatch):
    """The autotuner times the Darcy forms and launch shapes on a small mesh,
    applies and caches the fastest; the tuned assembly writes the values of
    the default one (FP32: to rounding, the forms differ in fusion)."""
    from nfempy_gb300 import autotune
    monkeypatch.setenv("NFEM_TUNING_CACHE", str(tmp_path / "t.json"))
    m = mesh_gen.cube(10)
    T = m["blocks"][-1][1].shape[0]
    kappa = np.exp(np.sin(np.arange(T)))
    sp, A, res = assemble_gpu(m, kappa, 1.0, torch.float32)
    ref = A.values.clone()
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"kappa": kappa, "rhs": 1.0}
    key = autotune.darcy_key(sp, torch.float32)
    try:
        best, ms, times = autotune.tune(key, lambda: wf.assemble(A, res), autotune.darcy_candidates(3), form=wf,
                                        reps=2)
        assert len(times) == len(autotune.darcy_candidates(3)) and ms > 0
        wf.assemble(A, res)
        torch.cuda.synchronize()
        A.check_status("tuned")
        assert ((A.values - ref).abs().max() / ref.abs().max()).item() <= 2e-6
        assert autotune.apply_cached(key, wf)["config"] == best
    finally:
        autotune.reset_knobs()


def _lattice_meshes():
    """Meshes for the FP64 lattice records: a dyadic cube (every cell a
    lattice cell), the same cube scaled by 3 and moved by (0.5, -2, 1.25)
    (still dyadic), a cube with a third of its vertices moved by
    non-dyadic amounts (lattice and double-float cells side by side) and
    cube(6) (coordinates k/6: no lattice cell)."""
    m16 = mesh_gen.cube(16)
    moved = dict(m16, points=m16["points"] * 3.0 + np.array([0.5, -2.0, 1.25]))
    m8 = mesh_gen.cube(8)
    rng = np.random.default_rng(8)
    pts = m8["points"].copy()
    pick = rng.random(len(pts)) < 0.33
    pts[pick] += rng.uniform(-0.03, 0.03, (int(pick.sum()), 3))
    return {"cube16": m16, "moved16": moved, "mixed8": dict(m8, points=pts), "cube6": mesh_gen.cube(6)}


@pytest.mark.parametrize("name", ["cube16", "moved16", "mixed8", "cube6"])
@pytest.mark.parametrize("qpoint", [False, True])
def test_darcy_f64_lattice_records(cuda_lib, name, qpoint):
    """FP64 tetrahedra on lattice cells take exact integer records (G, det
    and the T120 combinations in integers, one rounded factor 1/(30 kappa
    |det|)): against the FP64 oracle within 1e-12 row-scaled, and against the
    double-float records of every cell (knob NFEM_KNOB_DARCY_F64_RECORDS = 1)
    within 1e-13, the double-float path's own accuracy."""
    from nfempy_gb300 import autotune
    m = _lattice_meshes()[name]
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(T)
    kappa = np.exp(rng.normal(0.0, 2.0, T))
    f_cell = rng.normal(0.0, 1.0, T)
    rhs = f2d if qpoint else f_cell
    sp, A, res = assemble_gpu(m, kappa, rhs, torch.float64, use_records=True, use_slices=False)
    A.check_status(name)
    autotune.set_knobs({"darcy_f64_records": 1})
    try:
        _, A_df, res_df = assemble_gpu(m, kappa, rhs, torch.float64, use_records=True, use_slices=False)
    finally:
        autotune.reset_knobs()
    Ao, ro, *_ = darcy_oracle(m, kappa, f_callable=f2d) if qpoint else darcy_oracle(m, kappa, f_cell=f_cell)
    Ag = A.to_scipy()
    np.testing.assert_array_equal(Ag.indptr, Ao.indptr)
    np.testing.assert_array_equal(Ag.indices, Ao.indices)
    assert row_scaled_err(Ag, Ao) <= 1e-12
    rg = res.cpu().numpy()
    assert np.abs(rg - ro).max() <= 1e-12 * np.abs(ro).max()
    assert row_scaled_err(A.to_scipy(), A_df.to_scipy()) <= 1e-13
    assert ((res - res_df).abs().max() / res_df.abs().max()).item() <= 1e-13
    if name == "cube6":  # no lattice cell: the same double-float records
        assert torch.equal(A.values, A_df.values)


@pytest.mark.parametrize("name", ["cube16", "moved16", "mixed8", "cube6"])
@pytest.mark.parametrize("qpoint,accumulate,lead", [(False, False, 0), (True, False, 0), (False, True, 0),
                                                    (False, False, 1), (False, False, 3)])
def test_darcy_fused_equals_two_pass(cuda_lib, name, qpoint, accumulate, lead):
    """The fused FP64 assembly (one persistent launch, record chunks and row
    chunks from a plan, row chunks waiting on their record chunks' flags)
    writes bitwise the values and residual of the two passes in turn: the
    same record and row arithmetic, only scheduled differently.  A lead of 1
    or 3 record chunks makes the row chunks wait on records still being
    formed."""
    m = _lattice_meshes()[name]
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(T + 1)
    kappa = np.exp(rng.normal(0.0, 2.0, T))
    f_cell = rng.normal(0.0, 1.0, T)
    rhs = f2d if qpoint else f_cell
    sp = product_space(m, DARCY)
    out = []
    for fused in (False, True):
        A = nf.CSRMatrix(sp, dtype=torch.float64)
        res = torch.zeros(A.n_rows, dtype=torch.float64, device="cuda")
        wf = nf.LaplaceDualWeakForm(sp)
        wf.use_records = True
        wf.use_fused = fused
        wf.fused_lead = lead
        wf.functions = {"kappa": kappa, "rhs": rhs}
        wf.assemble(A, res)
        if accumulate:  # a second pass adds the same element data again
            wf.assemble(A, res, accumulate=True)
        torch.cuda.synchronize()
        A.check_status(f"fused={fused}")
        out.append((A.values.clone(), res.clone()))
    assert torch.equal(out[0][0], out[1][0])
    assert torch.equal(out[0][1], out[1][1])


def _badly_shaped(gen, n, flat):
    """A mesh of flat cells in general orientation: cube(n) squeezed by
    `flat` along z and rotated (tetrahedra of shape quality ~ flat), or
    square(n) squeezed along y and turned in its plane (triangles with
    angles ~ flat)."""
    m = getattr(mesh_gen, gen)(n)
    pts = m["points"].copy()
    if gen == "cube":
        pts[:, 2] *= flat
        a, b, c = 0.3, 0.7, 1.1
        Rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
        Ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
        Rz = np.array([[np.cos(c), -np.sin(c), 0], [np.sin(c), np.cos(c), 0], [0, 0, 1]])
        pts = pts @ (Rz @ Ry @ Rx).T
    else:
        pts[:, 1] *= flat
        t = 0.6
        xy = pts[:, :2] @ np.array([[np.cos(t), -np.sin(t)], [np.sin(t), np.cos(t)]]).T
        pts = np.column_stack([xy, pts[:, 2]])
    return dict(m, points=pts)


@pytest.mark.parametrize("gen,n,flat", [("cube", 3, 1 / 512), ("cube", 4, 1 / 4096), ("square", 6, 1 / 512)])
@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-5)])
def test_darcy_badly_shaped_cells(cuda_lib, gen, n, flat, dtype, tol):
    """Flat cells in general orientation (shape quality q ~ 1e-3 .. 1e-4),
    where |det J| carries a few ulps / q of the arithmetic it is formed in:
    the FP32 cell pass leaves such cells to the follow-up launch, which
    takes |det J| in FP64 from the points; the FP64 records take it in
    hardware FP64 instead of double-float.  Against the FP64 oracle at the
    usual tolerance, except that FP64 is held to max(1e-12, 10 ulp / q_min):
    the oracle's own |det J| (QR, FP64) is only that accurate there."""
    m = _badly_shaped(gen, n, flat)
    X = m["points"][m["blocks"][-1][1]]
    E = X[:, 1:] - X[:, :1]
    if gen == "cube":
        q = np.abs(np.linalg.det(E)) / np.prod(np.linalg.norm(E, axis=2), axis=1)
    else:
        q = np.linalg.norm(np.cross(E[:, 0], E[:, 1]), axis=1) / np.prod(np.linalg.norm(E, axis=2), axis=1)
    if dtype == torch.float64:
        tol = max(tol, 10 * 2.0 ** -53 / q.min())
    T = m["blocks"][-1][1].shape[0]
    rng = np.random.default_rng(T + 7)
    kappa = np.exp(rng.normal(0.0, 1.0, T))
    f_cell = rng.normal(0.0, 1.0, T)
    sp, A, res = assemble_gpu(m, kappa, f_cell, dtype, use_slices=False)
    A.check_status("badly shaped")
    Ao, ro, *_ = darcy_oracle(m, kappa, f_cell=f_cell)
    Ag = A.to_scipy()
    np.testing.assert_array_equal(Ag.indptr, Ao.indptr)
    assert row_scaled_err(Ag, Ao) <= tol
    rg = res.double().cpu().numpy()
    assert np.abs(rg - ro).max() <= tol * np.abs(ro).max()
