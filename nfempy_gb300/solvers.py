"""Device Krylov solve: the step the reference drivers hand to PETSc KSP.

    A = CSRMatrix(space, torch.float64); assemble ...
    ksp = KrylovSolver(A, pc="cell_block")
    x, info = ksp.solve(b, rtol=1e-8)

A is the FP64 matrix (the residual is always measured on it, in FP64); the
solver keeps an FP32 copy with the same pattern for the inner FGMRES
iterations, refreshed from A (or assembled directly in FP32 by the caller
and passed as A32).  Preconditioners: "none", "jacobi", "cell_block"
(cell-patch block Jacobi = weighted additive Schwarz over the element
cliques, blocks inverted in FP64, applied in FP32), "two_level" (that
smoother plus a Galerkin coarse correction over aggregates of cells, see
TwoLevelCoarse).
Reference call sites: examples/md_elliptic_scalar/md_elliptic_scalar.py:343-363,
examples/cauchy_elasticity/cg_elasticity_example_1.py:159-170.
"""
import numpy as np
import torch

from . import _lib


class SolveResult:
    def __init__(self, info, seconds=None):
        self.inner_iterations = info.inner_iterations
        self.outer_iterations = info.outer_iterations
        self.initial_relres = info.initial_relres
        self.final_relres = info.final_relres
        self.status = info.status
        self.n_snapshots = info.n_snapshots
        self.seconds = seconds

    def as_dict(self):
        return {k: getattr(self, k) for k in ("inner_iterations", "outer_iterations", "initial_relres",
                                              "final_relres", "status", "seconds")}


def _csr(A, values=None):
    v = A.values if values is None else values
    vt = _lib.NFEM_F64 if v.dtype == torch.float64 else _lib.NFEM_F32
    return _lib.Csr(A.n_rows, _lib.ptr(A.row_ptr).value, _lib.ptr(A.col_idx).value, _lib.ptr(v).value, vt)


# FP32 inner tolerance per preconditioner when solve() is given none: each
# outer FP64 refinement step restarts FGMRES, and a looser inner target with
# more outer steps reached 1e-8 sooner in measured sweeps (two-level at
# 64^3 x 6: 1e-2 128 ms against 1e-4 153 ms; point Jacobi on P2 elasticity
# 40^3 x 6: 1e-2 0.76 s against 1.27 s; block Jacobi: 1e-3 8.1 s, 1e-4 8.5 s,
# 1e-2 9.5 s).
INNER_RTOL = {"two_level": 1e-2, "cell_block": 1e-3, "jacobi": 1e-2, "none": 1e-2}


class KrylovSolver:
    def __init__(self, A, pc="cell_block", A32_values=None, restart=30, weighted=True, two_level=None, graphs=True,
                 smoother_matrix=True):
        """graphs: replay each restart cycle after the first as one CUDA graph
        (False launches every kernel from the host).  smoother_matrix: store
        the cell-block smoother in A's CSR pattern (one SpMV per smoothing
        step, nnz more FP32 values) instead of applying it cell by cell."""
        if A.dtype != torch.float64:
            raise ValueError("A must be the FP64 matrix (the residual is measured in FP64)")
        self.A = A
        self.restart = int(restart)
        self.graphs = bool(graphs)
        self.smoother_matrix = bool(smoother_matrix)
        self.values32 = A32_values
        self.pc_kind = pc
        self.weighted = weighted
        self.two_level = two_level
        self._setup_done = False
        self.status = torch.zeros(1, dtype=torch.int32, device=A.values.device)

    def set_operators(self, A32_values=None):
        """Refresh the FP32 copy and the preconditioner after A changed."""
        if A32_values is not None:
            self.values32 = A32_values
        self._setup_done = False

    def setup(self, stream=None):
        A = self.A
        dev = A.values.device
        if self.values32 is None or self.values32.data_ptr() == 0:
            self.values32 = A.values.to(torch.float32)
        if self.values32.dtype != torch.float32 or self.values32.numel() < A.nnz:
            raise ValueError("A32_values must be the FP32 values of A's pattern")
        st = _lib.stream_ptr(stream)
        sp = A.space
        if self.pc_kind == "none":
            self.pc = _lib.Precond(_lib.PC_NONE, 0, 0, None, None, None, None, None, None, None, None)
        elif self.pc_kind == "jacobi":
            self.diag_inv = torch.empty(A.n_rows, dtype=torch.float32, device=dev)
            self.pc = _lib.Precond(_lib.PC_JACOBI, 0, 0, None, None, None, None, _lib.ptr(self.diag_inv).value,
                                   None, None, None)
        elif self.pc_kind in ("cell_block", "two_level"):
            n_loc = sp.n_loc
            if not 4 <= n_loc <= 32 or (self.pc_kind == "two_level" and n_loc not in (4, 5)):
                raise NotImplementedError("cell_block for 4 to 32 local DoFs per cell; two_level for mixed Darcy")
            self.block_inv = torch.empty((sp.n_cells, n_loc, n_loc), dtype=torch.float32, device=dev)
            kind = _lib.PC_CELL_BLOCK if self.pc_kind == "cell_block" else _lib.PC_TWO_LEVEL
            self.pc = _lib.Precond(kind, n_loc, sp.n_cells, _lib.ptr(sp.cell_dofs).value,
                                   _lib.ptr(A.inc_ptr).value, _lib.ptr(A.inc).value,
                                   _lib.ptr(self.block_inv).value, None, None, None, None)
            if self.smoother_matrix:
                self.smoother_vals = torch.empty(max(1, A.nnz), dtype=torch.float32, device=dev)
                self._smoother = _csr(A, self.smoother_vals)
                self.pc.smoother = _lib.C.pointer(self._smoother)
            if self.pc_kind == "two_level":
                if self.two_level is None:
                    raise ValueError("pc='two_level' needs two_level=TwoLevelCoarse(...)")
                self._a32 = _csr(A, self.values32)
                self.pc.two_level = _lib.C.pointer(self.two_level.struct)
                self.pc.a32 = _lib.C.pointer(self._a32)
        else:
            raise ValueError(f"unknown preconditioner {self.pc_kind}")
        if self.weighted:
            self.wsqrt = torch.empty(A.n_rows, dtype=torch.float32, device=dev)
            self.winvsqrt = torch.empty(A.n_rows, dtype=torch.float32, device=dev)
            # kept with the solver: every preconditioner setup writes it
            self._setup_scratch = torch.empty(2 * A.n_rows, dtype=torch.float64, device=dev)
            self.pc.wsqrt = _lib.ptr(self.wsqrt).value
            self.pc.winvsqrt = _lib.ptr(self.winvsqrt).value
            self.pc.setup_scratch = _lib.ptr(self._setup_scratch).value
        a64 = _csr(A)
        _lib.call("nfem_precond_setup", _lib.C.byref(self.pc), _lib.C.byref(a64), _lib.ptr(self.status), st)
        ws_b = _lib.C.c_size_t(0)
        _lib.call("nfem_solve_workspace_bytes", A.n_rows, self.restart, _lib.C.byref(ws_b))
        self.ws = torch.empty(int(ws_b.value), dtype=torch.uint8, device=dev)
        self._setup_done = True
        if int(self.status.item()):
            s = int(self.status.item())
            self.status.zero_()
            raise _lib.NfemError(s, "preconditioner setup")

    def refresh(self, stream=None):
        """Preconditioner setup again for new values of A (and of the FP32
        copy), in place: no allocation and no host synchronisation, so it can
        be captured in a CUDA graph.  setup() must have run once."""
        if not self._setup_done:
            raise RuntimeError("refresh() needs a first setup()")
        a64 = _csr(self.A)
        _lib.call("nfem_precond_setup", _lib.C.byref(self.pc), _lib.C.byref(a64), _lib.ptr(self.status),
                  _lib.stream_ptr(stream))

    def solve(self, b, x=None, rtol=1e-8, inner_rtol=None, max_inner=100000, max_outer=20, stream=None,
              raise_on_failure=True, snapshots=None, record_schedule=False, replay=False, relres_out=None):
        """Solve A x = b (FP64 device tensors) to ||b - A x|| / ||b|| <= rtol.

        inner_rtol: reduction of the weighted residual each FP32 inner solve
        aims for (None: the preconditioner's entry of INNER_RTOL).

        snapshots: optional FP32 tensor [S, n] that receives the iterate after
        each restart cycle (res.n_snapshots of them).

        record_schedule: keep the launch schedule this solve took
        (self.schedule).  replay: launch that schedule again with no host
        synchronisation (capturable in a CUDA graph); relres_out, a device
        double, receives the final FP64 relative residual, which the caller
        checks: x is a solution only where it is <= rtol."""
        if not self._setup_done:
            self.setup(stream)
        A = self.A
        if x is None:
            x = torch.zeros(A.n_rows, dtype=torch.float64, device=b.device)
        if inner_rtol is None:
            inner_rtol = INNER_RTOL.get(self.pc_kind, 1e-4)
        prm = _lib.SolveParams(float(rtol), float(inner_rtol), self.restart, int(max_inner), int(max_outer))
        prm.no_graphs = 0 if self.graphs else 1
        if record_schedule:
            self.schedule = np.full(1 << 14, -1, dtype=np.int32)
            prm.schedule = self.schedule.ctypes.data
            prm.schedule_capacity = self.schedule.size
            prm.schedule_mode = 1
        if replay:
            if getattr(self, "schedule", None) is None or self.schedule[0] < 0 or relres_out is None:
                raise ValueError("replay needs a recorded schedule and relres_out")
            prm.schedule = self.schedule.ctypes.data
            prm.schedule_capacity = self.schedule.size
            prm.schedule_mode = 2
            prm.relres_out = _lib.ptr(relres_out).value
        if snapshots is not None:
            prm.snapshots = _lib.ptr(snapshots).value
            prm.max_snapshots = int(snapshots.shape[0])
        info = _lib.SolveInfo()
        a64 = _csr(A)
        a32 = _csr(A, self.values32)
        rc = _lib.lib().nfem_solve_ir_fgmres(_lib.C.byref(a64), _lib.C.byref(a32), _lib.C.byref(self.pc),
                                              _lib.ptr(b), _lib.ptr(x), _lib.C.byref(prm), _lib.ptr(self.ws),
                                              self.ws.numel(), _lib.C.byref(info), _lib.stream_ptr(stream))
        res = SolveResult(info)
        if rc != 0 and raise_on_failure:
            raise _lib.NfemError(rc, f"solve ({res.as_dict()})")
        return x, res

    def residual(self, x, b, stream=None):
        r = torch.empty_like(b)
        A = self.A
        _lib.call("nfem_residual_f64", A.n_rows, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), _lib.ptr(A.values),
                  _lib.ptr(x), _lib.ptr(b), _lib.ptr(r), _lib.stream_ptr(stream))
        return r


class CGSolver:
    """Conjugate gradients for symmetric positive definite systems (the P2
    elasticity driver's PETSc CG, cg_elasticity_example_1.py:159-170): FP32
    CG on the FP32 copy of A inside FP64 iterative refinement on A, with
    point Jacobi (pc="jacobi") or the inverses of the 3 x 3 diagonal node
    blocks of a vector field (pc="node_block", DoF = 3 node + component) in
    place of the driver's incomplete Cholesky."""

    def __init__(self, A, pc="node_block", A32_values=None):
        if A.dtype != torch.float64:
            raise ValueError("A must be the FP64 matrix (the residual is measured in FP64)")
        if pc not in ("jacobi", "node_block"):
            raise ValueError(f"unknown preconditioner {pc}")
        self.A = A
        self.pc_kind = pc
        self.values32 = A32_values
        self.status = torch.zeros(1, dtype=torch.int32, device=A.values.device)
        self._setup_done = False

    def setup(self, stream=None):
        A = self.A
        dev = A.values.device
        if self.values32 is None:
            self.values32 = A.values.to(torch.float32)
        if self.values32.dtype != torch.float32 or self.values32.numel() < A.nnz:
            raise ValueError("A32_values must be the FP32 values of A's pattern")
        kind = _lib.PC_JACOBI if self.pc_kind == "jacobi" else _lib.PC_NODE_BLOCK
        if kind == _lib.PC_NODE_BLOCK and A.n_rows % 3:
            raise NotImplementedError("node blocks need 3 DoFs per node")
        self.inv = torch.empty(A.n_rows * (1 if kind == _lib.PC_JACOBI else 3), dtype=torch.float32, device=dev)
        a64 = _csr(A)
        _lib.call("nfem_pcg_setup", kind, _lib.C.byref(a64), _lib.ptr(self.inv), _lib.ptr(self.status),
                  _lib.stream_ptr(stream))
        wsb = _lib.C.c_size_t(0)
        _lib.call("nfem_pcg_workspace_bytes", A.n_rows, _lib.C.byref(wsb))
        self.ws = torch.empty(int(wsb.value), dtype=torch.uint8, device=dev)
        self._kind = kind
        self._setup_done = True
        s = int(self.status.item())
        if s:
            self.status.zero_()
            raise _lib.NfemError(s, "CG preconditioner setup")

    def solve(self, b, rtol=1e-8, inner_rtol=1e-3, max_inner=20000, max_outer=50, x=None, stream=None,
              raise_on_failure=True):
        if not self._setup_done:
            self.setup(stream)
        A = self.A
        b = b.to(torch.float64).contiguous()
        x = torch.zeros_like(b) if x is None else x
        info = _lib.SolveInfo()
        a64 = _csr(A)
        a32 = _csr(A, self.values32)
        rc = _lib.lib().nfem_solve_ir_pcg(_lib.C.byref(a64), _lib.C.byref(a32), self._kind, _lib.ptr(self.inv),
                                           _lib.ptr(b), _lib.ptr(x), float(rtol), float(inner_rtol), int(max_inner),
                                           int(max_outer), _lib.ptr(self.ws), self.ws.numel(), _lib.C.byref(info),
                                           _lib.ptr(self.status), _lib.stream_ptr(stream))
        res = SolveResult(info)
        if rc != 0:
            self.status.zero_()
            if raise_on_failure:
                raise _lib.NfemError(rc, f"CG solve ({res.as_dict()})")
        return x, res

    def residual(self, x, b, stream=None):
        r = torch.empty_like(b)
        A = self.A
        _lib.call("nfem_residual_f64", A.n_rows, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), _lib.ptr(A.values),
                  _lib.ptr(x), _lib.ptr(b), _lib.ptr(r), _lib.stream_ptr(stream))
        return r


class TwoLevelCoarse:
    """Aggregates and prolongation structure of the two-level preconditioner.

    Cells are binned by centroid into an n_c^d grid of aggregates.  P maps an
    aggregate value to the pressure DoFs of its cells (weight 1) and to the
    flux rows whose cells lie in different aggregates or on the domain
    boundary (weight -w_f times the row's entries in that aggregate's
    pressure columns).  w = None gives the classical weights 1/|a_ff|; the
    learned preconditioner passes the network's prediction."""

    def __init__(self, A, n_c, w=None, cell_agg=None, blocks=None, fuse_ap=True, post_smooth=True, omega=0.9):
        """cell_agg: optional aggregate of every cell (0 .. n_agg - 1) in place
        of the centroid grid, e.g. per-problem grids for a batch of
        independent problems assembled as one disjoint union.

        blocks: optional [n_blocks + 1] ascending aggregate offsets when the
        aggregates of block b (blocks[b] .. blocks[b + 1] - 1) couple to no
        other block -- the problems of such a batch.  The coarse matrix is then
        stored, inverted and applied block by block (sum of s_b^2 entries in
        place of n_agg^2), which admits many more aggregates.

        fuse_ap: keep the product A P (its pattern is built here, its values
        in every preconditioner setup), so that the preconditioner hands back
        A z with z and the solver saves one SpMV per iteration.

        post_smooth, omega: a damped smoother (z = omega B v) and, with
        post_smooth, a second smoothing step after the coarse correction.
        Measured at 64^3 x 6 (restart 15, inner 1e-2): pre-smoothing only,
        omega 1: 175 iterations, 80 ms; symmetric cycle, omega 0.9: 103
        iterations, 67 ms (omega 1 does not converge with post-smoothing);
        the 512-problem batch: 168 -> 65 iterations, 196 -> 107 ms."""
        sp = A.space
        self.A = A
        dim = sp.dim
        dev = A.values.device
        # the aggregate structure is built on the device: sorts, scans and
        # scatters over the cells and rows, no host round trip of the mesh
        if cell_agg is not None:
            agg = torch.as_tensor(np.asarray(cell_agg) if not torch.is_tensor(cell_agg) else cell_agg,
                                  device=dev).long()
            if agg.shape != (sp.n_cells,) or int(agg.min().item()) < 0:
                raise ValueError("cell_agg needs one aggregate index >= 0 per cell")
            self.n_agg = int(agg.max().item()) + 1
        else:
            cent = sp.points[sp.cells.long()].mean(dim=1)[:, :dim]
            lo, hi = cent.min(dim=0).values, cent.max(dim=0).values
            idx = ((cent - lo) / (hi - lo).clamp_min(1e-300) * n_c).floor().long().clamp_(0, n_c - 1)
            agg = torch.zeros(sp.n_cells, dtype=torch.int64, device=dev)
            for d in range(dim):
                agg = agg * n_c + idx[:, d]
            self.n_agg = int(n_c ** dim)
        counts = torch.bincount(agg, minlength=self.n_agg)
        if bool((counts == 0).any().item()):
            raise ValueError("empty aggregate: choose a coarser grid")
        self._agg = agg
        self._counts = counts
        n = A.n_rows
        pb = sp.field_offsets["p"]
        self.p_base = pb
        nf = sp.dim + 1
        p_agg = torch.full((n, 2), -1, dtype=torch.int64, device=dev)
        p_agg[pb:pb + sp.n_cells, 0] = agg
        # flux rows: aggregates of the cells on either side of the face
        faces = sp.cell_dofs[:, :nf].reshape(-1).long()
        fagg = agg.repeat_interleave(nf)
        order = torch.sort(faces * self.n_agg + fagg).indices
        faces, fagg = faces[order], fagg[order]
        first = torch.ones(faces.numel(), dtype=torch.bool, device=dev)
        first[1:] = faces[1:] != faces[:-1]
        cnt = torch.bincount(faces, minlength=n)
        start = torch.nonzero(first).squeeze(1)
        f0 = faces[start]
        a0 = fagg[start]
        two = cnt[f0] == 2
        a1 = torch.where(two, fagg[(start + 1).clamp_max(faces.numel() - 1)], torch.full_like(a0, -1))
        boundary = cnt[f0] == 1
        differ = two & (a1 != a0)
        keep0 = boundary | differ
        p_agg[f0[keep0], 0] = a0[keep0]
        p_agg[f0[differ], 1] = a1[differ]
        self._p_agg = p_agg
        # P^T lists: the (row, slot) entries of every aggregate, rows ascending
        aa = p_agg.reshape(-1)
        slots = torch.nonzero(aa >= 0).squeeze(1)
        key_order = torch.sort(aa[slots] * (2 * n) + slots).indices
        pt_slot = slots[key_order]
        pt_agg = aa[pt_slot]
        pt_ptr = torch.zeros(self.n_agg + 1, dtype=torch.int64, device=dev)
        pt_ptr[1:] = torch.cumsum(torch.bincount(pt_agg, minlength=self.n_agg), 0)
        i32 = lambda a: torch.as_tensor(a, device=dev).to(torch.int32).contiguous()
        self.cell_agg = i32(agg)
        self.p_agg = i32(p_agg.reshape(-1))
        self.p_val = torch.zeros(2 * n, dtype=torch.float32, device=dev)
        self.pt_ptr = i32(pt_ptr)
        self.pt_row = i32(pt_slot // 2)
        self.pt_slot = i32(pt_slot)
        self.pt_val = torch.zeros(max(1, pt_slot.numel()), dtype=torch.float32, device=dev)
        na = self.n_agg
        self.n_blocks = 0
        if blocks is not None:
            bp = np.asarray(blocks, dtype=np.int64)
            sizes = np.diff(bp)
            if bp.ndim != 1 or bp.size < 2 or bp[0] != 0 or bp[-1] != na or np.any(sizes < 1):
                raise ValueError("blocks must rise strictly from 0 to n_agg")
            if sizes.max() > _lib.COARSE_BLOCK_MAX:
                raise ValueError(f"a coarse block has {sizes.max()} aggregates (at most {_lib.COARSE_BLOCK_MAX})")
            off = np.concatenate([[0], np.cumsum(sizes * sizes)])
            self.n_blocks = int(sizes.size)
            self.blk_ptr = i32(bp)
            self.blk_off = torch.as_tensor(off, dtype=torch.int64, device=dev)
            self.agg_blk = i32(np.repeat(np.arange(sizes.size), sizes))
            entries = int(off[-1])
            self.ac = torch.zeros(entries, dtype=torch.float64, device=dev)
            self.gj = torch.zeros(1, dtype=torch.float64, device=dev)  # unused by the block layout
            self.ac_inv = torch.zeros(entries, dtype=torch.float32, device=dev)
        else:
            entries = 0
            self.ac = torch.zeros((na, na), dtype=torch.float64, device=dev)
            self.gj = torch.zeros((na, 2 * na), dtype=torch.float64, device=dev)
            self.ac_inv = torch.zeros((na, na), dtype=torch.float32, device=dev)
        self.work = torch.zeros(64 + n + 2 * na, dtype=torch.float32, device=dev)
        self.set_weights(w)
        blk = (self.n_blocks, int(np.diff(blocks).max()) if self.n_blocks else 0, entries,
               _lib.ptr(self.blk_ptr).value if self.n_blocks else None,
               _lib.ptr(self.blk_off).value if self.n_blocks else None,
               _lib.ptr(self.agg_blk).value if self.n_blocks else None)
        self.struct = _lib.TwoLevel(pb, na, _lib.ptr(self.cell_agg).value, _lib.ptr(self.w).value,
                                    _lib.ptr(self.p_agg).value, _lib.ptr(self.p_val).value, int(pt_slot.numel()),
                                    _lib.ptr(self.pt_ptr).value, _lib.ptr(self.pt_row).value,
                                    _lib.ptr(self.pt_slot).value, _lib.ptr(self.pt_val).value,
                                    _lib.ptr(self.ac).value, _lib.ptr(self.gj).value, _lib.ptr(self.ac_inv).value,
                                    _lib.ptr(self.work).value, *blk)
        self.struct.omega = float(omega)
        self.struct.post_smooth = 1 if post_smooth else 0
        if fuse_ap:
            self._build_ap()

    # host copies of the structure, for the learned preconditioner's features
    @property
    def cell_agg_host(self):
        return self._agg.cpu().numpy()

    @property
    def counts_host(self):
        return self._counts.cpu().numpy()

    @property
    def p_agg_host(self):
        return self._p_agg.cpu().numpy()

    def _build_ap(self):
        A = self.A
        n = A.n_rows
        dev = A.values.device
        csr = _csr(A)
        ws_b = _lib.C.c_size_t(0)
        _lib.call("nfem_two_level_ap_workspace_bytes", n, _lib.C.byref(ws_b))
        ws = torch.empty(int(ws_b.value), dtype=torch.uint8, device=dev)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.ap_ptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
        nnz = _lib.C.c_int64(0)
        _lib.call("nfem_two_level_ap_pattern", _lib.C.byref(csr), _lib.C.byref(self.struct), _lib.ptr(ws),
                  ws.numel(), _lib.ptr(self.ap_ptr), None, _lib.C.byref(nnz), _lib.ptr(status), _lib.stream_ptr())
        self.ap_col = torch.empty(max(1, nnz.value), dtype=torch.int32, device=dev)
        self.ap_val = torch.zeros(max(1, nnz.value), dtype=torch.float32, device=dev)
        _lib.call("nfem_two_level_ap_pattern", _lib.C.byref(csr), _lib.C.byref(self.struct), _lib.ptr(ws),
                  ws.numel(), _lib.ptr(self.ap_ptr), _lib.ptr(self.ap_col), _lib.C.byref(nnz), _lib.ptr(status),
                  _lib.stream_ptr())
        st = int(status.item())
        if st:
            raise _lib.NfemError(st, "A P pattern")
        self.ap_nnz = int(nnz.value)
        self.struct.ap_nnz = self.ap_nnz
        self.struct.ap_ptr = _lib.ptr(self.ap_ptr).value
        self.struct.ap_col = _lib.ptr(self.ap_col).value
        self.struct.ap_val = _lib.ptr(self.ap_val).value

    def classical_weights(self):
        d = self.A.diagonal().abs()
        return torch.where(d > 0, 1.0 / d.clamp_min(1e-300), torch.zeros_like(d)).float()

    def set_weights(self, w):
        self.w = (self.classical_weights() if w is None else torch.as_tensor(w, device=self.A.values.device)
                  .float()).contiguous()
        if hasattr(self, "struct"):
            self.struct.w = _lib.ptr(self.w).value
