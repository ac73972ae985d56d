"""Device assembly behind the reference's WeakForm / SequentialAssembler API.

  * CSRMatrix        - stands where the reference passes a PETSc Mat
                       (setValue(addv=True) target, then assemble()); holds the
                       element-clique sparsity pattern built on the GPU
                       (nfem_pattern_rows/cols) and the values on the device.
  * LaplaceDualWeakForm - mixed Darcy RT1 x P0
                       (src/weak_forms/laplace_dual_weak_form.py:10-86);
                       all cells are assembled by one fused kernel
                       (nfem_darcy_rt1p0_assemble).
  * SequentialAssembler - same constructor and form_to_input_list /
                       scatter_forms as src/assembly/SequentialAssembler.py:13-86.

Coefficients: the reference calls Python functions at every quadrature point.
Here a function is sampled once on the host at the physical quadrature points
(kappa must then be constant on each cell), or the caller passes per-cell
arrays directly (numpy or torch, host or device).
"""
import time

import numpy as np
import torch

from . import _lib
from .elements import lagrange_p1_values


class CSRMatrix:
    """Global sparse matrix on the device with the pattern of a space's element cliques."""

    def __init__(self, space, dtype=torch.float64, codes=True, stream=None, extra_cliques=None):
        """extra_cliques: optional list of int arrays [n, k] of global DoFs
        whose (row, column) pairs join the pattern (the couplings of an
        interface form, whose two cells' DoFs meet in one element matrix).
        A matrix with extra cliques is filled by host-evaluated forms only:
        the device forms need the cell-clique pattern."""
        if space.cell_dofs is None:
            raise ValueError("build_structures() the space first")
        self.space = space
        self.dtype = dtype
        self.n_rows = space.n_dof + space.dof_shift
        dev = space.device
        st = _lib.stream_ptr(stream)
        T, n_loc = space.n_cells, space.n_loc
        ws_b = _lib.C.c_size_t(0)
        _lib.call("nfem_pattern_workspace_bytes", T, n_loc, self.n_rows, _lib.C.byref(ws_b))
        ws = torch.empty(int(ws_b.value), dtype=torch.uint8, device=dev)
        self.inc_ptr = torch.empty(self.n_rows + 1, dtype=torch.int32, device=dev)
        self.inc = torch.empty(T * n_loc, dtype=torch.int32, device=dev)
        self.row_ptr = torch.empty(self.n_rows + 1, dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        nnz = _lib.C.c_int64(0)
        _lib.call("nfem_pattern_rows", _lib.ptr(space.cell_dofs), T, n_loc, n_loc, self.n_rows, _lib.ptr(ws),
                  ws.numel(), _lib.ptr(self.inc_ptr), _lib.ptr(self.inc), _lib.ptr(self.row_ptr),
                  _lib.C.byref(nnz), _lib.ptr(self.status), st)
        self.nnz = int(nnz.value)
        self.col_idx = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=dev)
        _lib.call("nfem_pattern_cols", _lib.ptr(space.cell_dofs), T, n_loc, n_loc, self.n_rows,
                  _lib.ptr(self.inc_ptr), _lib.ptr(self.inc), _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx),
                  _lib.ptr(self.status), st)
        self.extended = False
        if extra_cliques:
            self._merge_cliques(extra_cliques)
            codes = False
        self.codes = None
        if codes and n_loc <= 8:
            self.codes = torch.empty(T * n_loc, dtype=torch.int32, device=dev)
            _lib.call("nfem_pattern_local_codes", _lib.ptr(space.cell_dofs), T, n_loc, n_loc, self.n_rows,
                      _lib.ptr(self.inc_ptr), _lib.ptr(self.inc), _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx),
                      _lib.ptr(self.codes), _lib.ptr(self.status), st)
        self.node_codes = None
        vec = [space.discrete_spaces[n] for n in space.names]
        ncs = {f.n_comp for f in vec}
        if (codes and self.codes is None and len(ncs) == 1 and vec[0].n_comp > 1 and n_loc % vec[0].n_comp == 0
                and n_loc // vec[0].n_comp <= 16 and space.dof_shift % vec[0].n_comp == 0):
            self.n_comp = vec[0].n_comp
            self.node_codes = torch.empty((T * n_loc, 16), dtype=torch.uint8, device=dev)
            _lib.call("nfem_pattern_node_codes", _lib.ptr(space.cell_dofs), T, n_loc, self.n_comp, space.dof_shift,
                      self.n_rows, _lib.ptr(self.inc_ptr), _lib.ptr(self.inc), _lib.ptr(self.row_ptr),
                      _lib.ptr(self.col_idx), _lib.ptr(self.node_codes), _lib.ptr(self.status), st)
        self.pairs = None
        if self.codes is not None and max_incidence(self.inc_ptr) <= 2:
            self.pairs = torch.empty((self.n_rows, 2), dtype=torch.int32, device=dev)
            self.pair_codes = torch.empty((self.n_rows, 2), dtype=torch.int32, device=dev)
            _lib.call("nfem_pattern_pairs", _lib.ptr(self.inc_ptr), _lib.ptr(self.inc), _lib.ptr(self.codes),
                      self.n_rows, _lib.ptr(self.pairs), _lib.ptr(self.pair_codes), _lib.ptr(self.status), st)
        self.chunk_rows = None
        if self.pairs is not None and _mixed_rt1_p0(space):
            # cell-chunk row table; a layout it does not cover keeps the row-owner kernel
            n_chunks = -(-T // _lib.DARCY_CHUNK_CELLS)
            cr = torch.empty(n_chunks + 1, dtype=torch.int32, device=dev)
            cst = torch.zeros(1, dtype=torch.int32, device=dev)
            rc = _lib.lib().nfem_pattern_darcy_chunks(_lib.ptr(self.pairs), self.n_rows, n_loc,
                                                      space.field_offsets[space.names[1]], T, _lib.ptr(cr),
                                                      _lib.ptr(cst), st)
            if rc == _lib.NFEM_OK and int(cst.item()) == 0:
                self.chunk_rows = cr
                # host copy of the chunk table and the largest distance between
                # a flux row's two cells: the plan of the overlapped assembly
                self.chunk_rows_host = cr.cpu().numpy().astype(np.int64)
                p_base = space.field_offsets[space.names[1]]
                pr = self.pairs[:p_base].long()
                two = pr[:, 1] >= 0
                gap = (pr[two, 1] // n_loc - pr[two, 0] // n_loc)
                self.lookahead_cells = int(gap.max().item()) if gap.numel() else 0
        self.values = torch.zeros(max(self.nnz, 1), dtype=dtype, device=dev)
        self.fresh = True
        self.check_status("pattern")

    def _merge_cliques(self, cliques):
        """Union of the cell-clique pattern and the (row, column) pairs of
        extra cliques, built on the device (sorted unique pair keys)."""
        dev = self.row_ptr.device
        n = self.n_rows
        rp = self.row_ptr.long()
        rows = torch.repeat_interleave(torch.arange(n, device=dev), rp[1:] - rp[:-1])
        keys = [rows * n + self.col_idx[: self.nnz].long()]
        for q in cliques:
            q = torch.as_tensor(np.asarray(q, dtype=np.int64), device=dev)
            if q.numel() == 0:
                continue
            if q.dim() != 2 or int(q.min().item()) < 0 or int(q.max().item()) >= n:
                raise ValueError("extra cliques must be [n, k] arrays of DoFs in [0, n_rows)")
            keys.append((q[:, :, None] * n + q[:, None, :]).reshape(-1))
        key = torch.unique(torch.cat(keys))
        r = key // n
        self.col_idx = (key % n).to(torch.int32).contiguous()
        self.row_ptr = torch.zeros(n + 1, dtype=torch.int32, device=dev)
        self.row_ptr[1:] = torch.cumsum(torch.bincount(r, minlength=n), 0).to(torch.int32)
        self.nnz = int(key.numel())
        self.extended = True

    def createVecLeft(self):
        """A zero device vector of the row space (PETSc Mat.createVecLeft)."""
        return torch.zeros(self.n_rows, dtype=self.dtype, device=self.values.device)

    def createVecRight(self):
        """A zero device vector of the column space (PETSc Mat.createVecRight)."""
        return torch.zeros(self.n_rows, dtype=self.dtype, device=self.values.device)

    def max_node_degree(self):
        """Largest number of node columns in a node row (row length / n_comp),
        computed once from row_ptr."""
        if getattr(self, "_max_node_degree", None) is None:
            lens = self.row_ptr[1:].long() - self.row_ptr[:-1].long()
            n_comp = getattr(self, "n_comp", 1) or 1
            self._max_node_degree = int(-(-int(lens.max().item()) // n_comp)) if lens.numel() else 1
        return self._max_node_degree

    def with_dtype(self, dtype):
        """A matrix with the same pattern (index arrays shared) and its own values."""
        other = object.__new__(CSRMatrix)
        other.__dict__.update(self.__dict__)
        other.dtype = dtype
        other.values = torch.zeros_like(self.values, dtype=dtype)
        other.status = torch.zeros_like(self.status)
        other.fresh = True
        return other

    def spmv(self, x, y=None, stream=None):
        """y = A x on the device (x of the matrix dtype)."""
        if y is None:
            y = torch.empty(self.n_rows, dtype=self.dtype, device=self.values.device)
        vt = _lib.NFEM_F64 if self.dtype == torch.float64 else _lib.NFEM_F32
        x = x.to(self.dtype).contiguous()
        _lib.call("nfem_spmv", vt, self.n_rows, _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx), _lib.ptr(self.values),
                  _lib.ptr(x), _lib.ptr(y), _lib.stream_ptr(stream))
        return y

    def diagonal(self):
        """Diagonal of the matrix (device tensor, zeros where the pattern has none)."""
        rp = self.row_ptr.long()
        rows = torch.repeat_interleave(torch.arange(self.n_rows, device=rp.device), rp[1:] - rp[:-1])
        cols = self.col_idx[: self.nnz].long()
        d = torch.zeros(self.n_rows, dtype=self.dtype, device=rp.device)
        on = rows == cols
        d[rows[on]] = self.values[: self.nnz][on]
        return d

    def check_status(self, where=""):
        s = int(self.status.item())
        if s:
            self.status.zero_()
            raise _lib.NfemError(s, where)

    # PETSc-like surface used by the drivers
    def zeroEntries(self):
        self.fresh = True
        self._pending = []

    def setValue(self, row, col, value, addv=True):
        """Mat.setValue: the entry is buffered on the host and added on the
        device at the next assemble() (addv=False is not supported: the
        reference's scatter always adds).  An entry outside the pattern is
        an error at assemble()."""
        if not addv:
            raise NotImplementedError("setValue(addv=False)")
        if getattr(self, "_pending", None) is None:
            self._pending = []
        self._pending.append((int(row), int(col), float(value)))

    def _flush(self):
        pend = getattr(self, "_pending", None)
        if not pend:
            return
        if self.fresh:  # the first additions of a pass go into zeros
            self.values.zero_()
            self.fresh = False
        a = np.asarray(pend, dtype=np.float64)
        dev = self.values.device
        rows = torch.as_tensor(a[:, 0].astype(np.int32), device=dev)
        cols = torch.as_tensor(a[:, 1].astype(np.int32), device=dev)
        vals = torch.as_tensor(a[:, 2], device=dev)
        vt = _lib.NFEM_F64 if self.dtype == torch.float64 else _lib.NFEM_F32
        _lib.call("nfem_csr_add_entries", vt, len(pend), _lib.ptr(rows), _lib.ptr(cols), _lib.ptr(vals),
                  _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx), self.n_rows, _lib.ptr(self.values),
                  _lib.ptr(self.status), _lib.stream_ptr(None))
        self._pending = []

    def assemble(self):
        """Mat.assemble(): adds the buffered setValue entries and checks the
        device status word."""
        self._flush()
        self.check_status("assemble")

    def getValue(self, row, col):
        """One entry (0 where the pattern has none)."""
        rp0, rp1 = int(self.row_ptr[row].item()), int(self.row_ptr[row + 1].item())
        cols = self.col_idx[rp0:rp1]
        hit = (cols == int(col)).nonzero()
        return float(self.values[rp0 + int(hit[0, 0])].item()) if hit.numel() else 0.0

    def getSize(self):
        return (self.n_rows, self.n_rows)

    def getInfo(self):
        return {"nz_allocated": self.nnz, "nz_used": self.nnz, "nz_unneeded": 0}

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.values[: self.nnz].double().cpu().numpy(),
                              self.col_idx[: self.nnz].cpu().numpy(), self.row_ptr.cpu().numpy()),
                             shape=(self.n_rows, self.n_rows))


def _mixed_rt1_p0(space):
    """True for a two-field RT1 x discontinuous P0 product space (mixed Darcy)."""
    if len(space.names) != 2:
        return False
    u, p = (space.discrete_spaces[n] for n in space.names)
    return (u.family == "RT" and u.k_order == 1 and u.n_comp == 1 and p.family == "Lagrange" and p.k_order == 0
            and p.n_comp == 1 and p.discontinuous)


def max_incidence(inc_ptr):
    return int((inc_ptr[1:] - inc_ptr[:-1]).max().item()) if inc_ptr.numel() > 1 else 0


def _to_device(x, dtype, device, n):
    t = torch.as_tensor(x)
    t = t.to(device=device, dtype=dtype).reshape(-1).contiguous()
    if t.numel() == 1 and n > 1:
        t = t.expand(n).contiguous()
    return t


def element_view(space, indices):
    """The cells `indices` of a space with disjoint DoFs: every selected cell
    gets its own copy of its DoFs, each field's block kept contiguous and in
    the space's local column order (field offset + cell * width + column).
    A device form assembled over the view gives a block-diagonal matrix
    whose row r holds exactly its cell's n_loc columns in local order: the
    element matrices, with the cells' own geometry and orientation signs."""
    idx = np.asarray(indices, dtype=np.int64).reshape(-1)
    if idx.size and (idx.min() < 0 or idx.max() >= space.n_cells):
        raise IndexError("cell index outside the space")
    view = object.__new__(type(space))
    view.__dict__.update(space.__dict__)
    T = int(idx.size)
    dev = space.device
    idx_t = torch.as_tensor(idx, device=dev)
    view.view_of = space
    view.view_indices = idx
    view.n_cells = T
    view.cells = space.cells[idx_t].contiguous()
    view.cells_host = space.cells_host[idx]
    if getattr(space, "rt_sign_mask", None) is not None:
        view.rt_sign_mask = space.rt_sign_mask[idx_t].contiguous()
    view._dof_shift = 0
    cd = np.empty((T, space.n_loc), dtype=np.int64)
    off = 0
    view.field_offsets = {}
    for name in space.names:
        sl = space.field_slices[name]
        w = sl.stop - sl.start
        view.field_offsets[name] = off
        cd[:, sl] = off + np.arange(T)[:, None] * w + np.arange(w)[None, :]
        off += T * w
    if off >= 2 ** 31 - 1:
        raise _lib.NfemError(4, "element_view (DoF count)")
    view.n_dof = off
    view.cell_dofs = torch.as_tensor(cd.astype(np.int32), device=dev)
    view._bc_cache = {}
    return view


def _slice_cells(v, idx, T):
    """A coefficient restricted to the cells idx: per-cell arrays (first
    dimension = number of cells) are sliced, scalars and callables kept."""
    if v is None or callable(v) or np.isscalar(v):
        return v
    if torch.is_tensor(v):
        return v[torch.as_tensor(idx, device=v.device)] if v.dim() and v.shape[0] == T else v
    a = np.asarray(v)
    return a[idx] if a.ndim and a.shape[0] == T else v


class WeakForm:
    """Base with the reference's attributes (src/weak_forms/weak_from.py:6-29).

    Cell forms (cell_form = True) also offer the reference's per-element
    evaluate_form(i, alpha) and a batched evaluate_forms(indices, alphas),
    both computed on the device by the form's own assembly kernel over an
    element_view of the cells."""

    cell_form = False

    def __init__(self, space):
        self.space = space
        self._functions = None

    @property
    def functions(self):
        return self._functions

    @functions.setter
    def functions(self, functions):
        self._functions = functions
        self._cache = {}

    def evaluate_forms(self, indices, alphas=None, dtype=torch.float64):
        """Element data of the cells `indices` on the device:
        (r [n, n_loc], j [n, n_loc, n_loc]) in the space's local DoF order,
        as the reference's evaluate_form returns them cell by cell.  alphas
        [n, n_loc] (the cells' slices of alpha) adds j @ alpha_l to r: the
        forms are linear in alpha, so r(alpha) = r(0) + j alpha_l with
        j = dr/dalpha."""
        if not self.cell_form:
            raise NotImplementedError(f"{type(self).__name__} is not a cell form")
        sp = self.space
        idx = np.asarray(indices, dtype=np.int64).reshape(-1)
        n_loc = sp.n_loc
        if idx.size == 0:
            return (torch.zeros((0, n_loc), dtype=dtype, device=sp.device),
                    torch.zeros((0, n_loc, n_loc), dtype=dtype, device=sp.device))
        view = element_view(sp, idx)
        vf = object.__new__(type(self))
        vf.__dict__.update(self.__dict__)
        vf.space = view
        vf.functions = {k: _slice_cells(v, idx, sp.n_cells) for k, v in (self.functions or {}).items()}
        if hasattr(vf, "use_slices"):
            vf.use_slices = False
        A = CSRMatrix(view, dtype=dtype)
        res = torch.zeros(A.n_rows, dtype=dtype, device=sp.device)
        vf.assemble(A, res, accumulate=False)
        A.check_status("evaluate_forms")
        cd = view.cell_dofs.long()
        if A.nnz != view.n_dof * n_loc:
            raise _lib.NfemError(6, "evaluate_forms (view pattern)")
        j = A.values[: A.nnz].view(view.n_dof, n_loc)[cd]  # [n, n_loc (row a), n_loc (column b)]
        r = res[cd]
        if alphas is not None:
            al = torch.as_tensor(np.asarray(alphas.cpu() if torch.is_tensor(alphas) else alphas),
                                 dtype=dtype, device=sp.device).reshape(len(idx), n_loc)
            r = r + torch.einsum("nab,nb->na", j, al)
        return r, j

    def evaluate_form(self, element_index, alpha):
        """(r_el, j_el) of one cell as host arrays, the reference's
        per-element call (e.g. laplace_dual_weak_form.py:18-86)."""
        a = None if alpha is None else np.asarray(alpha.cpu() if torch.is_tensor(alpha) else alpha)[None, :]
        r, j = self.evaluate_forms([int(element_index)], a)
        return r[0].cpu().numpy(), j[0].cpu().numpy()

    def quadrature_points(self):
        """Physical quadrature points [T, Q, 3] (host float64)."""
        sp = self.space
        pts, _ = sp.quadrature[sp.dim]
        lam = lagrange_p1_values(sp.dim, pts)  # [Q, d+1]
        X = sp.mesh.points[sp.cells_host]  # [T, d+1, 3]
        return np.einsum("qv,tvg->tqg", lam, X)


class LaplaceDualWeakForm(WeakForm):
    """Mixed Darcy RT1 x P0 on triangles or tetrahedra; fields "u" (RT, k=1) and
    "p" (Lagrange, k=0, discontinuous), in that order.

    functions: "kappa" - scalar, per-cell array [T], or f(x, y, z) constant per cell;
               "rhs"   - None, scalar, per-cell array [T], per-quadrature-point
                         array [T, Q], or f(x, y, z) -> [1, N] (sampled at the
                         quadrature points).

    use_chunks: the cell-chunk kernel when the matrix has a chunk table (True),
    else the row-owner kernel (default; the faster one on GB300 at 64^3 x 6
    tets); both write the same values up to rounding.
    use_records: the row-owner kernel reads per-cell metric records from a
    first cell pass (True) instead of evaluating each (row, cell) incidence
    from the vertices (False); the values agree to rounding.  None (default)
    takes the two passes, from measurements: 64^3 x 6 tets FP32 0.096 ms
    against 0.101 ms, FP64 0.50 ms against 1.12 ms (the geometry is
    evaluated once per cell instead of once per incidence); the 512-problem
    triangle batch FP32 0.245 ms against 0.291 ms once the cell pass writes
    the pressure rows (before that, 0.280 against 0.250 ms).
    """

    cell_form = True

    use_chunks = False
    use_records = None
    # overlapped assembly of tetrahedra (nfem_darcy_rt1p0_assemble_sliced):
    # slices of at least 2^min_slice_shift cells, record_quarters blocks of
    # every four forming records while the others write rows.  Off by
    # default: at 64^3 x 6 it measured 0.31-0.53 ms (FP64) and 0.12-0.34 ms
    # (FP32) against 0.23 / 0.10 ms for the two passes one after the other.
    use_slices = False
    # K > 0: the two passes over K cell slices on two streams.  Off by
    # default: at 64^3 x 6 it measured FP64 0.246 / 0.236 / 0.284 ms (K = 4,
    # 8, 16) and FP32 0.124 / 0.143 / 0.203 ms against 0.228 / 0.102 ms in
    # turn: each cell-pass launch fills the GPU, so the row launches queue
    # behind it instead of running beside it, and every slice adds a fill
    # and a drain
    use_streams = 0
    min_slice_shift = 17
    record_quarters = {torch.float64: 2, torch.float32: 1}
    # FP64 tetrahedra: one persistent launch whose warps take 32-cell record
    # chunks and 32-row row chunks from a plan
    # (nfem_darcy_rt1p0_assemble_fused), bitwise the values of the two
    # passes; fused_lead record chunks run ahead of the rows (0: the
    # library's choice).  Off by default: at 64^3 x 6 it reads the records
    # back from L2 (548 against 627 MB per step) but measured 0.21-0.24 ms
    # against 0.16 ms for the two passes in turn
    use_fused = False
    fused_lead = 0

    def _check_space(self):
        sp = self.space
        if sp is None or self.functions is None:
            raise ValueError
        if sp.names[:2] != ["u", "p"] or len(sp.names) != 2:
            raise NotImplementedError("LaplaceDualWeakForm expects fields ('u', 'p') in that order")
        u, p = sp.discrete_spaces["u"], sp.discrete_spaces["p"]
        if not (u.family == "RT" and u.k_order == 1 and u.n_comp == 1 and not u.discontinuous):
            raise NotImplementedError("flux space must be continuous RT1 with one component")
        if not (p.family == "Lagrange" and p.k_order == 0 and p.n_comp == 1):
            raise NotImplementedError("pressure space must be P0 with one component")

    def coefficients(self, dtype):
        """(kappa [T], source, source_mode) on the device in `dtype`."""
        key = ("coef", dtype)
        if key in self._cache:
            return self._cache[key]
        sp = self.space
        T = sp.n_cells
        dev = sp.device
        kappa = self.functions["kappa"]
        xq = None
        if callable(kappa):
            xq = self.quadrature_points()
            kv = np.asarray(kappa(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).reshape(T, -1)
            if np.abs(kv - kv[:, :1]).max() > 1e-14 * max(1.0, np.abs(kv).max()):
                raise NotImplementedError("kappa must be constant on each cell")
            kappa = kv[:, 0]
        kt = _to_device(kappa, dtype, dev, T)
        rhs = self.functions.get("rhs")
        mode = _lib.COEF_NONE
        st = None
        if callable(rhs):
            xq = self.quadrature_points() if xq is None else xq
            fv = np.asarray(rhs(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64)
            fv = fv.reshape(-1, T, xq.shape[1])[0]
            st = _to_device(fv, dtype, dev, T * xq.shape[1])
            mode = _lib.COEF_QPOINT
        elif rhs is not None:
            r = torch.as_tensor(rhs)
            if r.numel() == 1:
                st = _to_device(r, dtype, dev, T)
                mode = _lib.COEF_CELL
            elif r.numel() == T:
                st = _to_device(r, dtype, dev, T)
                mode = _lib.COEF_CELL
            else:
                st = _to_device(r, dtype, dev, r.numel())
                mode = _lib.COEF_QPOINT
        self._cache[key] = (kt, st, mode)
        return self._cache[key]

    def assemble(self, jacobian, residual, accumulate=False, stream=None, coefficients=None):
        """Assemble every cell into `jacobian` (CSRMatrix) and `residual` (device tensor)."""
        self._check_space()
        sp = self.space
        dtype = jacobian.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        if residual.dtype != dtype or not residual.is_cuda:
            raise ValueError("residual must be a CUDA tensor of the matrix dtype")
        if jacobian.pairs is None:
            raise NotImplementedError("matrix built without the two-incidence row layout")
        kt, st, mode = coefficients if coefficients is not None else self.coefficients(dtype)
        pts, wts = sp.quadrature[sp.dim]
        qw = (_lib.C.c_double * len(wts))(*wts.tolist())
        split = sp.points_split if dtype == torch.float32 else sp.points_fixed64
        if (self.use_slices and not self.use_chunks and self.use_records is not False and sp.dim == 3
                and getattr(jacobian, "chunk_rows_host", None) is not None):
            plan, ring = self._slice_plan(jacobian, dtype, vt)
            _lib.call("nfem_darcy_rt1p0_assemble_sliced", vt, sp.n_cells, jacobian.n_rows, _lib.ptr(sp.points),
                      _lib.ptr(split), _lib.ptr(sp.cells), sp.field_offsets["p"], _lib.ptr(sp.rt_sign_mask),
                      _lib.ptr(kt), _lib.ptr(st), mode, _lib.C.cast(qw, _lib.C.c_void_p), len(wts),
                      _lib.ptr(jacobian.pairs), _lib.ptr(jacobian.pair_codes), _lib.ptr(jacobian.row_ptr),
                      _lib.C.byref(plan), _lib.ptr(jacobian.values), _lib.ptr(residual), int(accumulate),
                      _lib.ptr(ring), ring.numel(), _lib.ptr(jacobian.status), _lib.stream_ptr(stream))
            return
        ws = None
        records = self.use_records
        if records is None:
            records = True
        if records and not self.use_chunks:
            key = ("records", dtype)
            if key not in self._cache:
                nb = _lib.C.c_size_t(0)
                _lib.call("nfem_darcy_workspace_bytes", sp.dim, vt, sp.n_cells, _lib.C.byref(nb))
                self._cache[key] = torch.empty(max(int(nb.value), 16), dtype=torch.uint8, device=sp.device)
            ws = self._cache[key]
            p_base = sp.field_offsets["p"]
            if (self.use_fused and sp.dim == 3 and dtype == torch.float64 and not self.use_streams
                    and p_base + sp.n_cells == jacobian.n_rows):
                plan = self._fused_plan(jacobian, stream)
                _lib.call("nfem_darcy_rt1p0_assemble_fused", sp.n_cells, jacobian.n_rows, _lib.ptr(sp.points),
                          _lib.ptr(split), _lib.ptr(sp.cells), p_base, _lib.ptr(sp.rt_sign_mask), _lib.ptr(kt),
                          _lib.ptr(st), mode, _lib.C.cast(qw, _lib.C.c_void_p), len(wts), _lib.ptr(jacobian.pairs),
                          _lib.ptr(jacobian.pair_codes), _lib.ptr(jacobian.row_ptr), _lib.ptr(plan), plan.numel(),
                          _lib.ptr(jacobian.values), _lib.ptr(residual), int(accumulate), _lib.ptr(ws), ws.numel(),
                          _lib.ptr(jacobian.status), _lib.stream_ptr(stream))
                return
            if self.use_streams and getattr(jacobian, "chunk_rows_host", None) is not None:
                return self._assemble_two_streams(jacobian, residual, accumulate, stream, kt, st, mode, qw, len(wts),
                                                  split, ws, vt)
        _lib.call("nfem_darcy_rt1p0_assemble", sp.dim, vt, sp.n_cells, jacobian.n_rows,
                  _lib.ptr(sp.points), _lib.ptr(split), _lib.ptr(sp.cells), None,
                  sp.field_offsets["p"], _lib.ptr(sp.rt_sign_mask), _lib.ptr(kt), _lib.ptr(st), mode,
                  _lib.C.cast(qw, _lib.C.c_void_p), len(wts), _lib.ptr(jacobian.pairs),
                  _lib.ptr(jacobian.pair_codes), _lib.ptr(jacobian.row_ptr),
                  _lib.ptr(jacobian.chunk_rows if self.use_chunks else None), _lib.ptr(jacobian.values),
                  _lib.ptr(residual), int(accumulate), _lib.ptr(ws), 0 if ws is None else ws.numel(),
                  _lib.ptr(jacobian.status), _lib.stream_ptr(stream))

    def _assemble_two_streams(self, jacobian, residual, accumulate, stream, kt, st, mode, qw, n_qp, split, ws, vt):
        """The two passes over K cell slices on two streams: the records of
        slice k on the launching stream, the rows of slice k on a second
        stream once the records of every cell its rows touch are done
        (slice k + ceil(lookahead / S)), so the cell pass of later slices
        runs beside the row pass of earlier ones.  Same values as the
        one-stream form (the same kernels, each row written once)."""
        sp = self.space
        T = sp.n_cells
        K = int(self.use_streams)
        S = -(-T // K)
        S = -(-S // 32) * 32  # slice starts on the chunk table's 32-cell grid
        K = -(-T // S)
        cr = jacobian.chunk_rows_host
        p_base = sp.field_offsets["p"]
        F = [int(cr[k * S // 32]) for k in range(K)] + [p_base]
        ahead = -(-int(jacobian.lookahead_cells) // S)
        main = stream if stream is not None else torch.cuda.current_stream()
        key = ("side_stream", main.device)
        if key not in self._cache:
            self._cache[key] = (torch.cuda.Stream(device=main.device),
                                [torch.cuda.Event() for _ in range(K + 1)])
        side, events = self._cache[key]
        if len(events) < K + 1:
            events.extend(torch.cuda.Event() for _ in range(K + 1 - len(events)))
        common = (sp.dim, vt, T, jacobian.n_rows, _lib.ptr(sp.points), _lib.ptr(split), _lib.ptr(sp.cells), p_base,
                  _lib.ptr(sp.rt_sign_mask), _lib.ptr(kt), _lib.ptr(st), mode, _lib.C.cast(qw, _lib.C.c_void_p), n_qp,
                  _lib.ptr(jacobian.pairs), _lib.ptr(jacobian.pair_codes), _lib.ptr(jacobian.row_ptr),
                  _lib.ptr(jacobian.values), _lib.ptr(residual), int(accumulate), _lib.ptr(ws), ws.numel())
        events[K].record(main)
        side.wait_event(events[K])  # the side stream starts after the caller's earlier work
        for k in range(K):
            _lib.call("nfem_darcy_rt1p0_assemble_pass", *common, 1, k * S, min((k + 1) * S, T), 0, 0, 0, 0,
                      _lib.ptr(jacobian.status), _lib.stream_ptr(main))
            events[k].record(main)
        for k in range(K):
            side.wait_event(events[min(K - 1, k + ahead)])
            _lib.call("nfem_darcy_rt1p0_assemble_pass", *common, 2, 0, 0, F[k], F[k + 1], p_base + k * S,
                      p_base + min((k + 1) * S, T), _lib.ptr(jacobian.status), _lib.stream_ptr(side))
        events[K].record(side)
        main.wait_event(events[K])

    def _fused_plan(self, jacobian, stream=None):
        """Work plan of the fused FP64 assembly (nfem_darcy_fused_plan), built
        once per matrix pattern; `fused_lead` record chunks run ahead of the
        rows (0: the library's choice)."""
        key = ("fused", id(jacobian.pairs), int(self.fused_lead))
        if key not in self._cache:
            sp = self.space
            p_base = sp.field_offsets["p"]
            nb = _lib.C.c_size_t(0)
            _lib.call("nfem_darcy_fused_plan_bytes", sp.n_cells, p_base, _lib.C.byref(nb))
            plan = torch.zeros(max(int(nb.value), 16), dtype=torch.uint8, device=sp.device)
            _lib.call("nfem_darcy_fused_plan", _lib.ptr(jacobian.pairs), sp.n_cells, p_base, int(self.fused_lead),
                      _lib.ptr(plan), plan.numel(), _lib.stream_ptr(stream))
            self._cache[key] = plan
        return self._cache[key]

    def _slice_plan(self, jacobian, dtype, vt):
        """(nfem_darcy_slices, ring workspace) of the overlapped assembly,
        built once per matrix pattern and precision."""
        key = ("slices", dtype, id(jacobian.chunk_rows_host))
        if key not in self._cache:
            sp = self.space
            need = max(5, int(jacobian.lookahead_cells).bit_length())  # 2^shift > lookahead
            shift = max(need, int(self.min_slice_shift))
            S = 1 << shift
            K = -(-sp.n_cells // S)
            cr = jacobian.chunk_rows_host
            F = np.array([cr[k * S // 32] for k in range(K)] + [sp.field_offsets["p"]], dtype=np.int64)
            nb = _lib.C.c_size_t(0)
            _lib.call("nfem_darcy_ring_bytes", vt, shift, _lib.C.byref(nb))
            ring = torch.empty(int(nb.value), dtype=torch.uint8, device=sp.device)
            plan = _lib.DarcySlices(shift, int(jacobian.lookahead_cells), 1, F.ctypes.data)
            self._cache[key] = (plan, ring, F)
        plan, ring, F = self._cache[key]
        rq = self.record_quarters
        plan.record_quarters = int(rq[dtype] if isinstance(rq, dict) else rq)
        return plan, ring



class LaplaceDualWeakFormBCDirichlet(WeakForm):
    """Pressure Dirichlet data on boundary facets for mixed Darcy RT1 x P0
    (src/weak_forms/laplace_dual_weak_form.py:90-154): adds int_F p_D (psi . n)
    to the flux DoF of each boundary facet whose physical tag is in
    `bc_physical_tags` (default: the space's b_physical_tags["u"], or every
    tagged facet).  functions: {"p": f(x, y, z) -> [1, N]} or a scalar.
    Only the residual changes (the form's Jacobian is zero)."""

    residual_only = True  # zero Jacobian: the residual does not depend on alpha

    def __init__(self, space, bc_physical_tags=None):
        super().__init__(space)
        self.bc_physical_tags = bc_physical_tags

    def facets(self):
        if "facets" in self._cache:
            return self._cache["facets"]
        sp = self.space
        dim = sp.dim
        tags = self.bc_physical_tags
        if tags is None:
            tags = sp.b_physical_tags.get("u") or None
        fl = sp.facet_flags.cpu().numpy()
        occ = np.flatnonzero((fl.ravel() & 2) != 0)
        c = occ // (dim + 1)
        i = occ % (dim + 1)
        from .elements import P2_EDGES
        sub = np.array(P2_EDGES[2] if dim == 2 else ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)))
        verts = np.sort(sp.cells_host[c[:, None], sub[i]], axis=1)
        V = sp.mesh.points.shape[0]
        key = np.zeros(len(occ), dtype=np.int64)
        for k in range(dim):
            key = key * V + verts[:, k]
        from .meshes import BLOCK_DIM
        fconn, ftag = [], []
        for typ, conn, phys in sp.mesh.data["blocks"]:
            if BLOCK_DIM[typ] == dim - 1:
                fconn.append(np.asarray(conn, dtype=np.int64))
                ftag.append(np.asarray(phys))
        fconn = np.concatenate(fconn)
        ftag = np.concatenate(ftag)
        fkey = np.zeros(len(fconn), dtype=np.int64)
        fs = np.sort(fconn, axis=1)
        for k in range(dim):
            fkey = fkey * V + fs[:, k]
        order = np.argsort(fkey, kind="stable")
        pos = order[np.searchsorted(fkey[order], key)]
        keep = np.ones(len(occ), dtype=bool) if tags is None else np.isin(ftag[pos], np.asarray(tags))
        out = (occ[keep].astype(np.int32), fconn[pos[keep]])
        self._cache["facets"] = out
        return out

    def assemble(self, jacobian, residual, accumulate=True, stream=None):
        sp = self.space
        dim = sp.dim
        occ, fverts = self.facets()
        dtype = residual.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        pts, wts = sp.bc_quadrature[dim - 1]
        lam = lagrange_p1_values(dim - 1, pts)
        xq = np.einsum("qv,fvg->fqg", lam, sp.mesh.points[fverts])
        p = self.functions["p"]
        if callable(p):
            pv = np.asarray(p(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).reshape(-1, *xq.shape[:2])[0]
        else:
            pv = np.full(xq.shape[:2], float(p))
        pd = torch.as_tensor(np.ascontiguousarray(pv), dtype=dtype, device=sp.device)
        occ_t = torch.as_tensor(occ, device=sp.device)
        qw = np.ascontiguousarray(wts, dtype=np.float64)
        _lib.call("nfem_darcy_rt1_dirichlet", dim, vt, len(occ), _lib.ptr(occ_t), _lib.ptr(sp.rt_sign_mask),
                  _lib.ptr(sp.cell_dofs), sp.n_loc, _lib.ptr(pd), qw.ctypes.data_as(_lib.C.POINTER(_lib.C.c_double)),
                  len(wts), _lib.ptr(residual), _lib.stream_ptr(stream))
        if not hasattr(self, "_keep"):
            self._keep = []
        self._keep = [pd, occ_t]


class LCEDualWeakFormBCDirichlet(LaplaceDualWeakFormBCDirichlet):
    """Displacement and rotation data on boundary facets for the mixed
    Cosserat form (src/weak_forms/lce_dual_weak_form.py:651-756): for every
    component c, adds -int_F u_D[c] (tau . n) to the stress row c of the
    facet's flux DoF and -int_F t_D[c] (v . n) to its couple-stress row c.
    functions: {"u": f(x, y, z) -> [3, N], "t": f(x, y, z) -> [3, N]} (or
    3-vectors).  Facets whose tag is in bc_physical_tags (default: the
    space's b_physical_tags["s"], or every tagged facet).  Residual only."""

    FIELD_DATA = (("s", "u"), ("m", "t"))  # (RT1 field, its Dirichlet datum)

    def __init__(self, space, bc_physical_tags=None):
        super().__init__(space, bc_physical_tags if bc_physical_tags is not None
                         else (space.b_physical_tags.get("s") or None))

    def assemble(self, jacobian, residual, accumulate=True, stream=None):
        sp = self.space
        dim = sp.dim
        occ, fverts = self.facets()
        dtype = residual.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        pts, wts = sp.bc_quadrature[dim - 1]
        lam = lagrange_p1_values(dim - 1, pts)
        xq = np.einsum("qv,fvg->fqg", lam, sp.mesh.points[fverts])
        occ_t = torch.as_tensor(occ, device=sp.device)
        qw = np.ascontiguousarray(wts, dtype=np.float64)
        keep = [occ_t]
        for field, name in self.FIELD_DATA:
            fn = self.functions[name]
            if callable(fn):
                v = np.asarray(fn(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).reshape(3, *xq.shape[:2])
            else:
                v = np.broadcast_to(np.asarray(fn, dtype=np.float64).reshape(3, 1, 1), (3,) + xq.shape[:2])
            for c in range(3):
                pd = torch.as_tensor(np.ascontiguousarray(v[c]), dtype=dtype, device=sp.device)
                keep.append(pd)
                _lib.call("nfem_rt1_dirichlet_rows", dim, vt, len(occ), _lib.ptr(occ_t), _lib.ptr(sp.rt_sign_mask),
                          _lib.ptr(sp.cell_dofs), sp.n_loc, sp.field_slices[field].start + c, 3, -1.0, _lib.ptr(pd),
                          qw.ctypes.data_as(_lib.C.POINTER(_lib.C.c_double)), len(wts), _lib.ptr(residual),
                          _lib.stream_ptr(stream))
        self._keep = keep


class LEDualWeakFormBCDirichlet(LCEDualWeakFormBCDirichlet):
    """Displacement data on boundary facets for the mixed linear-elastic form
    (src/weak_forms/le_dual_weak_form.py:518-595): for every component c,
    adds -int_F u_D[c] (tau . n) to the stress row c of the facet's flux
    DoF.  functions: {"u": f(x, y, z) -> [3, N]} (or a 3-vector).  Residual
    only."""

    FIELD_DATA = (("s", "u"),)


class SequentialAssembler:
    """Drop-in for src/assembly/SequentialAssembler.py:13-86.

    `jacobian` is a CSRMatrix; `residual` a device tensor (or a host numpy
    array, updated in place with a device->host copy at the end).  A call to
    scatter_forms() is one assembly pass: the first form overwrites the
    matrix values and the residual (they are treated as zeroed, as every
    reference driver creates them), later forms of the pass add to them.

    The six form types of the reference (SequentialAssembler.py:20-30) are
    accepted with its input lists:
      "form" / "bc_form":               [type, sequence, form, alpha]
      "interface_form":                 [type, [(idx, (idx_p, idx_n)), ...], form, alpha]
      "bc_interface_form":              [type, [(idx, idx_p), ...], form, alpha]
      "time_dependent_form" / "..._bc_form": [type, sequence, form, (alpha_n, alpha), t]
    A device form (LaplaceDualWeakForm, LEPrimalWeakForm, LCEDualWeakForm,
    their boundary forms, ...) assembles every cell in one launch.  Any
    other form object is evaluated on the host element by element exactly
    as the reference calls it (ScatterFormData.py:28-79: evaluate_form on
    the element's slice of alpha, with the same arguments; a form may offer
    evaluate_forms(indices, alphas) returning batched (r [n, k], j [n, k, k])
    instead), and the batch is added into the device CSR and residual by
    one scatter kernel (nfem_scatter_elements).
    """

    _GENERIC = ("form", "bc_form", "interface_form", "bc_interface_form", "time_dependent_form",
                "time_dependent_bc_form")

    def __init__(self, space, jacobian, residual):
        self.space = space
        self.jacobian = jacobian
        self.residual = residual
        self._form_to_input_list = None
        self._dest = None

    @property
    def form_type_to_callable_map(self):
        return {t: (lambda *a, _t=t: self._scatter(_t, *a)) for t in self._GENERIC}

    @property
    def form_to_input_list(self):
        return self._form_to_input_list

    @form_to_input_list.setter
    def form_to_input_list(self, v):
        self._form_to_input_list = v

    @staticmethod
    def _is_device_form(form):
        return isinstance(form, WeakForm) and callable(getattr(form, "assemble", None))

    # ------------------------------------------------------------ device forms
    def _scatter_form(self, form, sequence, alpha, residual, accumulate):
        """All cells at alpha = 0: the form's one-launch row-owner assembly.
        A subset of the cells or alpha != 0: the form's element data of those
        cells (evaluate_forms, on the device) added by the scatter kernel."""
        n = self.space.n_cells
        seq = range(n) if sequence is None else sequence
        full = isinstance(seq, range) and seq.start == 0 and seq.stop == n and seq.step == 1
        if not full:
            full = np.array_equal(np.asarray(list(seq)), np.arange(n))
        zero = alpha is None or not np.any(self._host(alpha) != 0)
        if full and zero:
            form.assemble(self.jacobian, residual, accumulate=accumulate)
            return
        A = self.jacobian
        if not accumulate:
            A.values.zero_()
            residual.zero_()
        idx = np.asarray(list(seq), dtype=np.int64)
        al = None if zero else self._host(alpha)[self._cell_dest()[idx]]
        r, j = form.evaluate_forms(idx, al, dtype=A.dtype)
        d_t = torch.as_tensor(self._cell_dest()[idx].astype(np.int32), device=A.values.device)
        vt = _lib.NFEM_F64 if A.dtype == torch.float64 else _lib.NFEM_F32
        _lib.call("nfem_scatter_elements", vt, len(idx), r.shape[1], _lib.ptr(d_t), _lib.ptr(j.contiguous()),
                  _lib.ptr(r.contiguous()), _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), A.n_rows, _lib.ptr(A.values),
                  _lib.ptr(residual), _lib.ptr(A.status), _lib.stream_ptr(None))
        A.check_status("scatter of a device form's element data")

    def _scatter_bc_form(self, form, sequence, alpha, residual, accumulate):
        if not accumulate:
            raise NotImplementedError("a boundary form adds to a pass that starts with a cell form")
        if not getattr(form, "residual_only", False) and alpha is not None and np.any(self._host(alpha) != 0):
            raise NotImplementedError("this boundary form is assembled at alpha = 0")
        form.assemble(self.jacobian, residual, accumulate=True)

    # ------------------------------------------------------------ host-evaluated forms
    def _cell_dest(self):
        if self._dest is None:
            self._dest = self.space.all_destination_indexes()
        return self._dest

    @staticmethod
    def _host(a):
        if a is None:
            return None
        if torch.is_tensor(a):
            return a.detach().double().cpu().numpy()
        return np.asarray(a)

    def _evaluate(self, form_type, form, items, alpha, alpha_n, t):
        """Element data of a host-evaluated form: (dest list, r list, j list),
        with the reference's arguments per element."""
        sp = self.space
        dest_all = self._cell_dest()
        dests, rs, js = [], [], []
        batched = getattr(form, "evaluate_forms", None)
        if form_type == "form":
            idx = np.asarray(list(items), dtype=np.int64)
            d = dest_all[idx]
            if batched is not None:
                r, j = batched(idx, alpha[d])
                return list(d), list(np.asarray(r)), list(np.asarray(j))
            for i, di in zip(idx, d):
                r, j = form.evaluate_form(int(i), alpha[di])
                dests.append(di), rs.append(r), js.append(j)
        elif form_type == "time_dependent_form":
            for i in items:
                di = dest_all[int(i)]
                r, j = form.evaluate_form(int(i), alpha_n[di], alpha[di], t)
                dests.append(di), rs.append(r), js.append(j)
        elif form_type == "bc_form":
            for i in items:
                di = sp.bc_destination_indexes(int(i))
                r, j = form.evaluate_form(int(i), alpha[di])
                dests.append(di), rs.append(r), js.append(j)
        elif form_type == "time_dependent_bc_form":
            for i in items:
                di = sp.bc_destination_indexes(int(i))
                # the reference takes this slice from alpha_n (ScatterFormData.py:43-49)
                r, j = form.evaluate_form(int(i), alpha_n[di], t)
                dests.append(di), rs.append(r), js.append(j)
        elif form_type == "interface_form":
            for idx, pair in items:
                p, n = pair
                dp, dn = dest_all[int(p)], dest_all[int(n)]
                r, j = form.evaluate_form(idx, pair, (alpha[dp], alpha[dn]))
                dests.append(np.concatenate((dp, dn))), rs.append(r), js.append(j)
        elif form_type == "bc_interface_form":
            for idx, p in items:
                dp = dest_all[int(p)]
                r, j = form.evaluate_form(idx, p, alpha[dp])
                dests.append(dp), rs.append(r), js.append(j)
        else:
            raise NotImplementedError(f"form type {form_type}")
        return dests, rs, js

    def _scatter_host(self, form_type, form, items, alpha, alpha_n, t, residual):
        A = self.jacobian
        n = A.n_rows
        alpha = self._host(alpha) if alpha is not None else np.zeros(n)
        alpha_n = self._host(alpha_n) if alpha_n is not None else alpha
        dests, rs, js = self._evaluate(form_type, form, items, alpha, alpha_n, t)
        if not dests:
            return
        vt = _lib.NFEM_F64 if A.dtype == torch.float64 else _lib.NFEM_F32
        npdt = np.float64 if A.dtype == torch.float64 else np.float32
        dev = A.values.device
        groups = {}
        for k, d in enumerate(dests):
            groups.setdefault(len(d), []).append(k)
        for k_loc, ks in groups.items():
            if k_loc == 0:
                continue
            d = np.stack([np.asarray(dests[k], dtype=np.int64) for k in ks])
            if d.min() < 0 or d.max() >= n or d.max() >= 2 ** 31:
                raise ValueError("destination index outside the matrix")
            r = np.stack([np.asarray(rs[k], dtype=np.float64).reshape(k_loc) for k in ks]).astype(npdt)
            j = np.stack([np.asarray(js[k], dtype=np.float64).reshape(k_loc, k_loc) for k in ks]).astype(npdt)
            d_t = torch.as_tensor(d.astype(np.int32), device=dev)
            r_t = torch.as_tensor(r, device=dev)
            j_t = torch.as_tensor(j, device=dev)
            _lib.call("nfem_scatter_elements", vt, len(ks), k_loc, _lib.ptr(d_t), _lib.ptr(j_t), _lib.ptr(r_t),
                      _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), n, _lib.ptr(A.values), _lib.ptr(residual),
                      _lib.ptr(A.status), _lib.stream_ptr(None))
        A.check_status(f"scatter of a {form_type}")

    def _scatter(self, form_type, input_list, residual, accumulate):
        if "time_dependent" in form_type:
            _, sequence, form, alphas, t = input_list
            alpha_n, alpha = alphas
        else:
            _, sequence, form, alpha = input_list[:4]
            alpha_n, t = None, None
        if self._is_device_form(form):
            if form_type == "form":
                return self._scatter_form(form, sequence, alpha, residual, accumulate)
            if form_type == "bc_form":
                return self._scatter_bc_form(form, sequence, alpha, residual, accumulate)
            raise NotImplementedError(f"a device form in a {form_type} entry")
        return self._scatter_host(form_type, form, sequence, alpha, alpha_n, t, residual)

    def scatter_forms(self, measure_time_q=False):
        items = list(self.form_to_input_list.items())
        for name, input_list in items:
            if input_list[0] not in self._GENERIC:
                raise NotImplementedError(f"form type {input_list[0]}")
            want = 5 if "time_dependent" in input_list[0] else 4
            if len(input_list) != want:
                raise ValueError(f"{name}: a {input_list[0]} entry has {want} items")
        host_res = None
        residual = self.residual
        if not torch.is_tensor(residual):
            host_res = residual
            residual = torch.zeros(self.jacobian.n_rows, dtype=self.jacobian.dtype, device=self.space.device)
        accumulate = not self.jacobian.fresh
        first_device = bool(items) and self._is_device_form(items[0][1][2])
        if not accumulate and not first_device:
            # a pass that starts with a host-evaluated form adds into zeros
            self.jacobian.values.zero_()
            residual.zero_()
            accumulate = True
        first = True
        for name, input_list in items:
            if measure_time_q:
                torch.cuda.synchronize()
                st = time.time()
            self._scatter(input_list[0], input_list, residual, accumulate or not first)
            first = False
            if measure_time_q:
                torch.cuda.synchronize()
                print("SequentialAssembler:: Weak form: ", name)
                print("SequentialAssembler:: Scatter time:", time.time() - st, "seconds")
        self.jacobian.fresh = False
        if host_res is not None:
            host_res += residual.double().cpu().numpy()


def _cellwise(v, T, what, sp, form):
    """Scalar, per-cell array, or callable constant on each cell -> [T] float64."""
    if callable(v):
        xq = form.quadrature_points()
        vals = np.asarray(v(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).reshape(T, -1)
        if np.abs(vals - vals[:, :1]).max() > 1e-14 * max(1.0, np.abs(vals).max()):
            raise NotImplementedError(f"{what} must be constant on each cell")
        return vals[:, 0]
    a = np.asarray(v, dtype=np.float64).reshape(-1)
    return np.full(T, a[0]) if a.size == 1 else a


class LEPrimalWeakForm(WeakForm):
    """Vector P2 linear elasticity (src/weak_forms/le_primal_weak_form.py:10-129)
    on tetrahedra; field "u" (Lagrange, k=2, 3 components).

    functions: "lambda", "mu" - scalar, per-cell array, or f(x, y, z) constant
               per cell; "rhs" - None, a 3-vector, per-cell array [T, 3], or
               f(x, y, z) -> [3, N] constant per cell.  r = +int f . phi."""

    cell_form = True

    def _check_space(self):
        sp = self.space
        if sp is None or self.functions is None:
            raise ValueError
        u = sp.discrete_spaces.get("u")
        if (len(sp.names) != 1 or u is None or u.family != "Lagrange" or u.k_order != 2 or u.n_comp != 3
                or sp.dim != 3 or u.discontinuous):
            raise NotImplementedError("LEPrimalWeakForm expects one field 'u': continuous vector P2 on tetrahedra")

    def coefficients(self, dtype):
        key = ("coef", dtype)
        if key in self._cache:
            return self._cache[key]
        sp = self.space
        T = sp.n_cells
        lam = _cellwise(self.functions["lambda"], T, "lambda", sp, self)
        mu = _cellwise(self.functions["mu"], T, "mu", sp, self)
        f = self.functions.get("rhs")
        ft = None
        if f is not None:
            if callable(f):
                xq = self.quadrature_points()
                fv = np.asarray(f(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).reshape(3, T, -1)
                if np.abs(fv - fv[:, :, :1]).max() > 1e-14 * max(1.0, np.abs(fv).max()):
                    raise NotImplementedError("rhs must be constant on each cell")
                fv = fv[:, :, 0].T
            else:
                fv = np.asarray(f, dtype=np.float64)
                fv = np.broadcast_to(fv.reshape(-1, 3) if fv.size != 3 else fv.reshape(1, 3), (T, 3))
            ft = torch.as_tensor(np.array(fv, dtype=np.float64, order="C"), dtype=dtype, device=sp.device)
        from .elements import p2_reference_tables
        S, m, Mf = p2_reference_tables(3)
        out = (torch.as_tensor(lam, dtype=dtype, device=sp.device), torch.as_tensor(mu, dtype=dtype, device=sp.device),
               ft, np.ascontiguousarray(S.reshape(-1)), np.ascontiguousarray(m), np.ascontiguousarray(Mf.reshape(-1)))
        self._cache[key] = out
        return out

    def assemble(self, jacobian, residual, accumulate=False, stream=None, coefficients=None):
        self._check_space()
        sp = self.space
        dtype = jacobian.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        if jacobian.node_codes is None:
            raise NotImplementedError("matrix built without node codes")
        lam, mu, f, S, m, _ = coefficients if coefficients is not None else self.coefficients(dtype)
        dp = _lib.C.POINTER(_lib.C.c_double)
        key = ("geom", dtype)
        if key not in self._cache:
            nb = _lib.C.c_size_t(0)
            _lib.call("nfem_elasticity_p2_workspace_bytes", vt, sp.n_cells, _lib.C.byref(nb))
            self._cache[key] = torch.empty(max(int(nb.value), 16), dtype=torch.uint8, device=sp.device)
        ws = self._cache[key]
        _lib.call("nfem_elasticity_p2_assemble", vt, sp.n_cells, sp.n_dof // 3, sp.dof_shift, _lib.ptr(sp.points),
                  _lib.ptr(sp.points_split), _lib.ptr(sp.cells), _lib.ptr(lam), _lib.ptr(mu), _lib.ptr(f),
                  S.ctypes.data_as(dp), m.ctypes.data_as(dp), _lib.ptr(jacobian.inc_ptr), _lib.ptr(jacobian.inc),
                  _lib.ptr(jacobian.node_codes), _lib.ptr(jacobian.row_ptr), jacobian.max_node_degree(),
                  _lib.ptr(jacobian.values), _lib.ptr(residual), int(accumulate), _lib.ptr(ws), ws.numel(),
                  _lib.ptr(jacobian.status), _lib.stream_ptr(stream))


class LEPrimalWeakFormBCDirichlet(WeakForm):
    """Penalty Dirichlet condition u = 0 on the boundary facets
    (src/weak_forms/le_primal_weak_form.py:131-177, beta = 1e12): adds
    beta int_F phi_a phi_b to every component's (a, b) entry.  Accumulates
    into the matrix (use it as the second form of an assembly pass)."""

    beta = 1.0e12

    def facet_dofs(self):
        """[n_facets, 18] DoFs of the boundary facets in the facet's P2 order
        (vertices in file order, then edges (1,2), (0,2), (0,1))."""
        if "fdofs" in self._cache:
            return self._cache["fdofs"]
        sp = self.space
        cells = sp.cells_host
        T = sp.n_cells
        V = sp.mesh.points.shape[0]
        r0 = sp.occ_rank[0].cpu().numpy()
        vrank = np.full(V, -1, dtype=np.int64)
        vrank[cells.ravel()] = r0.ravel()
        from .elements import P2_EDGES
        tet_e = np.array(P2_EDGES[3])
        ekeys_c = np.sort(cells[:, tet_e], axis=2)
        ek = (ekeys_c[..., 0] * V + ekeys_c[..., 1]).ravel()
        r1 = sp.occ_rank[1].cpu().numpy().ravel()
        order = np.argsort(ek, kind="stable")
        ek_s, r1_s = ek[order], r1[order]
        fac = sp.facets.cpu().numpy().astype(np.int64)
        tri_e = np.array(P2_EDGES[2])
        fk = np.sort(fac[:, tri_e], axis=2)
        fkey = fk[..., 0] * V + fk[..., 1]
        pos = np.searchsorted(ek_s, fkey.ravel())
        if np.any(pos >= ek_s.size) or np.any(ek_s[np.minimum(pos, ek_s.size - 1)] != fkey.ravel()):
            raise ValueError("boundary facet edge not found among the cells' edges")
        erank = r1_s[pos].reshape(-1, 3)
        base_v = sp.field_offsets["u"]
        base_e = base_v + 3 * sp.n_entities[0]
        nodes = np.concatenate([base_v + 3 * vrank[fac], base_e + 3 * erank], axis=1)  # [F, 6]
        fd = (nodes[:, :, None] + np.arange(3)[None, None, :]).reshape(-1, 18)
        out = (torch.as_tensor(fd.astype(np.int32), device=sp.device),
               torch.as_tensor(fac.astype(np.int32), device=sp.device))
        self._cache["fdofs"] = out
        return out

    def assemble(self, jacobian, residual=None, accumulate=True, stream=None):
        sp = self.space
        fd, fv = self.facet_dofs()
        vt = _lib.NFEM_F64 if jacobian.dtype == torch.float64 else _lib.NFEM_F32
        from .elements import p2_reference_tables
        S, m, Mf = p2_reference_tables(3)
        S = np.ascontiguousarray(S.reshape(-1))
        Mf = np.ascontiguousarray(Mf.reshape(-1))
        dp = _lib.C.POINTER(_lib.C.c_double)
        _lib.call("nfem_elasticity_p2_penalty", vt, fd.shape[0], _lib.ptr(fd), _lib.ptr(fv), _lib.ptr(sp.points),
                  float(self.beta), S.ctypes.data_as(dp), m.ctypes.data_as(dp), Mf.ctypes.data_as(dp),
                  _lib.ptr(jacobian.row_ptr), _lib.ptr(jacobian.col_idx), _lib.ptr(jacobian.values),
                  _lib.ptr(jacobian.status), _lib.stream_ptr(stream))


class LCEDualWeakForm(WeakForm):
    """Mixed Cosserat elasticity, 3-D (src/weak_forms/lce_dual_weak_form.py:410-648):
    fields s (RT1, 3 rows), m (RT1, 3 rows), u (P0^3), t (P0^3) in that order.

    functions: lambda_s, mu_s, kappa_s, lambda_o, mu_o, kappa_o, l - scalars
    or f(x, y, z) callables like the reference drivers pass
    (mfe_cosserat_elasticity_example_3.py:120-125), sampled at the quadrature
    points and required to be constant over the mesh (the material of every
    benchmark and driver is); "rhs" - None, a 6-vector (f_u, f_t), a per-cell
    array [T, 6], or f(x, y, z) -> [6, N] sampled at the quadrature points.
    The u and t test functions are P0, so the reference's load
    -sum_q |det J| w_q f(x_q) (lce_dual_weak_form.py:490-502) is exactly the
    cell's quadrature-weighted mean of f times -|T|: that mean is what goes
    to the device."""

    cell_form = True

    NAMES = ("lambda_s", "mu_s", "kappa_s", "lambda_o", "mu_o", "kappa_o", "l")

    def _check_space(self):
        sp = self.space
        if sp is None or self.functions is None:
            raise ValueError
        if sp.names != ["s", "m", "u", "t"] or sp.dim != 3:
            raise NotImplementedError("LCEDualWeakForm expects fields ('s', 'm', 'u', 't') on tetrahedra")
        d = sp.discrete_spaces
        ok = (d["s"].family == "RT" and d["s"].k_order == 1 and d["m"].family == "RT" and d["m"].k_order == 1
              and d["u"].family == "Lagrange" and d["u"].k_order == 0 and d["t"].family == "Lagrange"
              and d["t"].k_order == 0 and all(d[n].n_comp == 3 for n in sp.names))
        if not ok:
            raise NotImplementedError("LCEDualWeakForm expects RT1^3 x RT1^3 x P0^3 x P0^3")

    def coefficients(self, dtype):
        key = ("coef", dtype)
        if key in self._cache:
            return self._cache[key]
        sp = self.space
        T = sp.n_cells
        xq = None
        par = []
        for k in self.NAMES:
            v = self.functions[k]
            if callable(v):
                xq = self.quadrature_points() if xq is None else xq
                vals = np.asarray(v(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).ravel()
                if vals.size == 0 or np.abs(vals - vals[0]).max() > 1e-14 * max(1.0, np.abs(vals).max()):
                    raise NotImplementedError(f"{k} must be constant over the mesh (the device form takes one material)")
                par.append(float(vals[0]))
            else:
                par.append(float(np.ravel(v)[0]))
        par = np.array(par, dtype=np.float64)
        f = self.functions.get("rhs")
        ft = None
        if f is not None:
            if callable(f):
                xq = self.quadrature_points() if xq is None else xq
                _, wts = sp.quadrature[sp.dim]
                fq = np.asarray(f(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).reshape(6, T, -1)
                fv = np.einsum("ktq,q->tk", fq, np.asarray(wts)) / float(np.sum(wts))
            else:
                fv = np.asarray(f, dtype=np.float64)
                fv = np.broadcast_to(fv.reshape(1, 6) if fv.size == 6 else fv.reshape(T, 6), (T, 6))
            ft = torch.as_tensor(np.ascontiguousarray(fv), dtype=dtype, device=sp.device)
        from .elements import rt1_tet_tables
        Psi, mhat, divhat = rt1_tet_tables()
        out = (par, ft, np.ascontiguousarray(Psi.reshape(-1)), np.ascontiguousarray(mhat.reshape(-1)),
               np.ascontiguousarray(divhat))
        self._cache[key] = out
        return out

    def assemble(self, jacobian, residual, accumulate=False, stream=None, coefficients=None):
        self._check_space()
        sp = self.space
        dtype = jacobian.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        if jacobian.node_codes is None:
            raise NotImplementedError("matrix built without node codes")
        par, f, Psi, mhat, divhat = coefficients if coefficients is not None else self.coefficients(dtype)
        dp = _lib.C.POINTER(_lib.C.c_double)
        key = ("geom", dtype)
        if key not in self._cache:
            nb = _lib.C.c_size_t(0)
            _lib.call("nfem_cosserat_workspace_bytes", vt, sp.n_cells, _lib.C.byref(nb))
            self._cache[key] = torch.empty(max(int(nb.value), 16), dtype=torch.uint8, device=sp.device)
        ws = self._cache[key]
        _lib.call("nfem_cosserat_assemble", vt, sp.n_cells, sp.n_dof // 3, sp.dof_shift, _lib.ptr(sp.points),
                  _lib.ptr(sp.points_split), _lib.ptr(sp.cells), _lib.ptr(sp.rt_sign_mask), par.ctypes.data_as(dp),
                  _lib.ptr(f), Psi.ctypes.data_as(dp), mhat.ctypes.data_as(dp), divhat.ctypes.data_as(dp),
                  _lib.ptr(jacobian.inc_ptr), _lib.ptr(jacobian.inc), _lib.ptr(jacobian.node_codes),
                  _lib.ptr(jacobian.row_ptr), _lib.ptr(jacobian.values), _lib.ptr(residual), int(accumulate),
                  _lib.ptr(ws), ws.numel(), _lib.ptr(jacobian.status), _lib.stream_ptr(stream))


class LCEScaledRieszMapWeakForm(LCEDualWeakForm):
    """The Cosserat preconditioning operator of the reference driver
    (src/weak_forms/lce_scaled_riesz_map_weak_form.py:415-598; assembled as P
    in mfe_cosserat_elasticity_example_3.py:189-240): block-diagonal by field,
    compliance + div-div on the stress and couple-stress rows, P0 mass on u
    and t.  functions: the material of LCEDualWeakForm, "l" (a constant, or a
    callable constant over the mesh) and optionally "grad_l" (must vanish:
    only a constant length scale is supported on the device).  Assembles the
    Jacobian only (the form has no load)."""

    def coefficients(self, dtype):
        gl = self.functions.get("grad_l")
        if gl is not None:
            xq = self.quadrature_points()
            g = np.asarray(gl(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64)
            if np.abs(g).max() > 0:
                raise NotImplementedError("a varying length scale l (grad_l != 0) is not supported on the device")
        saved = self.functions.get("rhs")
        self.functions["rhs"] = None
        try:
            return super().coefficients(dtype)
        finally:
            self.functions["rhs"] = saved

    def assemble(self, jacobian, residual=None, accumulate=False, stream=None, coefficients=None):
        self._check_space()
        sp = self.space
        dtype = jacobian.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        if jacobian.node_codes is None:
            raise NotImplementedError("matrix built without node codes")
        par, _, Psi, mhat, divhat = coefficients if coefficients is not None else self.coefficients(dtype)
        dp = _lib.C.POINTER(_lib.C.c_double)
        key = ("geom", dtype)
        if key not in self._cache:
            nb = _lib.C.c_size_t(0)
            _lib.call("nfem_cosserat_workspace_bytes", vt, sp.n_cells, _lib.C.byref(nb))
            self._cache[key] = torch.empty(max(int(nb.value), 16), dtype=torch.uint8, device=sp.device)
        ws = self._cache[key]
        _lib.call("nfem_cosserat_riesz_assemble", vt, sp.n_cells, sp.n_dof // 3, sp.dof_shift, _lib.ptr(sp.points),
                  _lib.ptr(sp.points_split), _lib.ptr(sp.cells), _lib.ptr(sp.rt_sign_mask), par.ctypes.data_as(dp),
                  Psi.ctypes.data_as(dp), mhat.ctypes.data_as(dp), divhat.ctypes.data_as(dp),
                  _lib.ptr(jacobian.inc_ptr), _lib.ptr(jacobian.inc), _lib.ptr(jacobian.node_codes),
                  _lib.ptr(jacobian.row_ptr), _lib.ptr(jacobian.values), int(accumulate), _lib.ptr(ws), ws.numel(),
                  _lib.ptr(jacobian.status), _lib.stream_ptr(stream))


class LEDualWeakForm(WeakForm):
    """Mixed linear elasticity with weakly imposed symmetry, 3-D
    (src/weak_forms/le_dual_weak_form.py:354-515): fields s (RT1^3), u (P0^3),
    t (P0^3).  functions: "lambda", "mu" (constants or callables constant
    over the mesh) and "rhs" (f_u then f_t, a 6-vector, per-cell [T, 6] or
    f(x, y, z) -> [6, N]: its quadrature-weighted cell mean is exact for the
    P0 test functions).  r = -int f . v at alpha = 0."""

    cell_form = True
    NAMES = ("lambda", "mu")

    def _check_space(self):
        LERieszMapWeakForm._check_space(self)

    def coefficients(self, dtype):
        key = ("coef", dtype)
        if key in self._cache:
            return self._cache[key]
        sp = self.space
        T = sp.n_cells
        lam, mu, Psi, mhat, divhat = LERieszMapWeakForm.coefficients(self, dtype)
        f = self.functions.get("rhs")
        ft = None
        if f is not None:
            if callable(f):
                xq = self.quadrature_points()
                _, wts = sp.quadrature[sp.dim]
                fq = np.asarray(f(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).reshape(6, T, -1)
                fv = np.einsum("ktq,q->tk", fq, np.asarray(wts)) / float(np.sum(wts))
            else:
                fv = np.asarray(f, dtype=np.float64)
                fv = np.broadcast_to(fv.reshape(1, 6) if fv.size == 6 else fv.reshape(T, 6), (T, 6))
            ft = torch.as_tensor(np.array(fv, dtype=np.float64, order="C"), dtype=dtype, device=sp.device)
        out = (lam, mu, ft, Psi, mhat, divhat)
        self._cache[key] = out
        return out

    def assemble(self, jacobian, residual, accumulate=False, stream=None, coefficients=None):
        self._check_space()
        sp = self.space
        dtype = jacobian.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        if jacobian.node_codes is None:
            raise NotImplementedError("matrix built without node codes")
        lam, mu, f, Psi, mhat, divhat = coefficients if coefficients is not None else self.coefficients(dtype)
        dp = _lib.C.POINTER(_lib.C.c_double)
        key = ("geom", dtype)
        if key not in self._cache:
            nb = _lib.C.c_size_t(0)
            _lib.call("nfem_cosserat_workspace_bytes", vt, sp.n_cells, _lib.C.byref(nb))
            self._cache[key] = torch.empty(max(int(nb.value), 16), dtype=torch.uint8, device=sp.device)
        ws = self._cache[key]
        _lib.call("nfem_le_dual_assemble", vt, sp.n_cells, sp.n_dof // 3, sp.dof_shift, _lib.ptr(sp.points),
                  _lib.ptr(sp.points_split), _lib.ptr(sp.cells), _lib.ptr(sp.rt_sign_mask), float(lam), float(mu),
                  _lib.ptr(f), Psi.ctypes.data_as(dp), mhat.ctypes.data_as(dp), divhat.ctypes.data_as(dp),
                  _lib.ptr(jacobian.inc_ptr), _lib.ptr(jacobian.inc), _lib.ptr(jacobian.node_codes),
                  _lib.ptr(jacobian.row_ptr), _lib.ptr(jacobian.values), _lib.ptr(residual), int(accumulate),
                  _lib.ptr(ws), ws.numel(), _lib.ptr(jacobian.status), _lib.stream_ptr(stream))


class LERieszMapWeakForm(WeakForm):
    """Riesz map of the mixed linear-elastic space s (RT1^3), u (P0^3),
    t (P0^3) on tetrahedra (src/weak_forms/le_riesz_map_weak_form.py:245-360,
    the preconditioning operator of the mixed elasticity drivers): per stress
    row the compliance 1/(2 mu) int psi_i . psi_j plus int div psi_i div psi_j,
    minus lambda / (2 mu (2 mu + 3 lambda)) int tr(psi) tr(psi) across the
    rows, and the P0 mass on u and t.  functions: "lambda", "mu" (constants
    or callables constant over the mesh; "rhs" is read by the reference but
    does not enter the operator).  Jacobian only."""

    cell_form = True
    NAMES = ("lambda", "mu")

    def _check_space(self):
        sp = self.space
        if sp is None or self.functions is None:
            raise ValueError
        if sp.names != ["s", "u", "t"] or sp.dim != 3:
            raise NotImplementedError("LERieszMapWeakForm expects fields ('s', 'u', 't') on tetrahedra")
        d = sp.discrete_spaces
        ok = (d["s"].family == "RT" and d["s"].k_order == 1 and d["u"].family == "Lagrange" and d["u"].k_order == 0
              and d["t"].family == "Lagrange" and d["t"].k_order == 0 and all(d[n].n_comp == 3 for n in sp.names))
        if not ok:
            raise NotImplementedError("LERieszMapWeakForm expects RT1^3 x P0^3 x P0^3")

    def coefficients(self, dtype):
        key = ("coef", dtype)
        if key in self._cache:
            return self._cache[key]
        par = []
        for k in self.NAMES:
            v = self.functions[k]
            if callable(v):
                xq = self.quadrature_points()
                vals = np.asarray(v(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64).ravel()
                if vals.size == 0 or np.abs(vals - vals[0]).max() > 1e-14 * max(1.0, np.abs(vals).max()):
                    raise NotImplementedError(f"{k} must be constant over the mesh (the device form takes one material)")
                par.append(float(vals[0]))
            else:
                par.append(float(np.ravel(v)[0]))
        from .elements import rt1_tet_tables
        Psi, mhat, divhat = rt1_tet_tables()
        out = (par[0], par[1], np.ascontiguousarray(Psi.reshape(-1)), np.ascontiguousarray(mhat.reshape(-1)),
               np.ascontiguousarray(divhat))
        self._cache[key] = out
        return out

    def assemble(self, jacobian, residual=None, accumulate=False, stream=None, coefficients=None):
        self._check_space()
        sp = self.space
        dtype = jacobian.dtype
        vt = _lib.NFEM_F64 if dtype == torch.float64 else _lib.NFEM_F32
        if jacobian.node_codes is None:
            raise NotImplementedError("matrix built without node codes")
        lam, mu, Psi, mhat, divhat = coefficients if coefficients is not None else self.coefficients(dtype)
        dp = _lib.C.POINTER(_lib.C.c_double)
        key = ("geom", dtype)
        if key not in self._cache:
            nb = _lib.C.c_size_t(0)
            _lib.call("nfem_cosserat_workspace_bytes", vt, sp.n_cells, _lib.C.byref(nb))
            self._cache[key] = torch.empty(max(int(nb.value), 16), dtype=torch.uint8, device=sp.device)
        ws = self._cache[key]
        _lib.call("nfem_le_riesz_assemble", vt, sp.n_cells, sp.n_dof // 3, sp.dof_shift, _lib.ptr(sp.points),
                  _lib.ptr(sp.points_split), _lib.ptr(sp.cells), _lib.ptr(sp.rt_sign_mask), float(lam), float(mu),
                  Psi.ctypes.data_as(dp), mhat.ctypes.data_as(dp), divhat.ctypes.data_as(dp),
                  _lib.ptr(jacobian.inc_ptr), _lib.ptr(jacobian.inc), _lib.ptr(jacobian.node_codes),
                  _lib.ptr(jacobian.row_ptr), _lib.ptr(jacobian.values), int(accumulate), _lib.ptr(ws), ws.numel(),
                  _lib.ptr(jacobian.status), _lib.stream_ptr(stream))
        if residual is not None and not accumulate:
            residual.zero_()


# ---------------------------------------------------------------- norms
_RT1_SIGMA = {2: np.array([-1.0, 1.0, -1.0]), 3: np.array([1.0, -1.0, 1.0, -1.0])}


def _field_tables(space, name):
    """(family code, n_phi, reference table, reference divergences) of a field
    at the space's quadrature points: Lagrange P0/P1/P2 values [Q, n_phi];
    RT1 values [Q, n_phi, dim] with the reference normal signs (psihat_i =
    sigma_i kappa (xhat - vhat_i), kappa = 2 on tetrahedra, 1 on triangles)
    and their divergences."""
    from .elements import lagrange_p2
    s = space.discrete_spaces[name]
    dim = space.dim
    pts, _ = space.quadrature[dim]
    if s.family == "Lagrange" and s.k_order in (0, 1, 2):
        if s.k_order == 0:
            tab = np.ones((pts.shape[0], 1))
        elif s.k_order == 1:
            tab = lagrange_p1_values(dim, pts)
        else:
            tab = lagrange_p2(dim, pts)[0]
        return 0, tab.shape[1], np.ascontiguousarray(tab), None
    if s.family == "RT" and s.k_order == 1:
        verts = np.vstack([np.zeros(dim), np.eye(dim)])
        kap = 2.0 if dim == 3 else 1.0
        sig = _RT1_SIGMA[dim]
        psi = kap * sig[None, :, None] * (pts[:, None, :] - verts[None, :, :])
        return 1, dim + 1, np.ascontiguousarray(psi), np.ascontiguousarray(kap * dim * sig)
    raise NotImplementedError(f"norms of a {s.family} k={s.k_order} field")


def _quad_x(space):
    pts, _ = space.quadrature[space.dim]
    lam = lagrange_p1_values(space.dim, pts)
    return np.einsum("qv,tvg->tqg", lam, space.mesh.points[space.cells_host])


def _eval_rows(fn, xq, rows):
    """f(x, y, z) on the [T, Q] point arrays -> [rows, ..., T, Q] float64."""
    T, Q = xq.shape[:2]
    v = np.asarray(fn(xq[..., 0], xq[..., 1], xq[..., 2]), dtype=np.float64)
    return v.reshape(rows, -1, T, Q)


def _field_error(space, name, quantity, exact_q, alpha, gamma_q=None, grad_gamma_q=None, stream=None):
    sp = space
    dim = sp.dim
    fam, n_phi, tab, div = _field_tables(sp, name)
    s = sp.discrete_spaces[name]
    pts, wts = sp.quadrature[dim]
    n_cmp = exact_q.shape[-1] if (fam == 0 or quantity == 0) else 1
    dev = sp.device
    ex = torch.as_tensor(np.ascontiguousarray(exact_q), dtype=torch.float64, device=dev)
    a = None if alpha is None else torch.as_tensor(alpha, dtype=torch.float64, device=dev).contiguous()
    g = None if gamma_q is None else torch.as_tensor(np.ascontiguousarray(gamma_q), dtype=torch.float64, device=dev)
    gg = None if grad_gamma_q is None else torch.as_tensor(np.ascontiguousarray(grad_gamma_q), dtype=torch.float64,
                                                           device=dev)
    nb = _lib.C.c_size_t(0)
    _lib.call("nfem_field_error_workspace_bytes", _lib.C.byref(nb))
    ws = torch.empty(int(nb.value) // 8 + 1, dtype=torch.float64, device=dev)
    out = torch.empty(1, dtype=torch.float64, device=dev)
    dp = _lib.C.POINTER(_lib.C.c_double)
    qw = np.ascontiguousarray(wts, dtype=np.float64)
    off = sp.field_slices[name].start
    _lib.call("nfem_field_error", dim, fam, quantity, sp.n_cells, _lib.ptr(sp.points), _lib.ptr(sp.cells),
              _lib.ptr(sp.rt_sign_mask) if fam == 1 else None, _lib.ptr(sp.cell_dofs), sp.n_loc, off, n_phi, s.n_comp,
              n_cmp, _lib.ptr(a), _lib.ptr(ex), _lib.ptr(g), _lib.ptr(gg), tab.ctypes.data_as(dp),
              None if div is None else div.ctypes.data_as(dp), qw.ctypes.data_as(dp), len(wts), _lib.ptr(out),
              _lib.ptr(ws), ws.numel() * 8, _lib.stream_ptr(stream))
    return float(out.item())


def _value_exact(space, name, fn, xq):
    s = space.discrete_spaces[name]
    dim = space.dim
    if s.family == "Lagrange":
        v = _eval_rows(fn, xq, 1).reshape(-1, *xq.shape[:2])  # [rows, T, Q]
        n_cmp = min(dim, s.n_comp, v.shape[0])
        return np.moveaxis(v[:n_cmp], 0, -1)  # [T, Q, n_cmp]
    v = _eval_rows(fn, xq, s.n_comp)[:, :dim]  # [n_comp, dim, T, Q]
    return np.moveaxis(np.moveaxis(v, 0, -1), 0, -1)  # [T, Q, n_comp, dim]


def l2_error(dim, space, functions, alpha, skip_fields=(), stream=None):
    """||u - u_h||_L2 of every field of the space, FP64 on the device, like
    l2_error (src/postprocess/l2_error_post_processor.py:7-63): Lagrange
    fields compare components 0..dim-1 (functions[name](x, y, z) -> [n, N]),
    RT1 fields every row (functions[name] -> [n_comp, 3, N], or [3, N] for one
    row).  Returns one value per field not in skip_fields, in field order."""
    sp = space
    xq = _quad_x(sp)
    out = []
    for name in sp.names:
        if name in skip_fields:
            continue
        out.append(_field_error(sp, name, 0, _value_exact(sp, name, functions[name], xq), alpha, stream=stream))
    return out


def l2_norm(dim, space, functions, skip_fields=(), stream=None):
    """||u||_L2 of the exact fields (solution_norms_post_processor.py:7-39),
    on the device: the l2_error kernel with no discrete solution."""
    return l2_error(dim, space, functions, None, skip_fields, stream)


def _rt_fields(space, skip_fields):
    return [n for n in space.names if space.discrete_spaces[n].family == "RT" and n not in skip_fields]


def div_error(dim, space, functions, alpha, skip_fields=(), stream=None):
    """||div u - div u_h||_L2 of every RT field (l2_error_post_processor.py:
    185-238); functions["div_" + name](x, y, z) -> [n_comp, N] (or [N])."""
    sp = space
    xq = _quad_x(sp)
    out = []
    for name in _rt_fields(sp, skip_fields):
        nc = sp.discrete_spaces[name].n_comp
        ex = np.moveaxis(_eval_rows(functions["div_" + name], xq, nc).reshape(nc, *xq.shape[:2]), 0, -1)
        out.append(_field_error(sp, name, 1, ex, alpha, stream=stream))
    return out


def div_norm(dim, space, functions, skip_fields=(), stream=None):
    """||div u||_L2 of the exact RT fields (solution_norms_post_processor.py:42-78)."""
    return div_error(dim, space, functions, None, skip_fields, stream)


def div_scaled_error(dim, space, functions, alpha, skip_fields=(), stream=None):
    """||div(l u) - div(l u_h)|| style error of l2_error_post_processor.py:
    240-306: the discrete divergence is grad l . psi + l div psi with
    functions["l"](x, y, z) -> [N] and functions["grad_l"] -> [dim, N]; an
    empty list when either is missing (as the reference skips)."""
    sp = space
    if functions.get("l") is None or functions.get("grad_l") is None:
        return []
    xq = _quad_x(sp)
    T, Q = xq.shape[:2]
    gam = _eval_rows(functions["l"], xq, 1).reshape(T, Q)
    ggam = np.moveaxis(_eval_rows(functions["grad_l"], xq, 1).reshape(-1, T, Q)[:sp.dim], 0, -1)
    out = []
    for name in _rt_fields(sp, skip_fields):
        nc = sp.discrete_spaces[name].n_comp
        ex = np.moveaxis(_eval_rows(functions["div_" + name], xq, nc).reshape(nc, T, Q), 0, -1)
        out.append(_field_error(sp, name, 2, ex, alpha, gam, ggam, stream=stream))
    return out
