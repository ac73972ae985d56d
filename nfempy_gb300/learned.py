"""Learned preconditioner: a network that predicts the coarse pressure error.

No reference counterpart (nfempy has no learned component).  The plain
method is flexible GMRES with the cell-patch block Jacobi preconditioner
B.  One-level block Jacobi cannot remove smooth pressure errors, which is
why its iteration count grows with the mesh.  The learned preconditioner
adds a coarse correction computed by a 3-layer MLP (width 256, BF16
weights, FP32 accumulation):

    M(v) = B(v) + P (s * f([R v / s, k]))

  * aggregates: the cells binned by centroid into an n_c^3 grid;
  * R v: sum of v's pressure entries over each aggregate, s = ||R v||;
  * k: mean log-permeability of each aggregate;
  * f: the network, trained on (residual, error) pairs that the plain
    solver's own iterates give on sampled permeability fields: for an
    iterate x_j of a solve with solution x*, r_j = b - A x_j and the target
    is the aggregate mean of the pressure part of x* - x_j;
  * P: the predicted aggregate value added to the pressure DoFs of its cells.

The forward, backward and Adam kernels are the library's own
(nfem_mlp_forward / nfem_mlp_backward / nfem_adam_step); the preconditioner
runs inside the device FGMRES (NFEM_PC_LEARNED).  Plain block-Jacobi FGMRES
remains the fallback and the FP64 residual judges convergence.
"""
import numpy as np
import torch

from . import _lib


class CoarseGrid:
    """Cells of a space binned into an n_c^3 (or n_c^2) grid of aggregates."""

    def __init__(self, space, n_c):
        self.space = space
        self.n_c = int(n_c)
        dim = space.dim
        X = space.mesh.points[space.cells_host]
        cent = X.mean(axis=1)[:, :dim]
        lo = cent.min(axis=0)
        hi = cent.max(axis=0)
        idx = np.floor((cent - lo) / np.maximum(hi - lo, 1e-300) * self.n_c).astype(np.int64)
        idx = np.clip(idx, 0, self.n_c - 1)
        agg = np.zeros(space.n_cells, dtype=np.int64)
        for d in range(dim):
            agg = agg * self.n_c + idx[:, d]
        self.n_agg = self.n_c ** dim
        order = np.argsort(agg, kind="stable")
        counts = np.bincount(agg, minlength=self.n_agg)
        if np.any(counts == 0):
            raise ValueError("empty aggregate: choose a coarser grid")
        dev = space.device
        self.cell_agg_host = agg
        self.counts = counts
        self.cell_agg = torch.as_tensor(agg.astype(np.int32), device=dev)
        self.agg_cells = torch.as_tensor(order.astype(np.int32), device=dev)
        self.agg_ptr = torch.as_tensor(np.concatenate([[0], np.cumsum(counts)]).astype(np.int32), device=dev)
        self.p_base = space.field_offsets["p"]

    def features(self, kappa):
        logk = np.log(np.asarray(kappa, dtype=np.float64))
        f = np.bincount(self.cell_agg_host, weights=logk, minlength=self.n_agg) / self.counts
        return torch.as_tensor(f.astype(np.float32), device=self.space.device)

    def restrict_sum(self, v):
        """Aggregate sums of the pressure entries of v [.., n_dof] (torch, any device)."""
        p = v[..., self.p_base:self.p_base + self.space.n_cells]
        idx = torch.as_tensor(self.cell_agg_host, device=v.device)
        out = torch.zeros(v.shape[:-1] + (self.n_agg,), dtype=v.dtype, device=v.device)
        return out.index_add_(-1, idx, p)

    def restrict_mean(self, v):
        cnt = torch.as_tensor(self.counts, dtype=v.dtype, device=v.device)
        return self.restrict_sum(v) / cnt


class CoarseMLP:
    """The network f: [2 n_agg] -> [n_agg], dims {2 n_agg, width, width, n_agg}."""

    def __init__(self, n_agg, width=256, seed=0, device="cuda"):
        self.dims = np.array([2 * n_agg, width, width, n_agg], dtype=np.int32)
        self.dims_t = torch.as_tensor(self.dims)
        self.n_agg = n_agg
        n = _lib.C.c_int64(0)
        _lib.call("nfem_mlp_param_count", self._dims_ptr(), _lib.C.byref(n))
        self.n_params = int(n.value)
        rng = np.random.default_rng(seed)
        parts = []
        for a, b in ((self.dims[0], self.dims[1]), (self.dims[1], self.dims[2]), (self.dims[2], self.dims[3])):
            parts.append(rng.normal(0.0, np.sqrt(2.0 / a), (b, a)).ravel())
            parts.append(np.zeros(b))
        self.params = torch.as_tensor(np.concatenate(parts).astype(np.float32), device=device)
        assert self.params.numel() == self.n_params
        self.params_bf16 = torch.empty(self.n_params, dtype=torch.bfloat16, device=device)
        _lib.call("nfem_to_bf16", self.n_params, _lib.ptr(self.params), _lib.ptr(self.params_bf16),
                  _lib.stream_ptr())
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = 0

    def _dims_ptr(self):
        return _lib.C.c_void_p(self.dims_t.data_ptr())

    def forward(self, x, bf16=True):
        B = x.shape[0]
        h1 = torch.empty((B, int(self.dims[1])), device=x.device)
        h2 = torch.empty((B, int(self.dims[2])), device=x.device)
        y = torch.empty((B, int(self.dims[3])), device=x.device)
        if bf16:
            _lib.call("nfem_mlp_forward", self._dims_ptr(), _lib.NFEM_BF16, _lib.ptr(self.params_bf16),
                      _lib.ptr(self.params), B, _lib.ptr(x), _lib.ptr(h1), _lib.ptr(h2), _lib.ptr(y),
                      _lib.stream_ptr())
        else:
            _lib.call("nfem_mlp_forward", self._dims_ptr(), _lib.NFEM_F32, _lib.ptr(self.params), None, B,
                      _lib.ptr(x), _lib.ptr(h1), _lib.ptr(h2), _lib.ptr(y), _lib.stream_ptr())
        return h1, h2, y

    def train_step(self, x, t, lr=1e-3):
        """One Adam step on a batch (BF16 forward weights, FP32 master weights)."""
        B = x.shape[0]
        h1, h2, y = self.forward(x, bf16=True)
        wsb = _lib.C.c_size_t(0)
        _lib.call("nfem_mlp_backward_workspace_bytes", self._dims_ptr(), B, _lib.C.byref(wsb))
        if getattr(self, "_ws", None) is None or self._ws.numel() < int(wsb.value):
            self._ws = torch.empty(int(wsb.value), dtype=torch.uint8, device=x.device)
            self._g = torch.empty_like(self.params)
            self._loss = torch.zeros(1, dtype=torch.float64, device=x.device)
        _lib.call("nfem_mlp_backward", self._dims_ptr(), _lib.NFEM_BF16, _lib.ptr(self.params_bf16), B,
                  _lib.ptr(x), _lib.ptr(h1), _lib.ptr(h2), _lib.ptr(y), _lib.ptr(t), _lib.ptr(self._g),
                  _lib.ptr(self._ws), self._ws.numel(), _lib.ptr(self._loss), _lib.stream_ptr())
        self.step_count += 1
        _lib.call("nfem_adam_step", self.n_params, _lib.ptr(self.params), _lib.ptr(self._g), _lib.ptr(self.m),
                  _lib.ptr(self.v), _lib.C.c_float(lr), _lib.C.c_float(0.9), _lib.C.c_float(0.999),
                  _lib.C.c_float(1e-8), self.step_count, _lib.ptr(self.params_bf16), _lib.stream_ptr())
        return self._loss

    def state_dict(self):
        return {"dims": self.dims.tolist(), "params": self.params.cpu(), "m": self.m.cpu(), "v": self.v.cpu(),
                "step": self.step_count}

    def load_state_dict(self, st):
        assert list(st["dims"]) == self.dims.tolist()
        self.params.copy_(st["params"])
        self.m.copy_(st["m"])
        self.v.copy_(st["v"])
        self.step_count = int(st["step"])
        _lib.call("nfem_to_bf16", self.n_params, _lib.ptr(self.params), _lib.ptr(self.params_bf16),
                  _lib.stream_ptr())


def make_pairs(grid, A, b, x_star, snapshots, feat):
    """Training pairs from a solve: inputs [S, 2 n_agg], targets [S, n_agg] (FP32, device)."""
    from .solvers import KrylovSolver  # noqa: F401  (same device)
    S = snapshots.shape[0]
    xs = snapshots.double()
    r = b[None, :].expand(S, -1).clone()
    for s in range(S):
        r[s] = b - A.spmv(xs[s])
    e = x_star[None, :] - xs
    rc = grid.restrict_sum(r)
    ec = grid.restrict_mean(e)
    nrm = rc.norm(dim=1, keepdim=True).clamp_min(1e-300)
    x_in = torch.cat([rc / nrm, feat[None, :].double().expand(S, -1)], dim=1).float()
    tgt = (ec / nrm).float()
    keep = (nrm[:, 0] > 0) & torch.isfinite(tgt).all(dim=1)
    return x_in[keep], tgt[keep]


class LearnedPreconditioner:
    """Binds a trained CoarseMLP and a CoarseGrid to a KrylovSolver (pc="learned")."""

    def __init__(self, grid, model, kappa, out_scale=1.0):
        self.grid = grid
        self.model = model
        self.feat = grid.features(kappa)
        dims = model.dims
        self.work = torch.zeros(int(2 * grid.n_agg + dims[1] + dims[2] + 2 * grid.n_agg + 64),
                                dtype=torch.float32, device=grid.space.device)
        self.struct = _lib.LearnedCoarse(
            grid.p_base, grid.n_agg, (_lib.C.c_int32 * 4)(*[int(d) for d in dims]), _lib.ptr(grid.agg_ptr).value,
            _lib.ptr(grid.agg_cells).value, _lib.ptr(grid.cell_agg).value, _lib.ptr(self.feat).value,
            _lib.ptr(model.params_bf16).value, _lib.ptr(model.params).value, _lib.ptr(self.work).value,
            float(out_scale))


class DarcyProblem:
    """A Darcy RT1 x P0 space on cube(n) with reusable matrices (only K changes)."""

    def __init__(self, n, device="cuda"):
        from . import meshes, workloads
        from .assembly import CSRMatrix, LaplaceDualWeakForm
        self.n = n
        self.mesh = meshes.cube(n)
        self.space = workloads.darcy_space(self.mesh, device=device)
        cells = self.mesh["blocks"][-1][1]
        self.centroids = self.mesh["points"][cells].mean(axis=1)
        self.A = CSRMatrix(self.space, dtype=torch.float64)
        self.A32 = self.A.with_dtype(torch.float32)
        self.res = torch.empty(self.A.n_rows, dtype=torch.float64, device=device)
        self.res32 = torch.empty(self.A.n_rows, dtype=torch.float32, device=device)
        self.form = LaplaceDualWeakForm(self.space)

    def field(self, seed, corr_len=0.05, sigma=2.0):
        from . import meshes
        return np.exp(meshes.grf_log_field(self.centroids, corr_len, sigma, seed))

    def assemble(self, kappa, f=1.0):
        self.form.functions = {"kappa": kappa, "rhs": f}
        self.form.assemble(self.A, self.res)
        self.form.assemble(self.A32, self.res32)
        return -self.res


def generate_pairs(problem, grid, seeds, restart=30, max_snapshots=64, max_iters=20000, log=None):
    """Plain-solver (residual, error) pairs on the permeability fields of `seeds`."""
    from .solvers import KrylovSolver
    xs, ts, stats = [], [], []
    n = problem.A.n_rows
    snaps = torch.empty((max_snapshots, n), dtype=torch.float32, device=problem.A.values.device)
    for i, seed in enumerate(seeds):
        kappa = problem.field(seed)
        b = problem.assemble(kappa)
        ksp = KrylovSolver(problem.A, pc="cell_block", A32_values=problem.A32.values, restart=restart)
        x, info = ksp.solve(b, rtol=1e-8, max_inner=max_iters, raise_on_failure=False, snapshots=snaps)
        S = info.n_snapshots
        if S == 0 or info.status != 0:
            continue
        feat = grid.features(kappa)
        xi, ti = make_pairs(grid, problem.A, b, x, snaps[:S], feat)
        xs.append(xi)
        ts.append(ti)
        stats.append(info.inner_iterations)
        if log and (i % 50 == 0):
            log(f"field {i}: seed {seed} iters {info.inner_iterations} pairs {xi.shape[0]}")
    return torch.cat(xs), torch.cat(ts), stats


def train(model, X, T, steps=4000, batch=256, lr=1e-3, seed=0, log=None):
    """Adam on the pairs with the library's kernels; returns the loss history."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    N = X.shape[0]
    hist = []
    for s in range(steps):
        idx = torch.randint(0, N, (batch,), generator=g).to(X.device)
        cur_lr = lr * 0.5 * (1 + np.cos(np.pi * s / steps))
        loss = model.train_step(X[idx].contiguous(), T[idx].contiguous(), lr=cur_lr)
        if s % 200 == 0 or s == steps - 1:
            hist.append((s, float(loss.item())))
            if log:
                log(f"step {s} loss {hist[-1][1]:.4e}")
    return hist
