"""Learned preconditioner: a network that builds the coarse space of a
two-level method for mixed Darcy.

No reference counterpart (nfempy has no learned component).

The plain method is flexible GMRES with the cell-patch block Jacobi
preconditioner B.  Block Jacobi is one-level and cannot remove smooth
pressure errors, so its iteration count grows with the mesh.  The learned
preconditioner adds a Galerkin coarse correction (solvers.TwoLevelCoarse):

    z = B v;   z += P Ac^-1 P^T (v - A z),   Ac = P^T A P

where P prolongs one value per aggregate of cells to the pressure DoFs of
its cells (weight 1) and to the fluxes of the faces between aggregates
(weight w_f times the face's divergence coupling).  The classical
flux-extension weight is w_f = 1/|a_ff| (a lumped mass).  The network
predicts w_f from local features of the face:
  * log K of the two cells of the face;
  * the mean log K of the two aggregates;
  * log |a_ff| (normalised over the faces);
  * whether the face lies on the domain boundary;
  * the log K jump across the face.

Training data are (residual, correction) pairs that the plain method's own
solves give on sampled permeability fields.  For the iterates x_j of a
solve with solution x* and the coarse pressure error e_c(j) (aggregate
means of x* - x_j), the best weight of face f over the iterates is the
least-squares fit of the face's flux error against the prolonged coarse
error.  The network regresses log(w_f |a_ff|) on the face features.

Network: 3 layers, width 256, BF16 weights, FP32 accumulation.  Forward,
backward and Adam are the library's own kernels (nfem_mlp_forward /
nfem_mlp_backward / nfem_adam_step), checked against oracle/mlp.py.  Plain
block-Jacobi FGMRES stays the fallback, and the FP64 residual judges
convergence.
"""
import numpy as np
import torch

from . import _lib

N_FEAT = 8


class MLP:
    """dims {in, width, width, out}; FP32 master weights + BF16 inference copy."""

    def __init__(self, n_in, width=256, n_out=1, seed=0, device="cuda"):
        self.dims = np.array([n_in, width, width, n_out], dtype=np.int32)
        self.dims_t = torch.as_tensor(self.dims)
        n = _lib.C.c_int64(0)
        _lib.call("nfem_mlp_param_count", self._dims_ptr(), _lib.C.byref(n))
        self.n_params = int(n.value)
        rng = np.random.default_rng(seed)
        parts = []
        for a, b in ((self.dims[0], self.dims[1]), (self.dims[1], self.dims[2]), (self.dims[2], self.dims[3])):
            parts.append(rng.normal(0.0, np.sqrt(2.0 / a), (b, a)).ravel())
            parts.append(np.zeros(b))
        self.params = torch.as_tensor(np.concatenate(parts).astype(np.float32), device=device)
        self.params_bf16 = torch.empty(self.n_params, dtype=torch.bfloat16, device=device)
        _lib.call("nfem_to_bf16", self.n_params, _lib.ptr(self.params), _lib.ptr(self.params_bf16),
                  _lib.stream_ptr())
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step_count = 0
        self._ws = None

    def _dims_ptr(self):
        return _lib.C.c_void_p(self.dims_t.data_ptr())

    def forward(self, x):
        x = x.contiguous()
        B = x.shape[0]
        h1 = torch.empty((B, int(self.dims[1])), device=x.device)
        h2 = torch.empty((B, int(self.dims[2])), device=x.device)
        y = torch.empty((B, int(self.dims[3])), device=x.device)
        _lib.call("nfem_mlp_forward", self._dims_ptr(), _lib.NFEM_BF16, _lib.ptr(self.params_bf16),
                  _lib.ptr(self.params), B, _lib.ptr(x), _lib.ptr(h1), _lib.ptr(h2), _lib.ptr(y),
                  _lib.stream_ptr())
        return h1, h2, y

    def tensor_core_shape(self):
        """True when nfem_mlp_infer_tc covers the network (<= 16 inputs, two
        hidden layers of 256, one output)."""
        d = self.dims
        return int(d[0]) <= 16 and int(d[1]) == 256 and int(d[2]) == 256 and int(d[3]) == 1

    def infer_tc(self, x, status=None):
        """Network output [B, 1] from the fused tensor-core kernel."""
        x = x.contiguous().float()
        y = torch.empty((x.shape[0], 1), device=x.device)
        st = status if status is not None else torch.zeros(1, dtype=torch.int32, device=x.device)
        _lib.call("nfem_mlp_infer_tc", self._dims_ptr(), _lib.ptr(self.params_bf16), _lib.ptr(self.params),
                  x.shape[0], _lib.ptr(x), _lib.ptr(y), _lib.ptr(st), _lib.stream_ptr())
        if status is None and int(st.item()):
            raise _lib.NfemError(int(st.item()), "nfem_mlp_infer_tc")
        return y

    def predict(self, x, chunk=1 << 16):
        """Inference: the tensor-core kernel for the preconditioner's shape,
        else the tiled CUDA-core GEMMs in chunks."""
        if self.tensor_core_shape():
            return self.infer_tc(x)
        out = torch.empty((x.shape[0], int(self.dims[3])), device=x.device)
        for s in range(0, x.shape[0], chunk):
            out[s:s + chunk] = self.forward(x[s:s + chunk])[2]
        return out

    def train_step(self, x, t, lr=1e-3):
        """One Adam step on a batch (BF16 forward weights, FP32 master weights)."""
        B = x.shape[0]
        h1, h2, y = self.forward(x)
        wsb = _lib.C.c_size_t(0)
        _lib.call("nfem_mlp_backward_workspace_bytes", self._dims_ptr(), B, _lib.C.byref(wsb))
        if self._ws is None or self._ws.numel() < int(wsb.value):
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


class DarcyProblem:
    """Darcy RT1 x P0 on cube(n) with reusable FP64/FP32 matrices (only K changes)."""

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


class FaceData:
    """Faces of a TwoLevelCoarse prolongation (flux rows with P entries) and
    their features for a given permeability field."""

    def __init__(self, tl):
        A = tl.A
        sp = A.space
        dev = A.values.device
        self.tl = tl
        n_flux = tl.p_base
        p_agg = torch.as_tensor(tl.p_agg_host, device=dev)
        self.rows = torch.nonzero(p_agg[:n_flux, 0] >= 0).flatten()
        pairs = A.pairs.long()[self.rows]
        n_loc = sp.n_loc
        c0 = pairs[:, 0] // n_loc
        c1 = torch.where(pairs[:, 1] >= 0, pairs[:, 1] // n_loc, c0)
        self.cells = torch.stack([c0, c1], 1)
        self.boundary = (pairs[:, 1] < 0).float()
        cell_agg = torch.as_tensor(tl.cell_agg_host, device=dev)
        self.aggs = cell_agg[self.cells]
        self.counts = torch.as_tensor(tl.counts_host, dtype=torch.float64, device=dev)

    def features(self, kappa):
        tl = self.tl
        dev = self.rows.device
        logk = torch.as_tensor(np.log(np.asarray(kappa, dtype=np.float64)), device=dev)
        agg_logk = torch.zeros(tl.n_agg, dtype=torch.float64, device=dev)
        agg_logk.index_add_(0, torch.as_tensor(tl.cell_agg_host, device=dev), logk)
        agg_logk /= self.counts
        d = tl.A.diagonal()[self.rows].abs().clamp_min(1e-300).log()
        d = d - d.mean()
        lk = logk[self.cells]
        f = torch.stack([lk[:, 0], lk[:, 1], agg_logk[self.aggs[:, 0]], agg_logk[self.aggs[:, 1]], d,
                         self.boundary.double(), (lk[:, 0] - lk[:, 1]).abs(), torch.ones_like(d)], 1)
        return f.float().contiguous()


def csr_values_at(A, rows, cols):
    """A[rows[k], cols[k]] (0 where the pattern has no entry)."""
    rp = A.row_ptr.long()
    start = rp[rows]
    length = rp[rows + 1] - start
    L = int(length.max().item()) if rows.numel() else 0
    ar = torch.arange(L, device=rows.device)
    idx = (start[:, None] + ar[None, :]).clamp(max=max(A.nnz - 1, 0))
    valid = ar[None, :] < length[:, None]
    hit = valid & (A.col_idx[idx].long() == cols[:, None])
    return (A.values[idx].double() * hit).sum(1)


def face_targets(tl, faces, A, x_star, snapshots, rel_floor=1e-6):
    """Least-squares flux-extension weights of each face over the iterates,
    as log(w* |a_ff|); returns (targets, mask of faces with a usable fit)."""
    pb = tl.p_base
    n_cells = A.space.n_cells
    p_agg = torch.as_tensor(tl.p_agg_host, device=x_star.device)[faces.rows]
    coef = torch.zeros((faces.rows.numel(), 2), dtype=torch.float64, device=x_star.device)
    for sl in range(2):
        a = p_agg[:, sl]
        cell = torch.where(faces.aggs[:, 0] == a, faces.cells[:, 0], faces.cells[:, 1])
        coef[:, sl] = torch.where(a >= 0, -csr_values_at(A, faces.rows, pb + cell), torch.zeros_like(coef[:, sl]))
    e = x_star[None, :] - snapshots.double()
    cell_agg = torch.as_tensor(tl.cell_agg_host, device=e.device)
    ec = torch.zeros((e.shape[0], tl.n_agg), dtype=torch.float64, device=e.device)
    ec.index_add_(1, cell_agg, e[:, pb:pb + n_cells])
    ec /= faces.counts[None, :]
    g = torch.zeros((e.shape[0], faces.rows.numel()), dtype=torch.float64, device=e.device)
    for sl in range(2):
        a = p_agg[:, sl]
        ok = a >= 0
        g[:, ok] += coef[ok, sl][None, :] * ec[:, a[ok]]
    eu = e[:, faces.rows]
    num = (eu * g).sum(0)
    den = (g * g).sum(0)
    wstar = num / den.clamp_min(1e-300)
    good = (den > rel_floor * den.max()) & (wstar > 0)
    t = torch.log((wstar * tl.A.diagonal()[faces.rows].abs()).clamp_min(1e-30))
    return t.float(), good


def generate_pairs(problem, coarse_sizes, seeds, restart=30, max_snapshots=64, max_iters=20000,
                   faces_per_field=4096, log=None):
    """(features, targets) from plain solves on the permeability fields of `seeds`."""
    from .solvers import KrylovSolver, TwoLevelCoarse
    dev = problem.A.values.device
    n = problem.A.n_rows
    snaps = torch.empty((max_snapshots, n), dtype=torch.float32, device=dev)
    tls = [TwoLevelCoarse(problem.A, nc) for nc in coarse_sizes]
    faces = [FaceData(t) for t in tls]
    X, T, iters = [], [], []
    g = torch.Generator(device="cpu").manual_seed(1234)
    for i, seed in enumerate(seeds):
        kappa = problem.field(seed)
        b = problem.assemble(kappa)
        ksp = KrylovSolver(problem.A, pc="cell_block", A32_values=problem.A32.values, restart=restart)
        x, info = ksp.solve(b, rtol=1e-8, max_inner=max_iters, raise_on_failure=False, snapshots=snaps)
        S = info.n_snapshots
        if S == 0 or info.status != 0:
            continue
        iters.append(info.inner_iterations)
        for tl, fd in zip(tls, faces):
            t, good = face_targets(tl, fd, problem.A, x, snaps[:S])
            feat = fd.features(kappa)
            idx = torch.nonzero(good).flatten()
            if idx.numel() > faces_per_field:
                idx = idx[torch.randperm(idx.numel(), generator=g)[:faces_per_field].to(dev)]
            X.append(feat[idx])
            T.append(t[idx, None])
        if log and i % 50 == 0:
            log(f"field {i}: seed {seed} plain iters {info.inner_iterations}")
    return torch.cat(X), torch.cat(T), iters


def train(model, X, T, steps=3000, batch=512, lr=2e-3, seed=0, log=None):
    g = torch.Generator(device="cpu").manual_seed(seed)
    N = X.shape[0]
    hist = []
    for s in range(steps):
        idx = torch.randint(0, N, (batch,), generator=g).to(X.device)
        cur_lr = lr * 0.5 * (1 + np.cos(np.pi * s / steps))
        loss = model.train_step(X[idx].contiguous(), T[idx].contiguous(), lr=cur_lr)
        if s % 500 == 0 or s == steps - 1:
            hist.append((s, float(loss.item())))
            if log:
                log(f"step {s} loss {hist[-1][1]:.4e}")
    return hist


def learned_weights(tl, model, kappa, alpha=1.0):
    """Flux-extension weights w_f = exp(alpha * tau_f) / |a_ff| with tau the
    network's prediction (alpha = 0: the classical weights)."""
    faces = FaceData(tl)
    tau = model.predict(faces.features(kappa))[:, 0].double()
    w = tl.classical_weights().double().clone()
    w[faces.rows] = torch.exp(alpha * tau.clamp(-5.0, 5.0)) / tl.A.diagonal()[faces.rows].abs().clamp_min(1e-300)
    return w.float()


def select_alpha(model, problem, n_c, seed, alphas=(0.0, 0.25, 0.5, 1.0), max_iters=20000, log=None):
    """Scale of the network's correction chosen on a validation field (a seed
    used neither in training nor in testing): the alpha whose two-level
    preconditioner needs the fewest iterations to 1e-8.  alpha = 0 (the
    classical weights) is among the candidates, so the chosen preconditioner
    is never worse on the validation field than the classical one."""
    from .solvers import KrylovSolver, TwoLevelCoarse
    kappa = problem.field(seed)
    b = problem.assemble(kappa)
    best = None
    results = {}
    for a in alphas:
        tl = TwoLevelCoarse(problem.A, n_c)
        tl.set_weights(learned_weights(tl, model, kappa, a))
        ksp = KrylovSolver(problem.A, pc="two_level", A32_values=problem.A32.values, two_level=tl)
        x, info = ksp.solve(b, rtol=1e-8, max_inner=max_iters, raise_on_failure=False)
        it = info.inner_iterations if info.status == 0 else 10 ** 9
        results[a] = it
        if log:
            log(f"alpha {a}: {info.inner_iterations} iterations, status {info.status}")
        if best is None or it < results[best]:
            best = a
    return best, results
