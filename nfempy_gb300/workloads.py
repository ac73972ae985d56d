"""Benchmark workloads (synthetic inputs with the named sizes).

darcy3d(n): unit cube, n^3 hexahedra x 6 Kuhn tetrahedra, RT1 x P0,
  log K from a Gaussian random field (correlation length 0.05, sigma 2.0,
  sampled at cell centroids), source f = 1 per cell.  n = 64 gives
  1,572,864 tets, 4,743,168 DoF, nnz 36,200,448.
darcy2d_batch(n_problems): a batch of independent 2-D mixed Darcy
  problems assembled together as one disjoint-union mesh: problem i is
  the unit square with n_i x n_i squares x 2 triangles, n_i ~ U{8..128},
  log K_i a Gaussian random field (correlation length 0.1, sigma 1.0,
  seed + i) at the cell centroids, f = 1.  512 problems give about 15 M DoF.
darcy2d(n): unit square, n x n squares x 2 triangles, RT1 x P0, K = 1,
  f = 2 pi^2 sin(pi x) sin(pi y) at the quadrature points (n = 32: 2,048
  triangles, 5,184 DoF).
Seeds: 20261203 + configuration index.
"""
import numpy as np

from . import meshes
from .spaces import Mesh, ProductSpace

SEED = 20261203


def darcy_space(mesh_dict, dof_shift=0, device=None):
    dim = mesh_dict["dim"]
    mesh = Mesh(dim, data=mesh_dict)
    sp = ProductSpace({"u": (dim, 1, "RT", 1, mesh), "p": (dim, 1, "Lagrange", 0, mesh)}, device=device)
    sp.make_subspaces_discontinuous({"u": False, "p": True})
    sp.dof_shift = dof_shift
    sp.build_structures({"u": [1], "p": [1]}, {})
    return sp


def darcy3d_coefficients(mesh_dict, corr_len=0.05, sigma=2.0, seed=SEED + 5):
    cells = mesh_dict["blocks"][-1][1]
    centroids = mesh_dict["points"][cells].mean(axis=1)
    logk = meshes.grf_log_field(centroids, corr_len, sigma, seed)
    return np.exp(logk), np.ones(cells.shape[0])


def darcy3d(n=64, device=None):
    m = meshes.cube(n)
    sp = darcy_space(m, device=device)
    kappa, f = darcy3d_coefficients(m)
    return m, sp, kappa, f


def darcy2d_batch(n_problems=512, n_min=8, n_max=128, corr_len=0.1, sigma=1.0, seed=SEED + 3, device=None):
    rng = np.random.default_rng(seed)
    sides = rng.integers(n_min, n_max + 1, size=n_problems)
    ms, kappas = [], []
    for i, n in enumerate(sides):
        m = meshes.square(int(n))
        cells = m["blocks"][-1][1]
        centroids = m["points"][cells].mean(axis=1)
        kappas.append(np.exp(meshes.grf_log_field(centroids, corr_len, sigma, seed + 1 + i, device="cpu")))
        ms.append(m)
    u = meshes.union(ms)
    sp = darcy_space(u, device=device)
    kappa = np.concatenate(kappas)
    return u, sp, kappa, np.ones(kappa.shape[0]), sides


def batch_aggregates(sides, k=4, size=None, blocks=False):
    """Per-problem coarse aggregates of a darcy2d_batch union: problem i's
    n_i x n_i square split into k x k blocks of squares (two triangles per
    square, in meshes.square's cell order), aggregate ids offset per problem,
    so no aggregate spans two problems.  size: aggregates of about size x size
    squares instead (k_i = round(n_i / size), at least 1).  blocks=True also
    returns the [n_problems + 1] aggregate offsets of the problems, the
    diagonal blocks of the coarse matrix."""
    out, ptr = [], [0]
    for n in sides:
        n = int(n)
        kk = min(k, n) if size is None else max(1, min(n, int(round(n / size))))
        sq = np.arange(n * n)
        i, j = sq % n, sq // n
        loc = (j * kk // n) * kk + (i * kk // n)
        out.append(np.repeat(loc, 2) + ptr[-1])
        ptr.append(ptr[-1] + kk * kk)
    agg = np.concatenate(out)
    return (agg, np.asarray(ptr, dtype=np.int64)) if blocks else agg


def elasticity3d(n=40, device=None):
    """Vector P2 linear elasticity on the unit cube, n^3 x 6 tetrahedra:
    per-cell Lame lambda and mu = exp(N(0, 0.5^2)) (lambda drawn first, seed
    20261203 + 1), body force (1, 1, 1).  n = 40 gives 384,000 tets,
    1,594,323 DoF.  Returns (mesh dict, space, functions)."""
    m = meshes.cube(n)
    mesh = Mesh(3, data=m)
    sp = ProductSpace({"u": (3, 3, "Lagrange", 2, mesh)}, device=device)
    sp.build_structures({"u": [1]}, {})
    rng = np.random.default_rng(SEED + 1)
    T = sp.n_cells
    functions = {"lambda": np.exp(rng.normal(0, 0.5, T)), "mu": np.exp(rng.normal(0, 0.5, T)),
                 "rhs": np.array([1.0, 1.0, 1.0])}
    return m, sp, functions


COSSERAT_MATERIAL = dict(lambda_s=1.0, mu_s=1.0, kappa_s=0.5, lambda_o=1.0, mu_o=1.0, kappa_o=0.5, l=1.0)
COSSERAT_U = np.array([1.0, -0.5, 0.75])      # u = a phi
COSSERAT_THETA = np.array([0.3, 0.6, -0.45])  # theta = b phi


def _bubble(x, y, z):
    """phi = sin(pi x) sin(pi y) sin(pi z), its gradient [3, ...] and Hessian [3, 3, ...]."""
    sx, sy, sz = np.sin(np.pi * x), np.sin(np.pi * y), np.sin(np.pi * z)
    cx, cy, cz = np.cos(np.pi * x), np.cos(np.pi * y), np.cos(np.pi * z)
    p2 = np.pi * np.pi
    phi = sx * sy * sz
    g = np.pi * np.array([cx * sy * sz, sx * cy * sz, sx * sy * cz])
    H = p2 * np.array([[-phi, cx * cy * sz, cx * sy * cz],
                       [cx * cy * sz, -phi, sx * cy * cz],
                       [cx * sy * cz, sx * cy * cz, -phi]])
    return phi, g, H


def _skew_of(v):
    """S(v) with (theta, Asym tau) = S(theta) : tau, Asym tau = (tau21 - tau12,
    tau02 - tau20, tau10 - tau01) (the (t, s) coupling of
    lce_dual_weak_form.py:562-580)."""
    z = np.zeros_like(v[0])
    return np.array([[z, -v[2], v[1]], [v[2], z, -v[0]], [-v[1], v[0], z]])


def _constitutive(G, mu, kappa, lam):
    """C e = 2 mu sym e + 2 kappa skew e + lambda tr(e) I (the inverse of the
    form's compliance 1/(2 mu) sym + 1/(2 kappa) skew - lambda/(2 mu (2 mu + 3
    lambda)) tr I), applied on the two leading axes."""
    Gt = np.swapaxes(G, 0, 1)
    tr = np.trace(G, axis1=0, axis2=1)
    eye = np.eye(3).reshape((3, 3) + (1,) * (G.ndim - 2))
    return mu * (G + Gt) + kappa * (G - Gt) + lam * tr * eye


def cosserat_manufactured(par=None):
    """Smooth manufactured solution of the mixed Cosserat system assembled by
    LCEDualWeakForm (unit cube, u = theta = 0 on the boundary, which the dual
    form imposes naturally).  With the form's blocks, A x = -r reads
      A_s sigma = grad u + S(theta),   A_o omega / l = grad theta,
      div sigma = f_u,                 div omega - Asym sigma = f_t,
    so u = a phi, theta = b phi (phi = sin pi x sin pi y sin pi z) give
      sigma = C_s(a (x) grad phi + phi S(b)),  omega = l C_o(b (x) grad phi)
    and the load below.  Returns (rhs f(x, y, z) -> [6, N], exact fields
    {"u", "t", "s", "m"}: f(x, y, z) -> [3, N] or [3, 3, N])."""
    p = dict(COSSERAT_MATERIAL if par is None else par)
    a, b = COSSERAT_U, COSSERAT_THETA
    Sb = _skew_of(b.reshape(3, 1))[..., 0]

    def parts(x, y, z):
        phi, g, H = _bubble(np.asarray(x, dtype=np.float64), np.asarray(y, dtype=np.float64),
                            np.asarray(z, dtype=np.float64))
        ex = (slice(None),) * 2 + (None,) * phi.ndim
        G = a[:, None, None] * g[None, :] if phi.ndim == 0 else np.einsum("i,j...->ij...", a, g)
        G = G + Sb[ex] * phi
        sigma = _constitutive(G, p["mu_s"], p["kappa_s"], p["lambda_s"])
        # dG[j, i, k] = d_j G_ik = a_i H_kj + g_j S_ik
        dG = np.einsum("i,kj...->jik...", a, H) + np.einsum("j...,ik->jik...", g, Sb)
        dsig = np.stack([_constitutive(dG[j], p["mu_s"], p["kappa_s"], p["lambda_s"]) for j in range(3)])
        div_sigma = np.einsum("jij...->i...", dsig)
        gt = np.einsum("i,j...->ij...", b, g)
        omega = p["l"] * _constitutive(gt, p["mu_o"], p["kappa_o"], p["lambda_o"])
        dgt = np.einsum("i,kj...->jik...", b, H)
        dom = np.stack([_constitutive(dgt[j], p["mu_o"], p["kappa_o"], p["lambda_o"]) for j in range(3)])
        div_omega = p["l"] * np.einsum("jij...->i...", dom)
        asym = np.array([sigma[2, 1] - sigma[1, 2], sigma[0, 2] - sigma[2, 0], sigma[1, 0] - sigma[0, 1]])
        return phi, sigma, omega, div_sigma, div_omega - asym

    def rhs(x, y, z):
        _, _, _, fu, ft = parts(x, y, z)
        return np.concatenate([fu, ft], axis=0)

    exact = {"u": lambda x, y, z: np.einsum("i,...->i...", a, parts(x, y, z)[0]),
             "t": lambda x, y, z: np.einsum("i,...->i...", b, parts(x, y, z)[0]),
             "s": lambda x, y, z: parts(x, y, z)[1],
             "m": lambda x, y, z: parts(x, y, z)[2]}
    return rhs, exact


def cosserat3d(n=24, device=None):
    """Mixed Cosserat elasticity on the unit cube, n^3 x 6 tetrahedra: s, m in
    RT1 (three rows each), u, t in P0^3; Lame 1/1, Cosserat coupling 0.5,
    l = 1, load of the manufactured solution (cosserat_manufactured), the
    material given as callables like the reference drivers.  n = 24 gives
    82,944 tets, 1,513,728 DoF.  Returns (mesh dict, space, functions,
    exact fields)."""
    m = meshes.cube(n)
    mesh = Mesh(3, data=m)
    sp = ProductSpace({"s": (3, 3, "RT", 1, mesh), "m": (3, 3, "RT", 1, mesh), "u": (3, 3, "Lagrange", 0, mesh),
                       "t": (3, 3, "Lagrange", 0, mesh)}, device=device)
    sp.make_subspaces_discontinuous({"u": True, "t": True})
    sp.build_structures({k: [1] for k in "smut"}, {})
    rhs, exact = cosserat_manufactured()
    functions = {k: (lambda v: (lambda x, y, z: np.full(np.shape(x), v)))(v) for k, v in COSSERAT_MATERIAL.items()}
    functions["rhs"] = rhs
    return m, sp, functions, exact
