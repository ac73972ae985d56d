"""Benchmark workloads (synthetic inputs with the named sizes).

darcy3d(n): unit cube, n^3 hexahedra x 6 Kuhn tetrahedra, RT1 x P0,
  log K from a Gaussian random field (correlation length 0.05, sigma 2.0,
  sampled at cell centroids), source f = 1 per cell.  n = 64 gives
  1,572,864 tets, 4,743,168 DoF, nnz 36,200,448.
darcy2d_batch(n_problems): a batch of independent 2-D mixed Darcy
  problems assembled in one launch as one disjoint-union mesh: problem i is
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
