"""The flux-extension weights of the two-level preconditioner at their
optimum: the exact harmonic (energy-minimising) extension of the aggregate
pressures, which any learned face weight could at best approximate, takes
as many GMRES iterations as the classical weights w_f = 1/|a_ff|.

Host experiment on the oracle's matrices (mixed Darcy RT1 x P0, log-normal
K, sigma 2): the same symmetric two-level cycle as solvers.TwoLevelCoarse
(damped cell-block smoother, Galerkin coarse correction, smoother again)
inside scipy GMRES(30) to 1e-8."""
import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla

from oracle import assembly, forms, mesh_gen, quadrature, topology
from oracle.solve import cell_block_jacobi


def grf(cent, corr, sigma, seed):
    """Smooth log field: a sum of random Fourier modes (host restatement for
    the experiment, not the library's generator)."""
    rng = np.random.default_rng(seed)
    k = rng.normal(0.0, 1.0 / corr, (64, 3))
    ph = rng.uniform(0, 2 * np.pi, 64)
    f = np.cos(cent @ k.T + ph).sum(axis=1)
    return sigma * f / f.std()


def darcy_system(n, seed):
    m = mesh_gen.cube(n)
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "RT", 1), topology.FieldSpec("p", "P", 0, 1, True)])
    X = m["points"][topo.cells]
    quad = quadrature.make_quadrature(3, 3)
    cent = X.mean(axis=1)
    kq = np.repeat(np.exp(grf(cent, 0.1, 2.0, seed))[:, None], len(quad[1]), 1)
    r, j = forms.darcy_batch(X, topo.rt1_signs(), 3, quad, kq, np.ones_like(kq))
    A, res = assembly.assemble_csr(cd, j, r, nd)
    return A.tocsr(), -res, cd, cent


def prolongation(A, cd, agg, n_agg, w):
    """P: aggregate value -> its cells' pressures (1) and the flux rows of
    faces between aggregates or on the boundary (-w_f times the row's entries
    in the aggregate's pressure columns)."""
    n = A.shape[0]
    T = cd.shape[0]
    pb = int(cd[:, 4].min())
    rows, cols, vals = list(cd[:, 4]), list(agg), [1.0] * T
    faces = cd[:, :4].ravel()
    fagg = np.repeat(agg, 4)
    cnt = np.bincount(faces, minlength=n)
    seen = {}
    for f, a in zip(faces, fagg):
        seen.setdefault(int(f), set()).add(int(a))
    for f, aset in seen.items():
        if cnt[f] == 2 and len(aset) == 1:
            continue
        row = A[f]
        for a in aset:
            s = sum(v for c, v in zip(row.indices, row.data) if c >= pb and agg[c - pb] == a)
            rows.append(f)
            cols.append(a)
            vals.append(-w[f] * s)
    return sps.csr_matrix((vals, (rows, cols)), shape=(n, n_agg))


def two_level_its(A, b, cd, P, omega=0.9):
    B = cell_block_jacobi(A, cd)
    Aci = np.linalg.inv((P.T @ A @ P).toarray())

    def apply(v):
        z = omega * B(v)
        z = z + P @ (Aci @ (P.T @ (v - A @ z)))
        return z + omega * B(v - A @ z)
    k = [0]

    def cb(_):
        k[0] += 1
    x, _ = spla.gmres(A, b, M=spla.LinearOperator(A.shape, matvec=apply), rtol=1e-8, atol=0.0, restart=30,
                      maxiter=100, callback=cb, callback_type="pr_norm")
    assert np.linalg.norm(b - A @ x) <= 1e-7 * np.linalg.norm(b)
    return k[0]


@pytest.mark.parametrize("seed", [1, 2])
def test_harmonic_extension_does_not_beat_classical_weights(seed):
    n, nc = 6, 3
    A, b, cd, cent = darcy_system(n, seed)
    lo, hi = cent.min(0), cent.max(0)
    idx = np.clip(np.floor((cent - lo) / (hi - lo) * nc).astype(int), 0, nc - 1)
    agg = (idx[:, 0] * nc + idx[:, 1]) * nc + idx[:, 2]
    n_agg = nc ** 3
    pb = int(cd[:, 4].min())
    w = np.zeros(A.shape[0])
    w[:pb] = 1.0 / np.abs(A.diagonal()[:pb])
    classical = two_level_its(A, b, cd, prolongation(A, cd, agg, n_agg, w))
    Pp = sps.csr_matrix((np.ones(len(agg)), (np.arange(len(agg)), agg)), shape=(len(agg), n_agg))
    U = -spla.splu(A[:pb, :pb].tocsc()).solve((A[:pb, pb:] @ Pp).toarray())
    ideal = two_level_its(A, b, cd, sps.vstack([sps.csr_matrix(U), Pp]).tocsr())
    halved = two_level_its(A, b, cd, prolongation(A, cd, agg, n_agg, 0.5 * w))
    # the exact extension gains nothing over the classical weights, and a
    # weight far from them costs iterations
    assert ideal >= classical - 2, (ideal, classical)
    assert halved > classical, (halved, classical)
