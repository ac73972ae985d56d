"""Scatter of element matrices into a global CSR matrix (oracle).

Restates the library scatter (src/assembly/ScatterFormData.py:5-25): every
entry of every element clique is added, zeros included, with
row = repeat(dest, n) and col = tile(dest, n) ("pattern A"), and the
residual is accumulated with repeated-index-safe adds.  The driver variant
("pattern B", examples/cauchy_elasticity/cg_elasticity_example_1.py:92-122)
drops |v| <= 1e-8 (np.isclose(v, 1e-16) with its default atol), keeps
row <= col for SBAIJ storage and adds explicit zero diagonals.
"""
import numpy as np
import scipy.sparse as sp


def clique_coo(cell_dofs):
    cell_dofs = np.asarray(cell_dofs, dtype=np.int64)
    T, n = cell_dofs.shape
    rows = np.repeat(cell_dofs, n, axis=1).ravel()
    cols = np.tile(cell_dofs, (1, n)).ravel()
    return rows, cols


def pattern_csr(cell_dofs, n_dof):
    """Sparsity pattern A: indptr, indices (sorted per row)."""
    rows, cols = clique_coo(cell_dofs)
    key = np.unique(rows * np.int64(n_dof) + cols)
    r = key // n_dof
    c = key % n_dof
    indptr = np.zeros(n_dof + 1, dtype=np.int64)
    np.add.at(indptr, r + 1, 1)
    return np.cumsum(indptr), c


def assemble_csr(cell_dofs, j_el, r_el, n_dof):
    """Global matrix (pattern A, values summed) and residual vector."""
    rows, cols = clique_coo(cell_dofs)
    key = rows * np.int64(n_dof) + cols
    uk, inv = np.unique(key, return_inverse=True)
    vals = np.zeros(uk.size)
    np.add.at(vals, inv.ravel(), np.asarray(j_el).reshape(-1))
    r = uk // n_dof
    indptr = np.zeros(n_dof + 1, dtype=np.int64)
    np.add.at(indptr, r + 1, 1)
    A = sp.csr_matrix((vals, uk % n_dof, np.cumsum(indptr)), shape=(n_dof, n_dof))
    res = np.zeros(n_dof)
    np.add.at(res, np.asarray(cell_dofs).ravel(), np.asarray(r_el).ravel())
    return A, res


def pattern_b(cell_dofs, j_el, n_dof, symmetric=True, atol=1e-8):
    """Driver filter: |v| > atol (np.isclose default), row <= col, zero diagonals."""
    rows, cols = clique_coo(cell_dofs)
    v = np.asarray(j_el).reshape(-1)
    keep = ~np.isclose(v, 1e-16)
    if symmetric:
        keep &= rows <= cols
    d = np.unique(np.asarray(cell_dofs).ravel())
    r = np.concatenate([rows[keep], d])
    c = np.concatenate([cols[keep], d])
    key = np.unique(r * np.int64(n_dof) + c)
    rr = key // n_dof
    indptr = np.zeros(n_dof + 1, dtype=np.int64)
    np.add.at(indptr, rr + 1, 1)
    return np.cumsum(indptr), key % n_dof
