"""Helpers shared by the GPU parity tests."""
import numpy as np
import torch

import nfempy_gb300 as nf
from oracle import elements, forms, mesh_gen, quadrature, topology


def product_space(mesh_dict, fields, tags=(1,), b_tags=()):
    mesh = nf.Mesh(mesh_dict["dim"], data=mesh_dict)
    dim = mesh_dict["dim"]
    data = {n: (dim, nc, "Lagrange" if f == "P" else f, k, mesh) for n, f, k, nc, d in fields}
    sp = nf.ProductSpace(data)
    sp.make_subspaces_discontinuous({n: d for n, f, k, nc, d in fields})
    sp.build_structures({n: list(tags) for n, *_ in fields}, {n: list(b_tags) for n, *_ in fields} if b_tags else {})
    return sp


def darcy_oracle(mesh_dict, kappa_cell, f_callable=None, f_cell=None):
    """Oracle FP64 global matrix / residual for RT1 x P0 with per-cell kappa."""
    dim = mesh_dict["dim"]
    topo = topology.Topology(mesh_dict)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "RT", 1), topology.FieldSpec("p", "P", 0, 1, True)])
    X = mesh_dict["points"][topo.cells]
    s = topo.rt1_signs()
    quad = quadrature.make_quadrature(dim, 3)
    pts, _ = quad
    lam = elements.create_element("P", dim, 1).tabulate(0, pts)[0, :, :, 0]
    xq = np.einsum("qv,tvg->tqg", lam, X)
    if f_callable is not None:
        fq = f_callable(xq[..., 0], xq[..., 1], xq[..., 2])[0]
    elif f_cell is not None:
        fq = np.repeat(np.asarray(f_cell)[:, None], len(quad[1]), 1)
    else:
        fq = np.zeros(xq.shape[:2])
    kq = np.repeat(np.asarray(kappa_cell, dtype=np.float64)[:, None], len(quad[1]), 1)
    r, j = forms.darcy_batch(X, s, dim, quad, kq, fq)
    from oracle import assembly
    A, res = assembly.assemble_csr(cd, j, r, nd)
    return A, res, cd, nd, topo


def scaled_close(a, b, rtol):
    """|a - b| <= rtol * max(|b| over the row, 1e-300) entrywise on CSR data of equal pattern."""
    return np.abs(a - b) <= rtol * np.maximum(np.abs(b), 1e-300)


def incidences_of_rows(cell_dofs, rows):
    """(k, cell, local) for every occurrence of rows[k] in cell_dofs [T, n_loc]."""
    flat = np.asarray(cell_dofs).ravel()
    order = np.argsort(flat, kind="stable")
    sflat = flat[order]
    lo = np.searchsorted(sflat, rows, "left")
    hi = np.searchsorted(sflat, rows, "right")
    cnt = hi - lo
    k = np.repeat(np.arange(len(rows)), cnt)
    first = np.repeat(np.cumsum(cnt) - cnt, cnt)
    occ = order[np.repeat(lo, cnt) + (np.arange(int(cnt.sum())) - first)]
    n_loc = cell_dofs.shape[1]
    return k, occ // n_loc, occ % n_loc


def oracle_rows(cell_dofs, n_cols, rows, element_fn, chunk=20000):
    """The oracle's assembled rows `rows` (CSR [len(rows), n_cols], explicit
    zeros kept, columns sorted) and residual entries, from the element
    matrices of the incident cells only.  element_fn(cells) -> (r [U, n],
    j [U, n, n]) for an array of cell indices."""
    import scipy.sparse as sps
    k, c, a = incidences_of_rows(cell_dofs, rows)
    cells, inv = np.unique(c, return_inverse=True)
    n_loc = cell_dofs.shape[1]
    rs, js = [], []
    for s in range(0, len(cells), chunk):
        r, j = element_fn(cells[s:s + chunk])
        rs.append(r)
        js.append(j)
    r_el = np.concatenate(rs)
    j_el = np.concatenate(js)
    R = np.repeat(k, n_loc)
    C = np.asarray(cell_dofs)[c].ravel()
    V = j_el[inv, a, :].ravel()
    O = sps.csr_matrix((V, (R, C)), shape=(len(rows), n_cols))
    O.sum_duplicates()
    O.sort_indices()
    res = np.bincount(k, weights=r_el[inv, a], minlength=len(rows))
    return O, res


def gpu_rows(A, rows):
    """Rows `rows` of a device CSRMatrix as a host scipy CSR (float64), gathered
    on the device."""
    import scipy.sparse as sps
    rows_t = torch.as_tensor(np.asarray(rows, dtype=np.int64), device=A.row_ptr.device)
    rp = A.row_ptr.long()
    starts = rp[rows_t]
    lens = rp[rows_t + 1] - starts
    ptr = torch.zeros(len(rows) + 1, dtype=torch.int64, device=rp.device)
    ptr[1:] = torch.cumsum(lens, 0)
    idx = torch.repeat_interleave(starts - ptr[:-1], lens) + torch.arange(int(ptr[-1].item()), device=rp.device)
    cols = A.col_idx[idx].cpu().numpy()
    vals = A.values[idx].double().cpu().numpy()
    return sps.csr_matrix((vals, cols, ptr.cpu().numpy()), shape=(len(rows), A.n_rows))


def compare_rows(G, O, tol):
    """Pattern bit-exact, values within tol of each row's largest oracle entry.
    Returns the largest row-scaled error."""
    np.testing.assert_array_equal(G.indptr, O.indptr)
    np.testing.assert_array_equal(G.indices, O.indices)
    d = np.abs(G.data - O.data)
    rows = np.repeat(np.arange(O.shape[0]), np.diff(O.indptr))
    scale = np.zeros(O.shape[0])
    np.maximum.at(scale, rows, np.abs(O.data))
    err = (d / np.maximum(scale[rows], 1e-300)).max() if d.size else 0.0
    assert err <= tol, err
    return err


def sample_rows(n_rows, count, seed, extra=()):
    rng = np.random.default_rng(seed)
    rows = rng.choice(n_rows, size=min(count, n_rows), replace=False)
    return np.unique(np.concatenate([rows, np.asarray(extra, dtype=np.int64)]))


def quadrature_xq(X, dim, pts):
    lam = elements.create_element("P", dim, 1).tabulate(0, pts)[0, :, :, 0]
    return np.einsum("qv,tvg->tqg", lam, X)
