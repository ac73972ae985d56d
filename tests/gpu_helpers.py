"""Helpers shared by the GPU parity tests."""
import numpy as np
import torch

import nfempy_gb300 as nf
from oracle import elements, forms, mesh_gen, quadrature, topology


def product_space(mesh_dict, fields, tags=(1,)):
    mesh = nf.Mesh(mesh_dict["dim"], data=mesh_dict)
    dim = mesh_dict["dim"]
    data = {n: (dim, nc, "Lagrange" if f == "P" else f, k, mesh) for n, f, k, nc, d in fields}
    sp = nf.ProductSpace(data)
    sp.make_subspaces_discontinuous({n: d for n, f, k, nc, d in fields})
    sp.build_structures({n: list(tags) for n, *_ in fields}, {})
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
