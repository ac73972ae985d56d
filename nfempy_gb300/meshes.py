"""Synthetic meshes and coefficient fields for the benchmark workloads.

The reference reads gmsh meshes (src/mesh/mesh.py:13-19, :239-339); no gmsh
exists here, so these generators emit the same layout directly (points
[V, 3], blocks of (type, connectivity, physical tags), lower-dimensional
boundary blocks first as gmsh writes them):

  * square(n): unit square, n x n squares split along (0,0)->(1,1), triangles
    counter-clockwise, boundary lines counter-clockwise with tags
    2 (y=0), 3 (x=1), 4 (y=1), 5 (x=0); triangles tag 1.
  * cube(n): unit cube, n^3 hexahedra split into 6 positively oriented Kuhn
    tetrahedra along the main diagonal; boundary triangles tags
    2 (x=0), 3 (x=1), 4 (y=0), 5 (y=1), 6 (z=0), 7 (z=1); tetrahedra tag 1.

Coefficient fields (no reference counterpart; definitions are this
project's): log-permeability from a Gaussian random field with
squared-exponential covariance sigma^2 exp(-|x - y|^2 / (2 l^2)), sampled at
cell centroids through random Fourier features (Rahimi & Recht), seeded.
"""
import itertools

import numpy as np
import torch

BLOCK_DIM = {"vertex": 0, "line": 1, "triangle": 2, "tetra": 3}


def square(n):
    n = int(n)
    xs = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    points = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)

    def vid(i, j):
        return j * (n + 1) + i

    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    i, j = i.ravel(), j.ravel()
    v00, v10, v01, v11 = vid(i, j), vid(i + 1, j), vid(i, j + 1), vid(i + 1, j + 1)
    tris = np.stack([np.stack([v00, v10, v11], 1), np.stack([v00, v11, v01], 1)], 1).reshape(-1, 3)
    k = np.arange(n)
    blocks = [
        ("line", np.stack([vid(k, 0), vid(k + 1, 0)], 1), np.full(n, 2)),
        ("line", np.stack([vid(n, k), vid(n, k + 1)], 1), np.full(n, 3)),
        ("line", np.stack([vid(n - k, n), vid(n - k - 1, n)], 1), np.full(n, 4)),
        ("line", np.stack([vid(0, n - k), vid(0, n - k - 1)], 1), np.full(n, 5)),
        ("triangle", tris, np.full(tris.shape[0], 1)),
    ]
    return {"dim": 2, "points": points, "blocks": blocks}


def _kuhn():
    tets = []
    for perm in itertools.permutations(range(3)):
        p = [np.zeros(3, dtype=int)]
        for a in perm:
            q = p[-1].copy()
            q[a] = 1
            p.append(q)
        P = np.array(p)
        if np.linalg.det((P[1:] - P[0]).astype(float)) < 0:
            P[[1, 2]] = P[[2, 1]]
        tets.append(P)
    return np.array(tets)


def cube(n):
    n = int(n)
    m = n + 1
    xs = np.linspace(0.0, 1.0, m)
    Z, Y, X = np.meshgrid(xs, xs, xs, indexing="ij")
    points = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)

    def vid(i, j, k):
        return (k * m + j) * m + i

    kk, jj, ii = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    loc = _kuhn()
    tets = np.empty((ii.size, 6, 4), dtype=np.int64)
    for t in range(6):
        for v in range(4):
            o = loc[t, v]
            tets[:, t, v] = vid(ii + o[0], jj + o[1], kk + o[2])
    tets = tets.reshape(-1, 4)
    a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a, b = a.ravel(), b.ravel()

    def face(c00, c10, c01, c11, outward_ccw):
        t = np.stack([np.stack([c00, c10, c11], 1), np.stack([c00, c11, c01], 1)], 1).reshape(-1, 3)
        return t if outward_ccw else t[:, [0, 2, 1]]

    blocks = []
    for xv, tag, out in ((0, 2, False), (n, 3, True)):
        t = face(vid(xv, a, b), vid(xv, a + 1, b), vid(xv, a, b + 1), vid(xv, a + 1, b + 1), out)
        blocks.append(("triangle", t, np.full(t.shape[0], tag)))
    for yv, tag, out in ((0, 4, True), (n, 5, False)):
        t = face(vid(a, yv, b), vid(a + 1, yv, b), vid(a, yv, b + 1), vid(a + 1, yv, b + 1), out)
        blocks.append(("triangle", t, np.full(t.shape[0], tag)))
    for zv, tag, out in ((0, 6, False), (n, 7, True)):
        t = face(vid(a, b, zv), vid(a + 1, b, zv), vid(a, b + 1, zv), vid(a + 1, b + 1, zv), out)
        blocks.append(("triangle", t, np.full(t.shape[0], tag)))
    blocks.append(("tetra", tets, np.full(tets.shape[0], 1)))
    return {"dim": 3, "points": points, "blocks": blocks}


def union(meshes_list):
    """Disjoint union of meshes of one dimension: points concatenated (each
    mesh's vertex ids offset by the points before it), blocks of one type
    concatenated in mesh order with their tags.  The cells of mesh 0 come
    first, so first-appearance numbering gives each mesh a contiguous range
    of every entity block and the assembled system is block diagonal up to
    that interleaving of blocks.  Used for batches of independent problems
    assembled together (one cell pass and one row pass over all of them)."""
    dim = meshes_list[0]["dim"]
    pts, off = [], 0
    by_type = {}
    order = []
    for m in meshes_list:
        if m["dim"] != dim:
            raise ValueError("union: meshes of different dimensions")
        pts.append(np.asarray(m["points"], dtype=np.float64))
        for typ, conn, tags in m["blocks"]:
            if typ not in by_type:
                by_type[typ] = ([], [])
                order.append(typ)
            by_type[typ][0].append(np.asarray(conn, dtype=np.int64) + off)
            by_type[typ][1].append(np.asarray(tags))
        off += pts[-1].shape[0]
    order.sort(key=lambda t: BLOCK_DIM[t])
    blocks = [(t, np.concatenate(by_type[t][0]), np.concatenate(by_type[t][1])) for t in order]
    return {"dim": dim, "points": np.concatenate(pts), "blocks": blocks}


def grf_log_field(x, corr_len, sigma, seed, n_features=512, device=None, chunk=1 << 20):
    """Gaussian random field values at points x [N, 3] (numpy or torch).

    Random Fourier features for the squared-exponential covariance:
    g(x) = sigma * sqrt(2 / M) * sum_m cos(w_m . x + b_m), w_m ~ N(0, I / l^2),
    b_m ~ U(0, 2 pi).  Deterministic for a given seed.  Returns float64 numpy.
    """
    gen = np.random.default_rng(int(seed))
    w = gen.normal(0.0, 1.0 / float(corr_len), size=(n_features, 3))
    b = gen.uniform(0.0, 2.0 * np.pi, size=n_features)
    dev = device if device is not None else ("cuda" if torch.cuda.is_available() else "cpu")
    W = torch.as_tensor(w, dtype=torch.float64, device=dev)
    B = torch.as_tensor(b, dtype=torch.float64, device=dev)
    X = torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev)
    out = torch.empty(X.shape[0], dtype=torch.float64, device=dev)
    for s in range(0, X.shape[0], chunk):
        out[s:s + chunk] = torch.cos(X[s:s + chunk] @ W.T + B).sum(dim=1)
    out *= float(sigma) * np.sqrt(2.0 / n_features)
    return out.cpu().numpy()


def cells_of_dim(mesh, dim, physical_tags=None):
    conns, tags = [], []
    for typ, conn, phys in mesh["blocks"]:
        if BLOCK_DIM[typ] == dim:
            conns.append(np.asarray(conn, dtype=np.int64))
            tags.append(np.asarray(phys))
    conn = np.concatenate(conns, axis=0)
    tag = np.concatenate(tags)
    if physical_tags is not None and list(physical_tags) != [None]:
        keep = np.isin(tag, np.asarray(physical_tags))
        conn, tag = conn[keep], tag[keep]
    return conn, tag
