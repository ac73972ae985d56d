"""Synthetic simplex meshes in the gmsh/meshio layout the reference ingests (oracle copy).

The reference reads a gmsh file through meshio (src/mesh/mesh.py:13-19) and
walks its cell blocks in file order (src/mesh/mesh.py:334-337).  These
generators emit the same layout directly: points [V, 3] and a list of blocks
(type, connectivity, physical tags).  Lower-dimensional boundary blocks come
first, as gmsh writes them; that order fixes the stored node order of
boundary edges, which the 2-D orientation rule reads
(src/basis/permute_and_transform.py:8-19).

  * square(n): unit square, n x n squares split along (0,0)->(1,1); triangles
    counter-clockwise; boundary lines counter-clockwise around the domain,
    tags 2 (y=0), 3 (x=1), 4 (y=1), 5 (x=0); triangles tag 1.
  * cube(n): unit cube, n^3 hexahedra split into 6 Kuhn tetrahedra along the
    main diagonal, all positively oriented; boundary triangles follow the
    induced face diagonals, tags 2 (x=0), 3 (x=1), 4 (y=0), 5 (y=1),
    6 (z=0), 7 (z=1); tetrahedra tag 1.

The product package carries its own generator (nfempy_gb300/meshes.py); the
tests check that both produce identical arrays.
"""
import itertools

import numpy as np


def square(n):
    n = int(n)
    xs = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    points = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size)], axis=1)

    def vid(i, j):
        return j * (n + 1) + i

    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    i = i.ravel()
    j = j.ravel()
    v00, v10, v01, v11 = vid(i, j), vid(i + 1, j), vid(i, j + 1), vid(i + 1, j + 1)
    t0 = np.stack([v00, v10, v11], axis=1)
    t1 = np.stack([v00, v11, v01], axis=1)
    tris = np.stack([t0, t1], axis=1).reshape(-1, 3)

    k = np.arange(n)
    bottom = np.stack([vid(k, 0), vid(k + 1, 0)], axis=1)
    right = np.stack([vid(n, k), vid(n, k + 1)], axis=1)
    top = np.stack([vid(n - k, n), vid(n - k - 1, n)], axis=1)
    left = np.stack([vid(0, n - k), vid(0, n - k - 1)], axis=1)
    blocks = [
        ("line", bottom, np.full(n, 2)),
        ("line", right, np.full(n, 3)),
        ("line", top, np.full(n, 4)),
        ("line", left, np.full(n, 5)),
        ("triangle", tris, np.full(tris.shape[0], 1)),
    ]
    return {"dim": 2, "points": points, "blocks": blocks}


def _kuhn_local():
    """The 6 Kuhn tetrahedra of the unit cube as corner offsets, det > 0."""
    tets = []
    for perm in itertools.permutations(range(3)):
        p = [np.zeros(3, dtype=int)]
        for a in perm:
            q = p[-1].copy()
            q[a] = 1
            p.append(q)
        P = np.array(p)
        d = np.linalg.det((P[1:] - P[0]).astype(float))
        if d < 0:
            P[[1, 2]] = P[[2, 1]]
        tets.append(P)
    return np.array(tets)  # [6, 4, 3]


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
    loc = _kuhn_local()
    tets = np.empty((ii.size, 6, 4), dtype=np.int64)
    for t in range(6):
        for v in range(4):
            o = loc[t, v]
            tets[:, t, v] = vid(ii + o[0], jj + o[1], kk + o[2])
    tets = tets.reshape(-1, 4)

    a, b = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a, b = a.ravel(), b.ravel()

    def face_tris(c00, c10, c01, c11, outward_ccw):
        # square split along its min->max diagonal c00 -> c11
        t0 = np.stack([c00, c10, c11], axis=1)
        t1 = np.stack([c00, c11, c01], axis=1)
        t = np.stack([t0, t1], axis=1).reshape(-1, 3)
        if not outward_ccw:
            t = t[:, [0, 2, 1]]
        return t

    blocks = []
    # x = 0 and x = 1: in-plane axes (y, z); normal of (y, z) ccw is +x
    for xval, tag, out in ((0, 2, False), (n, 3, True)):
        t = face_tris(vid(xval, a, b), vid(xval, a + 1, b), vid(xval, a, b + 1),
                      vid(xval, a + 1, b + 1), out)
        blocks.append(("triangle", t, np.full(t.shape[0], tag)))
    # y = 0 and y = 1: in-plane axes (x, z); normal of (x, z) ccw is -y
    for yval, tag, out in ((0, 4, True), (n, 5, False)):
        t = face_tris(vid(a, yval, b), vid(a + 1, yval, b), vid(a, yval, b + 1),
                      vid(a + 1, yval, b + 1), out)
        blocks.append(("triangle", t, np.full(t.shape[0], tag)))
    # z = 0 and z = 1: in-plane axes (x, y); normal of (x, y) ccw is +z
    for zval, tag, out in ((0, 6, False), (n, 7, True)):
        t = face_tris(vid(a, b, zval), vid(a + 1, b, zval), vid(a, b + 1, zval),
                      vid(a + 1, b + 1, zval), out)
        blocks.append(("triangle", t, np.full(t.shape[0], tag)))
    blocks.append(("tetra", tets, np.full(tets.shape[0], 1)))
    return {"dim": 3, "points": points, "blocks": blocks}


BLOCK_DIM = {"vertex": 0, "line": 1, "triangle": 2, "tetra": 3}


def cells_of_dim(mesh, dim, physical_tags=None):
    """Cells of `dim` in file order, filtered by physical tag (mesh.py:668-681)."""
    conns, tags = [], []
    for typ, conn, phys in mesh["blocks"]:
        if BLOCK_DIM[typ] == dim:
            conns.append(np.asarray(conn, dtype=np.int64))
            tags.append(np.asarray(phys))
    conn = np.concatenate(conns, axis=0)
    tag = np.concatenate(tags)
    if physical_tags is not None:
        keep = np.isin(tag, np.asarray(physical_tags))
        conn, tag = conn[keep], tag[keep]
    return conn, tag
