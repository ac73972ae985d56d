"""gmsh 4.1 ASCII mesh files -> the mesh layout the spaces consume.

The reference reads its meshes with meshio (src/mesh/mesh.py:13-19) and
then walks `points`, the cell blocks (`cells[i].type`, `.data`) and
`cell_data["gmsh:physical"]` (src/mesh/mesh.py:239-339).  This reader
produces the same three things from the file, with meshio's conventions:

  * points: every node in file order (node tags mapped to 0-based
    positions), [V, 3] float64;
  * blocks: one block per element block of the file, in file order, as
    (type, connectivity [n, k] int64, physical tag per element); element
    types 15 vertex, 1 line, 2 triangle, 4 tetrahedron;
  * the physical tag of a block is the first physical tag of its entity in
    the $Entities section (0 when the entity has none).

Only ASCII files of format 4.1 are read (the format of the reference's
fixtures, e.g. examples/cosserat_elasticity/gmsh_files/ex_3/*.msh).
"""
import numpy as np

_TYPES = {15: ("vertex", 1), 1: ("line", 2), 2: ("triangle", 3), 4: ("tetra", 4)}


def _sections(lines):
    out = {}
    i = 0
    while i < len(lines):
        s = lines[i].strip()
        if s.startswith("$") and not s.startswith("$End"):
            name = s[1:]
            j = i + 1
            while not lines[j].strip() == "$End" + name:
                j += 1
            out[name] = lines[i + 1:j]
            i = j + 1
        else:
            i += 1
    return out


def read_msh(path, dim=None):
    """Read a gmsh 4.1 ASCII file.  Returns {"dim", "points", "blocks",
    "physical_names"}; dim defaults to the largest element dimension."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    sec = _sections(lines)
    fmt = sec["MeshFormat"][0].split()
    if not fmt[0].startswith("4.1") or fmt[1] != "0":
        raise ValueError(f"{path}: only gmsh 4.1 ASCII files are read (got version {fmt[0]}, file type {fmt[1]})")
    names = {}
    for ln in sec.get("PhysicalNames", [])[1:]:
        d, tag, name = ln.split(maxsplit=2)
        names[(int(d), int(tag))] = name.strip('"')
    # $Entities: points carry (tag, x, y, z, n_phys, phys...); curves,
    # surfaces and volumes (tag, bbox[6], n_phys, phys..., n_bounding, ...)
    phys = {0: {}, 1: {}, 2: {}, 3: {}}
    ent = sec.get("Entities")
    if ent:
        counts = [int(v) for v in ent[0].split()]
        k = 1
        for d in range(4):
            for _ in range(counts[d]):
                v = ent[k].split()
                k += 1
                tag = int(v[0])
                at = 4 if d == 0 else 7
                n_ph = int(v[at])
                phys[d][tag] = [int(x) for x in v[at + 1:at + 1 + n_ph]]
    # $Nodes: header (n_blocks, n_nodes, min_tag, max_tag); per block
    # (entity dim, entity tag, parametric, n) then n tags then n coordinate lines
    nod = sec["Nodes"]
    n_blocks, n_nodes = (int(v) for v in nod[0].split()[:2])
    tags = np.empty(n_nodes, dtype=np.int64)
    pts = np.empty((n_nodes, 3), dtype=np.float64)
    k, p = 1, 0
    for _ in range(n_blocks):
        ed, et, param, n = (int(v) for v in nod[k].split())
        if param:
            raise ValueError(f"{path}: parametric nodes are not supported")
        k += 1
        for i in range(n):
            tags[p + i] = int(nod[k + i])
        k += n
        for i in range(n):
            pts[p + i] = [float(x) for x in nod[k + i].split()[:3]]
        k += n
        p += n
    index = np.full(int(tags.max()) + 1, -1, dtype=np.int64)
    index[tags] = np.arange(n_nodes)
    # $Elements: header (n_blocks, n_elements, ...); per block (entity dim,
    # entity tag, element type, n) then n lines "element_tag node_tags..."
    el = sec["Elements"]
    n_blocks = int(el[0].split()[0])
    blocks = []
    k = 1
    max_dim = 0
    for _ in range(n_blocks):
        ed, et, etype, n = (int(v) for v in el[k].split())
        k += 1
        if etype not in _TYPES:
            raise ValueError(f"{path}: element type {etype} is not supported")
        name, nv = _TYPES[etype]
        conn = np.array([[int(x) for x in el[k + i].split()[1:1 + nv]] for i in range(n)], dtype=np.int64)
        k += n
        ph = phys[ed].get(et, [])
        tag = ph[0] if ph else 0
        blocks.append((name, index[conn], np.full(n, tag, dtype=np.int64)))
        max_dim = max(max_dim, ed)
    return {"dim": int(dim if dim is not None else max_dim), "points": pts, "blocks": blocks,
            "physical_names": names}
