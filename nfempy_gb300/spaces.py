"""Function spaces on the device: the ProductSpace / DiscreteSpace / Mesh API.

Mirrors the reference's setup interface
(src/spaces/product_space.py:9-201, src/spaces/discrete_space.py:14-221,
src/mesh/mesh.py:13-19) so drivers keep their call sequence:

    space = ProductSpace({"u": (dim, 1, "RT", 1, mesh), "p": (dim, 1, "Lagrange", 0, mesh)})
    space.make_subspaces_discontinuous({"u": False, "p": True})
    space.build_structures({"u": [1], "p": [1]}, {})
    space.n_dof, space.destination_indexes(i)

build_structures numbers the mesh entities in first-appearance order, builds
the orientation flags and the per-cell DoF map entirely on the GPU
(libnfem_gb300: nfem_number_entities, nfem_rt1_sign_mask,
nfem_compose_cell_dofs).  The host keeps only array shapes.
"""
import numpy as np
import torch

from . import _lib
from .meshes import BLOCK_DIM, cells_of_dim
from .quadrature import make_quadrature

FAMILIES = ("Lagrange", "RT", "BDM", "N1E", "N2E")


def entity_dofs(family, dim, k, discontinuous=False):
    """DoFs per entity of each dimension 0..dim (int(mean(num_entity_dofs[d]))
    in src/spaces/dof_map.py:69-71) for the supported elements."""
    if family == "N2E":
        family = "N1E"  # src/basis/element_family.py:10
    if dim <= 1 and family in ("RT", "BDM", "N1E"):
        family = "Lagrange"  # src/spaces/discrete_space.py:38-49
    e = [0] * (dim + 1)
    if family == "Lagrange":
        if k == 0:
            e[dim] = 1
        elif k == 1:
            e[0] = 1
        elif k == 2:
            e[0] = 1
            if dim >= 1:
                e[1] = 1
        else:
            raise NotImplementedError(f"Lagrange degree {k}")
    elif family == "RT" and k == 1:
        e[dim - 1] = 1
    elif family == "BDM" and k == 1:
        e[dim - 1] = dim
    elif family == "N1E" and k == 1:
        e[1] = 1
    else:
        raise NotImplementedError(f"{family} degree {k}")
    if discontinuous:
        nsub = {1: (2, 1), 2: (3, 3, 1), 3: (4, 6, 4, 1)}[dim]
        n_local = sum(a * b for a, b in zip(nsub, e))
        e = [0] * dim + [n_local]
    return e


N_SUB = {2: (3, 3, 1), 3: (4, 6, 4, 1)}


class Mesh:
    """Points and cell blocks of a conformal simplex mesh (reference: src/mesh/mesh.py).

    Mesh(dimension, file_name) reads a gmsh 4.1 ASCII file like the
    reference (nfempy_gb300.gmsh.read_msh, meshio's conventions);
    Mesh(dimension, data=...) takes the in-memory layout produced by
    nfempy_gb300.meshes (any dict {"dim", "points", "blocks": [(type, conn,
    physical_tags)]})."""

    def __init__(self, dimension, file_name=None, data=None):
        if data is None:
            if file_name is None:
                raise ValueError("Mesh needs a gmsh file name or data=")
            from .gmsh import read_msh
            data = read_msh(file_name, dim=dimension)
        self.dimension = int(dimension)
        self.data = data
        self.points = np.asarray(data["points"], dtype=np.float64)

    def build_conformal_mesh(self):
        # entity numbering is performed on the device by each space
        return self


class DiscreteSpace:
    def __init__(self, dimension, n_components, family, k_order, mesh, integration_order=0):
        if family not in FAMILIES:
            raise ValueError(f"unknown family {family}")
        self.dimension = int(dimension)
        self.n_comp = int(n_components)
        self.family = family
        self.k_order = int(k_order)
        self.mesh = mesh
        self.integration_order = integration_order
        self.discontinuous = False
        self.name = "Unnamed"
        self.n_dof = 0
        self._product = None

    @property
    def elements(self):
        """One entry per cell (len() is the number of elements, as for the
        reference's FiniteElement list)."""
        return range(self._product.n_cells) if self._product is not None else range(0)

    @property
    def bc_elements(self):
        """One entry per boundary element (the facet's entity number), in the
        reference's order (src/spaces/discrete_space.py:163-207)."""
        if self._product is None:
            return np.zeros(0, dtype=np.int64)
        return self._product._bc_facets(self.name)["rank"]

    def make_discontinuous(self):
        self.discontinuous = True

    def entity_dofs(self):
        return entity_dofs(self.family, self.dimension, self.k_order, self.discontinuous)


class ProductSpace:
    def __init__(self, discrete_spaces_data, device=None):
        self.names = list(discrete_spaces_data.keys())
        self.device = torch.device(device if device is not None else "cuda")
        k_orders = [d[3] for d in discrete_spaces_data.values()]
        dims = [d[0] for d in discrete_spaces_data.values()]
        self.integration_order = 2 * int(np.max(k_orders)) + 1  # product_space.py:31
        self.quadrature = [None, None, None, None]
        for dim in range(int(np.max(dims)) + 1):
            self.quadrature[dim] = make_quadrature(dim, self.integration_order)
        self.bc_quadrature = [None, None, None, None]
        for dim in dims:
            if dim - 1 >= 0:
                self.bc_quadrature[dim - 1] = make_quadrature(dim - 1, self.integration_order)
        self.discrete_spaces = {}
        for name, (dim, nc, family, k, mesh) in discrete_spaces_data.items():
            s = DiscreteSpace(dim, nc, family, k, mesh, self.integration_order)
            s.name = name
            s._product = self
            self.discrete_spaces[name] = s
        self._dof_shift = 0
        self.n_dof = 0
        self.cell_dofs = None

    @property
    def dof_shift(self):
        return self._dof_shift

    @dof_shift.setter
    def dof_shift(self, value):
        if not isinstance(value, (int, np.integer)):
            raise TypeError("dof_shift must be an integer")
        if value < 0:
            raise ValueError("dof_shift must be non-negative")
        self._dof_shift = int(value)

    def dimension(self):
        return max(s.dimension for s in self.discrete_spaces.values())

    def make_subspaces_discontinuous(self, discrete_space_disc):
        for name in self.names:
            if discrete_space_disc.get(name, False):
                self.discrete_spaces[name].make_discontinuous()

    # ------------------------------------------------------------ build
    def build_structures(self, physical_tags, b_physical_tags=None, stream=None):
        spaces = list(self.discrete_spaces.values())
        dim = spaces[0].dimension
        mesh = spaces[0].mesh
        if any(s.dimension != dim or s.mesh is not mesh for s in spaces):
            raise NotImplementedError("all fields must live on the same mesh and dimension")
        tags = [tuple(physical_tags.get(n, [None])) for n in self.names]
        if len(set(tags)) != 1:
            raise NotImplementedError("all fields must use the same physical tags")
        self.physical_tags = list(tags[0])
        self.b_physical_tags = b_physical_tags or {}
        self._bc_cache = {}
        self.dim = dim
        self.mesh = mesh
        cells, _ = cells_of_dim(mesh.data, dim, self.physical_tags)
        self.n_cells = int(cells.shape[0])
        dev = self.device
        st = _lib.stream_ptr(stream)
        self.cells_host = cells
        self.cells = torch.as_tensor(cells.astype(np.int32), device=dev).contiguous()
        self.points = torch.as_tensor(mesh.points, dtype=torch.float64, device=dev).contiguous()
        self.points_split = torch.empty((mesh.points.shape[0] + 1, 4), dtype=torch.float32, device=dev)
        _lib.call("nfem_points_split", _lib.ptr(self.points), mesh.points.shape[0], _lib.ptr(self.points_split), st)
        # exact 64-bit fixed-point records for the FP64 kernels of tetrahedra
        self.points_fixed64 = torch.empty((mesh.points.shape[0] + 1, 4), dtype=torch.int64, device=dev)
        _lib.call("nfem_points_fixed64", _lib.ptr(self.points), mesh.points.shape[0], _lib.ptr(self.points_fixed64),
                  st)
        # boundary facets of the mesh file (all tagged lower-dimensional blocks)
        facet_blocks, facets_first, seen_cells = [], 1, False
        for typ, conn, phys in mesh.data["blocks"]:
            bd = BLOCK_DIM[typ]
            if bd == dim:
                seen_cells = True
            elif bd == dim - 1:
                facet_blocks.append(np.asarray(conn, dtype=np.int32))
                if seen_cells:
                    facets_first = 0
        facets = np.concatenate(facet_blocks) if facet_blocks else np.zeros((0, dim), np.int32)
        self.facets = torch.as_tensor(facets, device=dev).contiguous()
        self.n_facets = int(facets.shape[0])
        self._facets_first = facets_first

        need = set()
        for s in spaces:
            for d, e in enumerate(s.entity_dofs()):
                if e > 0 and d < dim:
                    need.add(d)
        if any(s.family == "RT" for s in spaces):
            need.add(dim - 1)
        self.occ_rank = {}
        self.n_entities = {dim: self.n_cells}
        self.facet_flags = None
        for d in sorted(need):
            self._number(d, st)
        self.rt_sign_mask = None
        if self.facet_flags is not None:
            self.rt_sign_mask = torch.empty(self.n_cells, dtype=torch.uint8, device=dev)
            _lib.call("nfem_rt1_sign_mask", _lib.ptr(self.facet_flags), self.n_cells, dim,
                      _lib.ptr(self.rt_sign_mask), st)
        self._compose(st)
        torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()

    def _number(self, d, st):
        dim = self.dim
        n_ent = N_SUB[dim][d]
        ws_b = _lib.C.c_size_t(0)
        _lib.call("nfem_numbering_workspace_bytes", self.n_cells, dim, d, self.points.shape[0], self.n_facets,
                  _lib.C.byref(ws_b))
        ws = torch.empty(int(ws_b.value), dtype=torch.uint8, device=self.device)
        rank = torch.empty((self.n_cells, n_ent), dtype=torch.int32, device=self.device)
        count = torch.zeros(1, dtype=torch.int64, device=self.device)
        flags = None
        if d == dim - 1:
            flags = torch.empty((self.n_cells, n_ent), dtype=torch.uint8, device=self.device)
        _lib.call("nfem_number_entities", _lib.ptr(self.cells), self.n_cells, dim, d, self.points.shape[0],
                  _lib.ptr(self.facets) if self.n_facets else None, self.n_facets, self._facets_first,
                  _lib.ptr(ws), ws.numel(), _lib.ptr(rank), _lib.ptr(flags), _lib.ptr(count), st)
        self.occ_rank[d] = rank
        self.n_entities[d] = int(count.item())
        if flags is not None:
            self.facet_flags = flags

    def _compose(self, st):
        dim = self.dim
        blocks = []
        offset = self._dof_shift
        self.field_offsets = {}
        self.field_slices = {}
        self.entity_blocks = {}
        col = 0
        for name in self.names:
            s = self.discrete_spaces[name]
            e = s.entity_dofs()
            start = offset
            self.field_offsets[name] = start
            self.entity_blocks[name] = {}
            c0 = col
            for d in range(dim + 1):
                w = e[d] * s.n_comp
                if w == 0:
                    continue
                self.entity_blocks[name][d] = (offset, w)
                n_ent = N_SUB[dim][d]
                blocks.append(_lib.DofBlock(
                    _lib.ptr(self.occ_rank[d]).value if d < dim else None, n_ent, w, offset))
                offset += self.n_entities[d] * w
                col += n_ent * w
            s.n_dof = offset - start
            self.field_slices[name] = slice(c0, col)
        self.n_dof = offset - self._dof_shift
        self.n_loc = col
        if offset >= 2 ** 31 - 1:
            raise _lib.NfemError(4, "build_structures (DoF count)")
        arr = (_lib.DofBlock * len(blocks))(*blocks)
        self.cell_dofs = torch.empty((self.n_cells, self.n_loc), dtype=torch.int32, device=self.device)
        _lib.call("nfem_compose_cell_dofs", self.n_cells, len(blocks), arr, _lib.ptr(self.cell_dofs), self.n_loc, st)
        self.discrete_spaces_dofs = {n: self.discrete_spaces[n].n_dof for n in self.names}

    # ------------------------------------------------------------ queries
    def destination_indexes(self, cell_index, field_name=None):
        """Global DoFs of one cell (product_space.py:164-170)."""
        row = self.cell_dofs[int(cell_index)].cpu().numpy().astype(np.int64)
        if field_name is None:
            return row
        return row[self.field_slices[field_name]]

    def all_destination_indexes(self):
        return self.cell_dofs.cpu().numpy().astype(np.int64)

    # ------------------------------------------------------------ boundary elements
    def _facet_records(self):
        """Facets of the mesh file, one record per distinct facet: sorted
        vertices, node order at creation and physical tag.

        The reference inserts the file's blocks in order
        (src/mesh/mesh.py:221-237, 335-336): a facet is created by its first
        insertion (a facet block, keeping the file's node order, or the first
        cell that holds it: a tetrahedron's face i keeps the cell's node order
        of vertices (1,2,3), (0,2,3), (0,1,3), (0,1,2) (mesh.py:180-215), a
        triangle's edges are sorted (mesh.py:153-175)), and every insertion
        with a tag sets its material id, so the last tagged block wins."""
        if "records" in self._bc_cache:
            return self._bc_cache["records"]
        dim = self.dim
        conns, tags, before = [], [], []
        seen_cells = False
        for typ, conn, phys in self.mesh.data["blocks"]:
            bd = BLOCK_DIM[typ]
            if bd == dim:
                seen_cells = True
            elif bd == dim - 1:
                c = np.asarray(conn, dtype=np.int64).reshape(-1, dim)
                conns.append(c)
                tags.append(np.asarray(phys, dtype=np.int64).reshape(-1))
                before.append(np.full(c.shape[0], not seen_cells))
        if not conns:
            rec = (np.zeros((0, dim), np.int64), np.zeros((0, dim), np.int64), np.zeros(0, np.int64),
                   np.zeros(0, bool))
            self._bc_cache["records"] = rec
            return rec
        conn = np.concatenate(conns)
        tag = np.concatenate(tags)
        before = np.concatenate(before)
        srt = np.sort(conn, axis=1)
        _, first, inv = np.unique(srt, axis=0, return_index=True, return_inverse=True)
        inv = inv.reshape(-1)
        last = np.zeros(len(first), dtype=np.int64)
        last[inv] = np.arange(len(inv))  # the last write of each facet wins
        rec = (srt[first], conn[first], tag[last], before[first])
        self._bc_cache["records"] = rec
        return rec

    def _bc_facets(self, name):
        """Boundary elements of field `name`: the file's facets whose tag is in
        b_physical_tags[name], ordered by entity number (first appearance
        over cells x local facets: src/mesh/mesh_topology.py:28-35 and
        src/spaces/discrete_space.py:163-207).  Each gets the first cell
        holding it (the first predecessor of product_space.py:132-145), its
        local facet index and its vertices in the reference's node order."""
        key = ("facets", name)
        if key in self._bc_cache:
            return self._bc_cache[key]
        dim = self.dim
        tags = list(self.b_physical_tags.get(name, []) or [])
        srt, node_order, tag, before = self._facet_records()
        keep = np.isin(tag, np.asarray(tags, dtype=np.int64)) if tags else np.zeros(len(tag), bool)
        srt, node_order, before = srt[keep], node_order[keep], before[keep]
        sub = np.array(((1, 2), (0, 2), (0, 1)) if dim == 2 else ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)))
        cells = self.cells_host
        occ = np.sort(cells[:, sub], axis=2).reshape(-1, dim)  # [T * (dim + 1), dim], flat = c * (dim + 1) + i
        V = int(max(self.mesh.points.shape[0], 1))
        if float(V) ** dim >= 2.0 ** 62:
            raise NotImplementedError("too many vertices for the facet keys")

        def keys(a):
            k = np.zeros(a.shape[0], dtype=np.int64)
            for j in range(dim):
                k = k * V + a[:, j]
            return k
        ok = keys(occ)
        order = np.argsort(ok, kind="stable")
        fk = keys(srt)
        pos = np.searchsorted(ok[order], fk)
        if len(fk) and (np.any(pos >= len(ok)) or np.any(ok[order][np.minimum(pos, len(ok) - 1)] != fk)):
            raise ValueError("a tagged boundary facet belongs to no cell of the space")
        flat = order[pos]  # the first (lowest) cell holding the facet
        c, i = flat // (dim + 1), flat % (dim + 1)
        if dim - 1 not in self.occ_rank:  # facets carry no DoF of any field: number them now for the order
            self._number(dim - 1, _lib.stream_ptr(None))
        rank = self.occ_rank[dim - 1].cpu().numpy()[c, i].astype(np.int64) if len(c) else np.zeros(0, np.int64)
        o = np.argsort(rank, kind="stable")
        c, i, rank, node_order, before = c[o], i[o], rank[o], node_order[o], before[o]
        verts = node_order.copy()
        if dim == 3:
            from_cell = cells[c[:, None], sub[i]] if len(c) else np.zeros((0, 3), np.int64)
        else:
            from_cell = np.sort(cells[c[:, None], sub[i]], axis=1) if len(c) else np.zeros((0, 2), np.int64)
        verts[~before] = from_cell[~before]
        out = {"cell": c, "local": i, "rank": rank, "vertices": verts}
        self._bc_cache[key] = out
        return out

    def _field_bc_dofs(self, name):
        """[n_bc, k] DoFs of field `name` on its boundary elements
        (src/spaces/dof_map.py:148-170): per dimension d < dim with entity
        DoFs, the facet's sub-entities in the facet's own order (vertices,
        then edges (v1,v2), (v0,v2), (v0,v1), then the facet), each entity's
        DoFs in the cell numbering."""
        key = ("dofs", name)
        if key in self._bc_cache:
            return self._bc_cache[key]
        dim = self.dim
        f = self._bc_facets(name)
        c, verts = f["cell"], f["vertices"]
        n = len(c)
        cols = []
        blocks = self.entity_blocks[name]
        cell_pos = None
        if n:
            # position of each facet vertex in its cell
            cell_pos = np.argmax(self.cells_host[c][:, None, :] == verts[:, :, None], axis=2)
        for d in range(dim):
            if d not in blocks or n == 0:
                continue
            off, w = blocks[d]
            rank = self.occ_rank[d].cpu().numpy()
            if d == dim - 1:
                ents = [f["local"]]
            elif d == 0:
                ents = [cell_pos[:, k] for k in range(dim)]
            else:  # d == 1 in 3D: the face's edges in its own order
                cell_edges = {frozenset(e): j for j, e in enumerate(((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)))}
                table = np.full((4, 4), -1, dtype=np.int64)
                for e, j in cell_edges.items():
                    a, b = tuple(e)
                    table[a, b] = table[b, a] = j
                ents = [table[cell_pos[:, a], cell_pos[:, b]] for a, b in ((1, 2), (0, 2), (0, 1))]
            for le in ents:
                r = rank[c, le].astype(np.int64)
                cols.append(off + r[:, None] * w + np.arange(w)[None, :])
        out = np.concatenate(cols, axis=1) if cols else np.zeros((n, 0), dtype=np.int64)
        self._bc_cache[key] = out
        return out

    def bc_destination_indexes(self, bc_index, field_name=None):
        """Global DoFs of one boundary element (product_space.py:172-201):
        the fields with boundary elements in order, or one field."""
        if field_name is not None:
            return self._field_bc_dofs(field_name)[int(bc_index)]
        parts = [self._field_bc_dofs(n)[int(bc_index)] for n in self.names
                 if len(self._bc_facets(n)["rank"]) > 0]
        return np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)
