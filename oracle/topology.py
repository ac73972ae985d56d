"""Entity numbering, DoF maps and orientation flags (oracle restatement).

Restates, vectorised over cells:
  * a1  global entities are the distinct sorted vertex tuples of the cells'
        sub-entities in the reference's local order
        (src/mesh/mesh.py:253-324 edges (2,3),(1,3),(1,2),(0,3),(0,2),(0,1) on
        tets, (1,2),(0,2),(0,1) on triangles; faces opposite v0..v3).
  * a2  entities_by_dimension = FIRST APPEARANCE order over the cells of the
        space's dimension in file order (networkx node insertion order in
        src/mesh/mesh.py:639-681 + src/mesh/mesh_topology.py:28-35).
  * a3  DoF blocks per entity dimension, e_dofs = int(mean(num_entity_dofs[d])),
        e_dofs * n_comp consecutive ids per entity, component fastest
        (src/spaces/dof_map.py:38-129); fields stacked in ProductSpace order
        plus dof_shift (src/spaces/product_space.py:147-170).
  * a4  per-cell destination indices: dims 0..d, local sub-entity order
        (src/spaces/dof_map.py:134-146).
  * a8  orientation: 2-D edge i is reflected unless the triangle's local pair
        equals the edge cell's stored node_tags (sorted for interior edges,
        file order for boundary lines created first)
        (src/basis/permute_and_transform.py:8-35, src/mesh/mesh.py:137-167,
        :226-229); 3-D face i is reflected iff its global tags are an odd
        permutation of sorted order, and boundary-tagged faces with local
        index 1 or 3 are forced to reflection=1 (permute_and_transform.py:57-107).
"""
import numpy as np

from . import elements as el
from .mesh_gen import BLOCK_DIM, cells_of_dim

LOCAL_SUB = {
    2: {0: ((0,), (1,), (2,)), 1: el.TRI_EDGES, 2: ((0, 1, 2),)},
    3: {0: ((0,), (1,), (2,), (3,)), 1: el.TET_EDGES, 2: el.TET_FACES, 3: ((0, 1, 2, 3),)},
}


def first_appearance_ranks(keys):
    """keys [T, n, k] -> rank [T, n] of each occurrence's entity in first-appearance order."""
    T, n, k = keys.shape
    flat = keys.reshape(T * n, k)
    _, first, inv = np.unique(flat, axis=0, return_index=True, return_inverse=True)
    inv = inv.ravel()
    order = np.argsort(first, kind="stable")
    rank_of_unique = np.empty_like(order)
    rank_of_unique[order] = np.arange(order.size)
    return rank_of_unique[inv].reshape(T, n), order.size


class Topology:
    """Entities of a mesh seen from the cells of dimension `dim`."""

    def __init__(self, mesh, dim=None, physical_tags=None):
        self.mesh = mesh
        self.dim = mesh["dim"] if dim is None else dim
        self.cells, self.cell_tags = cells_of_dim(mesh, self.dim, physical_tags)
        self.n_cells = self.cells.shape[0]
        self.rank = {}
        self.n_entities = {}
        for d in range(self.dim + 1):
            if d == self.dim:
                self.rank[d] = np.arange(self.n_cells).reshape(-1, 1)
                self.n_entities[d] = self.n_cells
                continue
            sub = np.array(LOCAL_SUB[self.dim][d])
            keys = np.sort(self.cells[:, sub], axis=2)
            self.rank[d], self.n_entities[d] = first_appearance_ranks(keys)
        self._orientation()

    def _facet_key(self, tup_sorted):
        V = int(self.mesh["points"].shape[0])
        k = np.zeros(tup_sorted.shape[:-1], dtype=np.int64)
        for j in range(tup_sorted.shape[-1]):
            k = k * V + tup_sorted[..., j].astype(np.int64)
        return k

    def _orientation(self):
        """Per (cell, local facet): boundary-tagged flag and reflection flag."""
        fd = self.dim - 1
        sub = np.array(LOCAL_SUB[self.dim][fd])
        local = self.cells[:, sub]  # [T, nf, dim]
        occ_key = self._facet_key(np.sort(local, axis=2))
        # facets of tagged lower-dimensional blocks, with the node order stored
        # by the first block that created them (mesh.py:137-151, :226-229)
        bkeys, border = [], []
        first_cell_block_seen = False
        for typ, conn, phys in self.mesh["blocks"]:
            bd = BLOCK_DIM[typ]
            if bd == self.dim:
                first_cell_block_seen = True
            if bd == fd:
                conn = np.asarray(conn, dtype=np.int64)
                bkeys.append(self._facet_key(np.sort(conn, axis=1)))
                # a boundary line created after the cells keeps the sorted order
                border.append(conn if not first_cell_block_seen else np.sort(conn, axis=1))
        if bkeys:
            bkeys = np.concatenate(bkeys)
            border = np.concatenate(border)
            uk, ui = np.unique(bkeys, return_index=True)  # first creator wins
            border = border[ui]
        else:
            uk = np.zeros(0, dtype=np.int64)
            border = np.zeros((0, self.dim), dtype=np.int64)
        pos = np.searchsorted(uk, occ_key)
        pos_c = np.minimum(pos, max(uk.size - 1, 0))
        tagged = (uk.size > 0) & (uk[pos_c] == occ_key) if uk.size else np.zeros(occ_key.shape, bool)
        self.facet_tagged = tagged
        if self.dim == 2:
            stored = np.sort(local, axis=2)
            if uk.size:
                stored = np.where(tagged[:, :, None], border[pos_c], stored)
            self.facet_reflected = np.any(local != stored, axis=2)
        else:
            a, b, c = local[:, :, 0], local[:, :, 1], local[:, :, 2]
            inv = (a > b).astype(int) + (a > c) + (b > c)
            self.facet_reflected = (inv % 2) == 1

    def rt1_signs(self):
        """Per cell and local facet, the sign the orientation transform puts on
        the RT1 basis function of that facet (+1 / -1)."""
        s = np.where(self.facet_reflected, -1.0, 1.0)
        if self.dim == 3:
            forced = self.facet_tagged.copy()
            forced[:, [0, 2]] = False
            s = np.where(forced, -1.0, s)
        return s


class FieldSpec:
    def __init__(self, name, family, degree, n_comp=1, discontinuous=False):
        self.name = name
        self.family = family
        self.degree = degree
        self.n_comp = n_comp
        self.discontinuous = discontinuous


def field_dof_layout(topo, spec):
    """(e_dofs per dim, block bases (relative), n_dof) for one field (dof_map.py:63-129)."""
    ref = el.create_element(spec.family, topo.dim, spec.degree, spec.discontinuous)
    e_dofs = [int(np.mean(ref.num_entity_dofs[d])) for d in range(topo.dim + 1)]
    sizes = [topo.n_entities[d] * e_dofs[d] * spec.n_comp for d in range(topo.dim + 1)]
    bases = np.concatenate([[0], np.cumsum(sizes)])
    return e_dofs, bases, int(bases[-1])


def cell_dofs(topo, specs, dof_shift=0):
    """Destination indices [T, n_loc] of the product space (product_space.py:147-170)."""
    cols = []
    offset = int(dof_shift)
    n_total = 0
    for spec in specs:
        e_dofs, bases, n_dof = field_dof_layout(topo, spec)
        for d in range(topo.dim + 1):
            w = e_dofs[d] * spec.n_comp
            if w == 0:
                continue
            r = topo.rank[d]  # [T, n_ent]
            ids = offset + bases[d] + r[:, :, None] * w + np.arange(w)[None, None, :]
            cols.append(ids.reshape(topo.n_cells, -1))
        offset += n_dof
        n_total += n_dof
    return np.concatenate(cols, axis=1).astype(np.int64), n_total
