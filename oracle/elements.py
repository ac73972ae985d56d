"""Reference finite elements on simplices (oracle).

Restates the element data the reference reads from basix objects in
src/basis/finite_element.py:85-123 (entity_dofs, num_entity_dofs, entity
transformations) and :156-186 (tabulate(1, pts) + push_forward on values only).

Families (src/basis/element_family.py:4-16, variant gll_centroid):
  * Lagrange P0, P1, P2 on interval / triangle / tetrahedron.  For degree <= 2
    the gll_centroid points are the vertices and edge midpoints.  Local order:
    vertices, then edges in basix's sub-entity order.
  * RT1 (lowest-order Raviart-Thomas, basix degree 1) on triangle / tetrahedron.
    DOFs are normal moments against P0 on each facet, with basix's facet
    normal: rot90(v1 - v0) on triangle edges, (v1 - v0) x (v2 - v0) on
    tetrahedron faces (facet vertices in sub-entity order).  The basis is
    psi_i = sigma_i * kappa * (x - v_i) with kappa = 1 (tri), 2 (tet) and
    sigma_i = +1 if that normal points out of the cell, -1 otherwise.
    Parity unpinned: no reference test fixes this scale or sign.

Tabulation shape follows basix: [1 + tdim, n_points, n_basis, value_size].
"""
import numpy as np

# basix sub-entity vertex lists (also the reference mesh's local order,
# src/mesh/mesh.py:160-163 and :187-204)
TRI_EDGES = ((1, 2), (0, 2), (0, 1))
TET_EDGES = ((2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1))
TET_FACES = ((1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2))

REF_VERTS = {
    1: np.array([[0.0], [1.0]]),
    2: np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]),
    3: np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]),
}

# RT1 reference normal orientation relative to the outward normal
RT1_SIGMA = {2: np.array([-1.0, 1.0, -1.0]), 3: np.array([1.0, -1.0, 1.0, -1.0])}
RT1_KAPPA = {2: 1.0, 3: 2.0}

N_SUB = {0: (1,), 1: (2, 1), 2: (3, 3, 1), 3: (4, 6, 4, 1)}


def _barycentric(dim, pts):
    pts = np.atleast_2d(pts)
    lam = np.empty((pts.shape[0], dim + 1))
    lam[:, 0] = 1.0 - pts.sum(axis=1)
    lam[:, 1:] = pts
    dlam = np.zeros((dim, dim + 1))  # d lambda_j / d x_k
    dlam[:, 0] = -1.0
    dlam[:, 1:] = np.eye(dim)
    return lam, dlam


def _edges(dim):
    return {1: ((0, 1),), 2: TRI_EDGES, 3: TET_EDGES}[dim]


class RefElement:
    """A basix-like element object: the attributes the reference reads."""

    def __init__(self, family, dim, degree, discontinuous=False):
        self.family = family
        self.dim = dim
        self.degree = degree
        self.discontinuous = discontinuous
        nsub = N_SUB[dim]
        ed = [[[] for _ in range(n)] for n in nsub]
        if family == "P":
            if degree == 0:
                ed[dim][0] = [0]
            elif degree == 1:
                for v in range(dim + 1):
                    ed[0][v] = [v]
            elif degree == 2:
                for v in range(dim + 1):
                    ed[0][v] = [v]
                for e in range(len(_edges(dim))):
                    ed[1][e] = [dim + 1 + e]
            else:
                raise NotImplementedError("Lagrange degree > 2")
            self.value_size = 1
        elif family == "RT":
            if degree != 1:
                raise NotImplementedError("RT degree > 1")
            if dim == 1:
                raise ValueError("RT on an interval is Lagrange in the reference")
            for f in range(dim + 1):
                ed[dim - 1][f] = [f]
            self.value_size = dim
        else:
            raise NotImplementedError(family)
        self.dim_space = sum(len(x) for row in ed for x in row)
        if discontinuous:
            ed = [[[] for _ in range(n)] for n in nsub]
            ed[dim][0] = list(range(self.dim_space))
        self.entity_dofs = ed
        self.num_entity_dofs = [[len(x) for x in row] for row in ed]
        self.dof_transformations_are_identity = not (family == "RT" and not discontinuous)

    def entity_transformations(self):
        """Base transformations keyed by sub-entity type (basix convention)."""
        out = {}
        if self.dim >= 2:
            n = self.num_entity_dofs[1][0] if not self.discontinuous else 0
            if self.family == "RT" and self.dim == 2 and not self.discontinuous:
                out["interval"] = -np.ones((1, 1, 1))
            else:
                out["interval"] = np.array([np.eye(n)])
        if self.dim == 3:
            n = self.num_entity_dofs[2][0] if not self.discontinuous else 0
            if self.family == "RT" and not self.discontinuous:
                out["triangle"] = np.array([[[1.0]], [[-1.0]]])
            else:
                out["triangle"] = np.array([np.eye(n), np.eye(n)])
        return out

    def tabulate(self, nderiv, pts):
        assert nderiv <= 1
        pts = np.atleast_2d(np.asarray(pts, dtype=np.float64))
        dim = self.dim
        nq = pts.shape[0]
        if self.family == "P":
            tab = np.zeros((1 + dim, nq, self.dim_space, 1))
            lam, dlam = _barycentric(dim, pts)
            if self.degree == 0:
                tab[0, :, 0, 0] = 1.0
            elif self.degree == 1:
                tab[0, :, :, 0] = lam
                for k in range(dim):
                    tab[1 + k, :, :, 0] = dlam[k][None, :]
            else:
                for v in range(dim + 1):
                    tab[0, :, v, 0] = lam[:, v] * (2.0 * lam[:, v] - 1.0)
                    for k in range(dim):
                        tab[1 + k, :, v, 0] = dlam[k, v] * (4.0 * lam[:, v] - 1.0)
                for e, (a, b) in enumerate(_edges(dim)):
                    tab[0, :, dim + 1 + e, 0] = 4.0 * lam[:, a] * lam[:, b]
                    for k in range(dim):
                        tab[1 + k, :, dim + 1 + e, 0] = 4.0 * (
                            dlam[k, a] * lam[:, b] + lam[:, a] * dlam[k, b])
            return tab
        # RT1
        tab = np.zeros((1 + dim, nq, dim + 1, dim))
        kap = RT1_KAPPA[dim]
        for i in range(dim + 1):
            c = RT1_SIGMA[dim][i] * kap
            tab[0, :, i, :] = c * (pts - REF_VERTS[dim][i][None, :])
            for k in range(dim):
                tab[1 + k, :, i, k] = c
        return tab

    def push_forward(self, U, J, detJ, K):
        """Map reference values U [Q, n, vs] to the physical cell.

        Lagrange: identity.  RT: contravariant Piola (1/detJ) J U, so the
        physical value size is the geometric dimension (J is [Q, gdim, tdim]).
        """
        if self.family == "P":
            return U.copy()
        J = np.asarray(J)
        return np.einsum("qgt,qnt->qng", J, U) / np.asarray(detJ)[:, None, None]


def create_element(family, dim, degree, discontinuous=False):
    return RefElement(family, dim, degree, discontinuous)


def rt1_reference_moments(dim):
    """Closed-form reference integrals used by the RT1 mass matrix.

    Returns (area, m, S) with area = |T|, m = int x dx, S = int x x^T dx on the
    reference simplex.  Exact values: |T| = 1/d!, m_k = 1/(d+1)!,
    S = (I + 1 1^T)/(d+2)!.
    """
    fact = {2: (0.5, 1.0 / 6.0, 1.0 / 24.0), 3: (1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0)}[dim]
    area, mk, s = fact
    return area, np.full(dim, mk), s * (np.eye(dim) + np.ones((dim, dim)))
