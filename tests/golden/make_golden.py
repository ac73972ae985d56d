"""Generate golden fixtures by running the reference's OWN code (this container only).

The reference (nfempy, pure Python) cannot run end to end here: basix,
auto_diff, petsc4py, gmsh, meshio and matplotlib are absent.  Its mesh,
topology, DoF-map, assembler, mapping and orientation code is plain
Python/numpy, so this script runs exactly those files unchanged with small
stand-ins:

  * meshio   - `read(name)` returns an in-memory mesh from oracle.mesh_gen
  * basix    - element metadata, tabulation and push-forward from
               oracle.elements, quadrature from oracle.quadrature
  * matplotlib - empty module (imported but unused by src/assembly/ScatterFormData.py:2)
  * auto_diff  - forward-mode AutoDiff / VecValDer written from the weak
                 forms' own call sites (the forms are linear in alpha, so the
                 derivative carried through is the element Jacobian)

What the fixtures pin, from the reference's own code paths:
  * destination indices of every cell   (ProductSpace.destination_indexes,
                                          src/spaces/product_space.py:164-170)
  * the assembled sparsity pattern and per-slot multiplicity (SequentialAssembler
    + scatter_form_data, src/assembly/*.py, recorded through a Mat stand-in)
  * orientation flags (src/basis/permute_and_transform.py:8-107)
  * |det J| and J+ (src/geometry/mapping.py:23-55)
  * the oriented, pushed-forward RT1 basis (FiniteElement.evaluate_basis,
    src/basis/finite_element.py:156-186) - its Piola/orientation logic is the
    reference's, its reference-cell tables come from the basix stand-in.
  * element residuals and Jacobians (r_el, j_el) of every cell from the
    reference's own weak forms: LaplaceDualWeakForm.evaluate_form
    (src/weak_forms/laplace_dual_weak_form.py:10-86), LEPrimalWeakForm
    (src/weak_forms/le_primal_weak_form.py:10-129) and
    LCEDualWeakForm.evaluate_form_vectorized
    (src/weak_forms/lce_dual_weak_form.py:410-648), with the coefficient
    functions of FORM_FUNCTIONS below (tests/cases.py restates them for the
    oracle side).

Run:  python -B tests/golden/make_golden.py --reference-src <nfempy>/src
      (or set NFEM_REFERENCE_SRC; writes tests/golden/*.npz)
"""
import os
import sys
import types

sys.dont_write_bytecode = True
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def reference_src():
    """The reference's src/ directory: --reference-src PATH, else the
    NFEM_REFERENCE_SRC environment variable."""
    path = None
    if "--reference-src" in sys.argv:
        i = sys.argv.index("--reference-src")
        path = sys.argv[i + 1] if i + 1 < len(sys.argv) else None
    path = path or os.environ.get("NFEM_REFERENCE_SRC")
    if not path or not os.path.isdir(os.path.join(path, "weak_forms")):
        sys.exit("make_golden.py: pass --reference-src <nfempy checkout>/src (or set NFEM_REFERENCE_SRC); "
                 f"got {path!r}, which holds no weak_forms/ directory")
    return path


REF_SRC = reference_src() if __name__ == "__main__" else None

import numpy as np  # noqa: E402

from oracle import elements as oel  # noqa: E402
from oracle import mesh_gen, quadrature  # noqa: E402

# ---------------------------------------------------------------- stand-ins
_MESHES = {}


class _Block:
    def __init__(self, typ, data):
        self.type = typ
        self.data = np.asarray(data, dtype=np.int64)
        self.dim = mesh_gen.BLOCK_DIM[typ]


class _MeshioMesh:
    def __init__(self, m):
        self.points = np.asarray(m["points"], dtype=np.float64)
        self.cells = [_Block(t, c) for t, c, _ in m["blocks"]]
        self.cell_data = {"gmsh:physical": [np.asarray(p) for _, _, p in m["blocks"]]}

    def get_cells_type(self, name):
        n = {"vertex": 1, "line": 2, "triangle": 3, "tetra": 4}[name]
        blocks = [b.data for b in self.cells if b.type == name]
        if not blocks:
            return np.zeros((0, n), dtype=np.int64)
        return np.concatenate(blocks, axis=0)


meshio = types.ModuleType("meshio")
meshio.read = lambda name: _MeshioMesh(_MESHES[name])
meshio.Mesh = object
meshio.write = lambda *a, **k: None

basix = types.ModuleType("basix")


class ElementFamily:
    P = "P"
    RT = "RT"
    BDM = "BDM"
    N1E = "N1E"


class LagrangeVariant:
    gll_centroid = "gll_centroid"


class CellType:
    point = 0
    interval = 1
    triangle = 2
    tetrahedron = 3


class QuadratureType:
    gauss_jacobi = "gauss_jacobi"


class _PointElement:
    entity_dofs = [[[0]]]
    num_entity_dofs = [[1]]
    dof_transformations_are_identity = True

    def entity_transformations(self):
        return {}

    def tabulate(self, n, pts):
        return np.ones((1, 1, 1, 1))


def _create_element(family, celltype, degree, lagrange_variant=None, discontinuous=False):
    if celltype == 0:
        return _PointElement()
    return oel.create_element(family, celltype, degree, discontinuous)


basix.ElementFamily = ElementFamily
basix.LagrangeVariant = LagrangeVariant
basix.CellType = CellType
basix.QuadratureType = QuadratureType
basix.create_element = _create_element
basix.make_quadrature = lambda cell, degree, rule=None: quadrature.make_quadrature(cell, degree)

matplotlib = types.ModuleType("matplotlib")
matplotlib.pyplot = types.ModuleType("matplotlib.pyplot")


_np_zeros = np.zeros  # the stand-in's own arrays (np.zeros is replaced inside AutoDiff)


class VecValDer:
    """A value and its derivative with respect to the N local coefficients:
    der has shape val.shape + (N,).  Written from the operations the weak
    forms apply (slicing, @ with arrays, scalar and array products, sums,
    .T, reshape, item assignment)."""

    __array_ufunc__ = None  # ndarray op VecValDer defers to the reflected method

    def __init__(self, val, der):
        self.val = np.asarray(val, dtype=np.float64)
        self.der = np.asarray(der, dtype=np.float64)

    @property
    def n(self):
        return self.der.shape[-1]

    @property
    def shape(self):
        return self.val.shape

    def _lift(self, o):
        if isinstance(o, VecValDer):
            return o
        a = np.asarray(o, dtype=np.float64)
        return VecValDer(a, _np_zeros(a.shape + (self.n,)))

    def __add__(self, o):
        o = self._lift(o)
        return VecValDer(self.val + o.val, self.der + o.der)

    __radd__ = __add__

    def __neg__(self):
        return VecValDer(-self.val, -self.der)

    def __sub__(self, o):
        return self + (-self._lift(o))

    def __rsub__(self, o):
        return self._lift(o) - self

    def __mul__(self, o):
        if isinstance(o, VecValDer):
            return VecValDer(self.val * o.val, self.der * o.val[..., None] + self.val[..., None] * o.der)
        a = np.asarray(o, dtype=np.float64)
        return VecValDer(self.val * a, self.der * a[..., None])

    __rmul__ = __mul__

    def __truediv__(self, o):
        a = np.asarray(o, dtype=np.float64)
        return VecValDer(self.val / a, self.der / a[..., None])

    def __matmul__(self, o):
        if isinstance(o, VecValDer):
            raise NotImplementedError("product of two differentiated operands")
        a = np.asarray(o, dtype=np.float64)
        if a.ndim == 1:
            return VecValDer(self.val @ a, np.einsum("...kn,k->...n", self.der, a))
        return VecValDer(self.val @ a, np.einsum("...kn,km->...mn", self.der, a))

    def __rmatmul__(self, o):
        a = np.asarray(o, dtype=np.float64)
        if self.val.ndim == 1:
            return VecValDer(a @ self.val, np.einsum("pk,kn->pn", a, self.der))
        return VecValDer(a @ self.val, np.einsum("pk,kmn->pmn", a, self.der))

    @property
    def T(self):
        k = self.val.ndim
        return VecValDer(self.val.T, self.der.transpose(tuple(reversed(range(k))) + (k,)))

    def reshape(self, *shape):
        if len(shape) == 1 and isinstance(shape[0], tuple):
            shape = shape[0]
        return VecValDer(self.val.reshape(shape), self.der.reshape(tuple(shape) + (self.n,)))

    def __getitem__(self, idx):
        return VecValDer(self.val[idx], self.der[idx])

    def __setitem__(self, idx, o):
        o = self._lift(o)
        self.val[idx] = o.val
        self.der[idx] = o.der


class AutoDiff:
    """`with AutoDiff(alpha) as alpha:` yields alpha as a (1, N) row carrying
    the identity derivative; arrays the form creates with np.zeros inside the
    block carry a (zero) derivative too, so entries assigned into them keep
    theirs."""

    def __init__(self, x):
        self.x = np.asarray(x, dtype=np.float64).ravel()

    def __enter__(self):
        n = self.x.size
        real_zeros = _np_zeros

        def zeros(shape, dtype=float, *a, **k):
            if dtype not in (float, np.float64) or a or k:
                return real_zeros(shape, dtype, *a, **k)
            shape = (shape,) if np.isscalar(shape) else tuple(shape)
            return VecValDer(real_zeros(shape), real_zeros(shape + (n,)))

        np.zeros = zeros
        return VecValDer(self.x.reshape(1, n), np.eye(n).reshape(1, n, n))

    def __exit__(self, *exc):
        np.zeros = _np_zeros
        return False


auto_diff = types.ModuleType("auto_diff")
auto_diff.AutoDiff = AutoDiff
auto_diff.VecValDer = VecValDer
auto_diff.vecvalder = types.ModuleType("auto_diff.vecvalder")
auto_diff.vecvalder.VecValDer = VecValDer

sys.modules.update({"meshio": meshio, "basix": basix, "matplotlib": matplotlib,
                    "matplotlib.pyplot": matplotlib.pyplot, "auto_diff": auto_diff,
                    "auto_diff.vecvalder": auto_diff.vecvalder})
if REF_SRC is None:
    raise ImportError("make_golden.py runs as a script (it needs the reference's src/ directory)")
sys.path.insert(0, REF_SRC)

from mesh.mesh import Mesh  # noqa: E402
from spaces.product_space import ProductSpace  # noqa: E402
from assembly.SequentialAssembler import SequentialAssembler  # noqa: E402
from basis.permute_and_transform import (  # noqa: E402
    _validate_edge_orientation_2d, _validate_face_orientation_3d)
from weak_forms.laplace_dual_weak_form import LaplaceDualWeakForm  # noqa: E402
from weak_forms.le_primal_weak_form import LEPrimalWeakForm  # noqa: E402
from weak_forms.lce_dual_weak_form import LCEDualWeakForm  # noqa: E402
from weak_forms.lce_scaled_riesz_map_weak_form import LCEScaledRieszMapWeakForm  # noqa: E402
from weak_forms.le_riesz_map_weak_form import LERieszMapWeakForm  # noqa: E402
from weak_forms.le_dual_weak_form import LEDualWeakForm  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
from cases import FORM_FUNCTIONS, FORM_FUNCTIONS_DEVICE, LE_RIESZ_FUNCTIONS, RIESZ_FUNCTIONS  # noqa: E402


class RecordingMat:
    """Stands in for a PETSc Mat: records every setValue(addv=True)."""

    def __init__(self):
        self.entries = {}

    def setValue(self, row, col, value, addv=True):
        key = (int(row), int(col))
        self.entries[key] = self.entries.get(key, 0.0) + float(value)


class CountingForm:
    """A weak form whose element Jacobian is all ones (counts contributions)."""

    def __init__(self, space):
        self.space = space

    def evaluate_form(self, i, alpha):
        n = len(alpha)
        return np.zeros(n), np.ones((n, n))


def kind_of(name):
    return name.split("_")[0].rstrip("23d")


def element_forms(name, space, n_el, functions=None):
    """r_el, j_el of every cell from the reference's own weak form (alpha = 0)."""
    kind = name.split("_")[0].rstrip("23d")
    if kind == "darcy":
        wf = LaplaceDualWeakForm(space)
        ev = wf.evaluate_form
    elif kind == "elast":
        wf = LEPrimalWeakForm(space)
        ev = wf.evaluate_form
    elif kind == "le":
        wf = LEDualWeakForm(space)
        ev = wf.evaluate_form_vectorized
    else:
        wf = LCEDualWeakForm(space)
        ev = wf.evaluate_form_vectorized
    wf.functions = (functions or FORM_FUNCTIONS)[kind]
    rs, js = [], []
    for i in range(n_el):
        n = len(space.destination_indexes(i))
        r, j = ev(i, np.zeros(n))
        rs.append(np.asarray(r, dtype=np.float64).ravel())
        js.append(np.asarray(j, dtype=np.float64))
    return np.array(rs), np.array(js)


def make_case(name, mesh, fields):
    _MESHES[name] = mesh
    dim = mesh["dim"]
    gmesh = Mesh(dimension=dim, file_name=name)
    gmesh.build_conformal_mesh()
    data = {}
    disc = {}
    for fname, family, degree, nc, dsc in fields:
        data[fname] = (dim, nc, family, degree, gmesh)
        disc[fname] = dsc
    space = ProductSpace(data)
    space.make_subspaces_discontinuous(disc)
    # every tagged facet of the mesh is a boundary element of every field
    b_tags = sorted({int(t) for typ, conn, phys in mesh["blocks"] if mesh_gen.BLOCK_DIM[typ] == dim - 1
                     for t in np.unique(phys)})
    space.build_structures({f[0]: [1] for f in fields}, {f[0]: b_tags for f in fields})
    first = fields[0][0]
    n_el = len(space.discrete_spaces[first].elements)
    dest = np.array([space.destination_indexes(i) for i in range(n_el)], dtype=np.int64)

    mat = RecordingMat()
    res = np.zeros(space.n_dof)
    asm = SequentialAssembler(space, mat, res)
    asm.form_to_input_list = {"count": ["form", range(n_el), CountingForm(space),
                                        np.zeros(space.n_dof)]}
    asm.scatter_forms()
    keys = np.array(sorted(mat.entries.keys()), dtype=np.int64)
    mult = np.array([mat.entries[tuple(k)] for k in keys])

    out = {"cell_dofs": dest, "n_dof": np.int64(space.n_dof),
           "pattern_rows": keys[:, 0], "pattern_cols": keys[:, 1], "multiplicity": mult,
           "points": mesh["points"]}
    # node tags of the elements (file order of the cells)
    out["cell_vertices"] = np.array(
        [space.discrete_spaces[first].elements[i].data.cell.node_tags for i in range(n_el)],
        dtype=np.int64)

    rt_fields = [f for f in fields if f[1] == "RT"]
    if rt_fields:
        fe_list = space.discrete_spaces[rt_fields[0][0]].elements
        if dim == 2:
            flags = np.array([_validate_edge_orientation_2d(fe.data) for fe in fe_list])
            out["edge_oriented"] = flags
        else:
            o, rot, ref = zip(*[_validate_face_orientation_3d(fe.data) for fe in fe_list])
            out["face_oriented"] = np.array(o)
            out["face_rotations"] = np.array(rot)
            out["face_reflections"] = np.array(ref)
            out["bc_entities"] = np.array([fe.data.bc_entities for fe in fe_list])
        pts, wts = space.quadrature[dim]
        dets, invs, tabs = [], [], []
        for fe in fe_list:
            x, jac, det, inv = fe.evaluate_mapping(pts)
            dets.append(det)
            invs.append(inv)
            tabs.append(fe.evaluate_basis(pts, jac, det, inv))
        out["det_jac"] = np.array(dets)
        out["inv_jac"] = np.array(invs)
        out["rt_basis"] = np.array(tabs)
        out["quad_points"] = pts
        out["quad_weights"] = wts
    # boundary elements: DoFs of each (product_space.py:172-201) and the
    # facet's vertices in the reference's node order
    n_bc = len(space.discrete_spaces[first].bc_elements)
    out["bc_tags"] = np.array(b_tags, dtype=np.int64)
    out["bc_dest"] = np.array([space.bc_destination_indexes(i) for i in range(n_bc)], dtype=np.int64)
    out["bc_vertices"] = np.array(
        [space.discrete_spaces[first].bc_elements[i].data.cell.node_tags for i in range(n_bc)], dtype=np.int64)
    if kind_of(name) in FORM_FUNCTIONS:
        out["r_el"], out["j_el"] = element_forms(name, space, n_el)
    kind = kind_of(name)
    if kind in FORM_FUNCTIONS_DEVICE:
        out["r_el_dev"], out["j_el_dev"] = element_forms(name, space, n_el, FORM_FUNCTIONS_DEVICE)
    if name.startswith("le3d"):
        # LERieszMapWeakForm (le_riesz_map_weak_form.py:245-360)
        wf = LERieszMapWeakForm(space)
        wf.functions = LE_RIESZ_FUNCTIONS
        out["j_riesz"] = np.array([np.asarray(wf.evaluate_form_vectorized(i, np.zeros(dest.shape[1]))[1])
                                   for i in range(n_el)])
    if name.startswith("cosserat"):
        # LCEScaledRieszMapWeakForm (lce_scaled_riesz_map_weak_form.py:415-598)
        wf = LCEScaledRieszMapWeakForm(space)
        wf.functions = RIESZ_FUNCTIONS
        out["j_riesz"] = np.array([np.asarray(wf.evaluate_form_vectorized(i, np.zeros(dest.shape[1]))[1])
                                   for i in range(n_el)])
    if "msh" in name:  # the parsed gmsh mesh travels inside the fixture
        out["mesh_dim"] = np.int64(dim)
        for i, (typ, conn, phys) in enumerate(mesh["blocks"]):
            out[f"block{i}_type"] = np.array(typ)
            out[f"block{i}_conn"] = np.asarray(conn, dtype=np.int64)
            out[f"block{i}_phys"] = np.asarray(phys, dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "cells", n_el, "n_dof", space.n_dof, "nnz", len(keys))


def main():
    darcy = [("u", "RT", 1, 1, False), ("p", "Lagrange", 0, 1, True)]
    make_case("darcy2d_n4", mesh_gen.square(4), darcy)
    make_case("darcy3d_n2", mesh_gen.cube(2), darcy)
    make_case("elast3d_n2", mesh_gen.cube(2), [("u", "Lagrange", 2, 3, False)])
    make_case("elast2d_n3", mesh_gen.square(3), [("u", "Lagrange", 2, 2, False)])
    # a mesh gmsh made (the reference's own fixture), read with this
    # package's gmsh 4.1 reader; the reference's mesh / DoF-map code then
    # numbers it through the meshio stand-in
    from nfempy_gb300.gmsh import read_msh
    msh = read_msh(os.path.join(os.path.dirname(REF_SRC), "examples", "cosserat_elasticity", "gmsh_files", "ex_3",
                                "example_3_3d_l_0.msh"))
    msh = {"dim": 3, "points": msh["points"], "blocks": msh["blocks"]}
    make_case("darcy3d_msh0", msh, darcy)
    make_case("cosserat3d_msh0", msh,
              [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False),
               ("u", "Lagrange", 0, 3, True), ("t", "Lagrange", 0, 3, True)])
    le = [("s", "RT", 1, 3, False), ("u", "Lagrange", 0, 3, True), ("t", "Lagrange", 0, 3, True)]
    make_case("le3d_n1", mesh_gen.cube(1), le)
    make_case("le3d_msh0", msh, le)
    make_case("cosserat3d_n1", mesh_gen.cube(1),
              [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False),
               ("u", "Lagrange", 0, 3, True), ("t", "Lagrange", 0, 3, True)])


if __name__ == "__main__":
    main()
