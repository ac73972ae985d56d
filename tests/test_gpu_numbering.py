"""Device entity numbering, DoF maps and orientation vs the reference fixtures and the oracle."""
import numpy as np
import pytest
import torch

from oracle import mesh_gen, topology
from tests.cases import CASES, golden
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(CASES))
def test_cell_dofs_match_reference(cuda_lib, name):
    mk, fields = CASES[name]
    g = golden(name)
    sp = product_space(mk(), fields)
    assert sp.n_dof == int(g["n_dof"])
    np.testing.assert_array_equal(sp.all_destination_indexes(), g["cell_dofs"])
    np.testing.assert_array_equal(sp.destination_indexes(3), g["cell_dofs"][3])


@pytest.mark.parametrize("name", sorted(CASES))
def test_bc_dofs_match_reference(cuda_lib, name):
    """Boundary elements (order, node order) and their DoFs against the
    reference's bc_destination_indexes on the same mesh and tags."""
    mk, fields = CASES[name]
    g = golden(name)
    sp = product_space(mk(), fields, b_tags=tuple(int(t) for t in g["bc_tags"]))
    first = fields[0][0]
    n_bc = len(sp.discrete_spaces[first].bc_elements)
    assert n_bc == g["bc_dest"].shape[0]
    got = np.array([sp.bc_destination_indexes(i) for i in range(n_bc)], dtype=np.int64).reshape(g["bc_dest"].shape)
    np.testing.assert_array_equal(got, g["bc_dest"])
    np.testing.assert_array_equal(sp._bc_facets(first)["vertices"], g["bc_vertices"])


@pytest.mark.parametrize("gen,n", [("square", 1), ("square", 7), ("square", 32), ("cube", 1), ("cube", 5),
                                   ("cube", 12)])
def test_numbering_and_flags_match_oracle(cuda_lib, gen, n):
    m = getattr(mesh_gen, gen)(n)
    dim = m["dim"]
    fields_sets = [[("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)], [("u", "P", 2, dim, False)],
                   [("s", "RT", 1, dim, False), ("u", "P", 0, dim, True)]]
    topo = topology.Topology(m)
    for fields in fields_sets:
        sp = product_space(m, fields)
        cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in fields])
        assert sp.n_dof == nd
        np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
        if sp.facet_flags is not None:
            fl = sp.facet_flags.cpu().numpy()
            np.testing.assert_array_equal((fl & 1) != 0, topo.facet_reflected)
            np.testing.assert_array_equal((fl & 2) != 0, topo.facet_tagged)
            mask = sp.rt_sign_mask.cpu().numpy()
            bits = (mask[:, None] >> np.arange(dim + 1)[None, :]) & 1
            np.testing.assert_array_equal(bits == 1, topo.rt1_signs() < 0)


def test_shuffled_cells_and_dof_shift(cuda_lib):
    """First-appearance order follows the given cell order; dof_shift offsets all DoFs."""
    m = mesh_gen.cube(3)
    perm = np.random.default_rng(5).permutation(m["blocks"][-1][1].shape[0])
    blocks = list(m["blocks"])
    t, c, p = blocks[-1]
    blocks[-1] = (t, c[perm], p[perm])
    m2 = {"dim": 3, "points": m["points"], "blocks": blocks}
    fields = [("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)]
    topo = topology.Topology(m2)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in fields], dof_shift=17)
    import nfempy_gb300 as nf
    mesh = nf.Mesh(3, data=m2)
    sp = nf.ProductSpace({"u": (3, 1, "RT", 1, mesh), "p": (3, 1, "Lagrange", 0, mesh)})
    sp.make_subspaces_discontinuous({"p": True})
    sp.dof_shift = 17
    sp.build_structures({"u": [1], "p": [1]}, {})
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
