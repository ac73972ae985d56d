"""gmsh 4.1 ASCII reader (nfempy_gb300.gmsh): a file written from a
synthetic mesh reads back to the same points, blocks and physical tags, and
the reference's own fixture (when the nfempy checkout is present) reads to
the mesh stored in tests/golden/darcy3d_msh0.npz."""
import os

import numpy as np
import pytest

from nfempy_gb300.gmsh import read_msh
from oracle import mesh_gen
from tests.cases import golden_mesh

_TYPE_ID = {"vertex": 15, "line": 1, "triangle": 2, "tetra": 4}
_DIM = {"vertex": 0, "line": 1, "triangle": 2, "tetra": 3}


def write_msh41(path, m):
    """A minimal gmsh 4.1 ASCII file: one entity per (block, physical tag)."""
    pts = m["points"]
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat"]
    ents = {0: [], 1: [], 2: [], 3: []}
    for bi, (typ, conn, phys) in enumerate(m["blocks"]):
        ents[_DIM[typ]].append((bi + 1, int(phys[0])))
    lines.append("$Entities")
    lines.append(" ".join(str(len(ents[d])) for d in range(4)))
    for d in range(4):
        for tag, ph in ents[d]:
            head = [tag] + ([0.0, 0.0, 0.0] if d == 0 else [0.0] * 6)
            lines.append(" ".join(str(v) for v in head) + f" 1 {ph}" + ("" if d == 0 else " 0"))
    lines.append("$EndEntities")
    n = pts.shape[0]
    lines += ["$Nodes", f"1 {n} 1 {n}", f"{m['dim']} 1 0 {n}"]
    lines += [str(i + 1) for i in range(n)]
    lines += [" ".join(repr(float(x)) for x in p) for p in pts]
    lines.append("$EndNodes")
    n_el = sum(len(c) for _, c, _ in m["blocks"])
    lines += ["$Elements", f"{len(m['blocks'])} {n_el} 1 {n_el}"]
    k = 1
    for bi, (typ, conn, phys) in enumerate(m["blocks"]):
        lines.append(f"{_DIM[typ]} {bi + 1} {_TYPE_ID[typ]} {len(conn)}")
        for row in conn:
            lines.append(" ".join([str(k)] + [str(int(v) + 1) for v in row]))
            k += 1
    lines.append("$EndElements")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


@pytest.mark.parametrize("gen,n", [("square", 3), ("cube", 2)])
def test_round_trip(tmp_path, gen, n):
    m = getattr(mesh_gen, gen)(n)
    path = tmp_path / "m.msh"
    write_msh41(path, m)
    r = read_msh(str(path))
    assert r["dim"] == m["dim"]
    np.testing.assert_array_equal(r["points"], m["points"])
    assert len(r["blocks"]) == len(m["blocks"])
    for (t1, c1, p1), (t2, c2, p2) in zip(r["blocks"], m["blocks"]):
        assert t1 == t2
        np.testing.assert_array_equal(c1, c2)
        np.testing.assert_array_equal(p1, p2)


def test_reference_fixture_reads_to_stored_mesh():
    root = os.environ.get("NFEM_REFERENCE_ROOT", os.path.join(os.sep, "root", "reference"))
    path = os.path.join(root, "examples", "cosserat_elasticity", "gmsh_files", "ex_3", "example_3_3d_l_0.msh")
    if not os.path.exists(path):
        pytest.skip("the reference checkout is not present")
    r = read_msh(path)
    g = golden_mesh("darcy3d_msh0")
    np.testing.assert_array_equal(r["points"], g["points"])
    for (t1, c1, p1), (t2, c2, p2) in zip(r["blocks"], g["blocks"]):
        assert t1 == t2
        np.testing.assert_array_equal(c1, c2)
        np.testing.assert_array_equal(p1, p2)
    assert r["physical_names"][(3, 1)] == "domain"
