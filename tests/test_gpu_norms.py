"""Device norms against the oracle's restatement of the reference's
post-processing loops (oracle/solve.field_error): l2_error for vector P2 and
for the RT1 rows and P0 vectors of the Cosserat layout, div_error,
div_scaled_error, and the exact-field norms l2_norm / div_norm.  FP64 on
both sides: 1e-12 relative."""
import numpy as np
import pytest

import nfempy_gb300 as nf
from oracle import mesh_gen, quadrature, solve, topology
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu
COS = [("s", "RT", 1, 3, False), ("m", "RT", 1, 3, False), ("u", "P", 0, 3, True), ("t", "P", 0, 3, True)]


def tensor_field(x, y, z):
    """[3, 3, ...]: rows of a smooth tensor field (called on arrays or points)."""
    return np.array([[np.sin(x) + y, x * z, 1.0 + 0 * x],
                     [y * y, np.cos(z), x - y],
                     [z, x * y * z, np.exp(0.3 * x)]])


def vector_field(x, y, z):
    return np.array([np.sin(np.pi * x) * y, z * z + x, np.cos(y)])


def div_field(x, y, z):
    return np.array([np.cos(x) + z, y * y, x + 2.0 * z])


def test_vector_p2_l2_error(cuda_lib):
    m = mesh_gen.cube(3)
    sp = product_space(m, [("u", "P", 2, 3, False)])
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec("u", "P", 2, 3)])
    rng = np.random.default_rng(5)
    alpha = rng.normal(size=nd)
    quad = quadrature.make_quadrature(3, 5)
    X = m["points"][topo.cells]
    got = nf.l2_error(3, sp, {"u": vector_field}, alpha)
    want = solve.field_error("Lagrange", 3, quad, X, None, cd, 3, 2, alpha, vector_field)
    np.testing.assert_allclose(got, [want], rtol=1e-12)
    np.testing.assert_allclose(nf.l2_norm(3, sp, {"u": vector_field}),
                               [solve.field_error("Lagrange", 3, quad, X, None, cd, 3, 2, None, vector_field)],
                               rtol=1e-12)


def test_cosserat_layout_errors_and_norms(cuda_lib):
    m = mesh_gen.cube(2)
    sp = product_space(m, COS)
    topo = topology.Topology(m)
    cd, nd = topology.cell_dofs(topo, [topology.FieldSpec(*f) for f in COS])
    np.testing.assert_array_equal(sp.all_destination_indexes(), cd)
    rng = np.random.default_rng(6)
    alpha = rng.normal(size=nd)
    quad = quadrature.make_quadrature(3, 3)
    X = m["points"][topo.cells]
    s = topo.rt1_signs()
    fns = {"s": tensor_field, "m": tensor_field, "u": vector_field, "t": vector_field,
           "div_s": div_field, "div_m": div_field,
           "l": lambda x, y, z: 1.0 + 0.5 * x * y, "grad_l": lambda x, y, z: np.array([0.5 * y, 0.5 * x, 0 * z])}
    sl = {"s": slice(0, 12), "m": slice(12, 24), "u": slice(24, 27), "t": slice(27, 30)}

    def oracle(name, a, quantity="value"):
        fam, k = ("RT", 1) if name in "sm" else ("Lagrange", 0)
        ex = fns["div_" + name] if quantity != "value" else fns[name]
        return solve.field_error(fam, 3, quad, X, s, cd[:, sl[name]], 3, k, a, ex, quantity, fns["l"], fns["grad_l"])

    np.testing.assert_allclose(nf.l2_error(3, sp, fns, alpha), [oracle(n, alpha) for n in "smut"], rtol=1e-12)
    np.testing.assert_allclose(nf.l2_error(3, sp, fns, alpha, skip_fields=["m", "t"]),
                               [oracle("s", alpha), oracle("u", alpha)], rtol=1e-12)
    np.testing.assert_allclose(nf.div_error(3, sp, fns, alpha), [oracle(n, alpha, "div") for n in "sm"],
                               rtol=1e-12)
    np.testing.assert_allclose(nf.div_scaled_error(3, sp, fns, alpha),
                               [oracle(n, alpha, "div_scaled") for n in "sm"], rtol=1e-12)
    np.testing.assert_allclose(nf.l2_norm(3, sp, fns), [oracle(n, None) for n in "smut"], rtol=1e-12)
    np.testing.assert_allclose(nf.div_norm(3, sp, fns), [oracle(n, None, "div") for n in "sm"], rtol=1e-12)
    assert nf.div_scaled_error(3, sp, {k: v for k, v in fns.items() if k != "l"}, alpha) == []
