"""Host-evaluated weak forms through SequentialAssembler's six form types
(src/assembly/SequentialAssembler.py:20-30, src/assembly/ScatterFormData.py:5-79):
element data evaluated per element with the reference's arguments, added
into the device CSR by nfem_scatter_elements."""
import numpy as np
import pytest
import scipy.sparse as sps
import torch

import nfempy_gb300 as nf
from nfempy_gb300 import _lib
from oracle import assembly
from tests.cases import CASES, golden
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu


class GoldenForm:
    """Returns the reference's own element matrices of a fixture (the
    LaplaceDualWeakForm / LEPrimalWeakForm / LCEDualWeakForm evaluate_form
    output at alpha = 0) and records the arguments it was called with."""

    def __init__(self, space, r_el, j_el):
        self.space = space
        self.r_el, self.j_el = r_el, j_el
        self.calls = []

    def evaluate_form(self, i, alpha_l):
        self.calls.append((i, np.array(alpha_l)))
        return self.r_el[i], self.j_el[i]


def coo(dests, rs, js, n):
    R = np.concatenate([np.repeat(d, len(d)) for d in dests])
    C = np.concatenate([np.tile(d, len(d)) for d in dests])
    V = np.concatenate([np.asarray(j).ravel() for j in js])
    A = sps.csr_matrix((V, (R, C)), shape=(n, n))
    A.sum_duplicates()
    res = np.zeros(n)
    for d, r in zip(dests, rs):
        np.add.at(res, d, r)
    return A, res


def dense_of(A):
    return A.to_scipy().toarray()


@pytest.mark.parametrize("name", ["darcy3d_n2", "elast2d_n3", "cosserat3d_msh0"])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_form_of_reference_element_matrices(cuda_lib, name, dtype):
    mk, fields = CASES[name]
    g = golden(name)
    sp = product_space(mk(), fields)
    A = nf.CSRMatrix(sp, dtype=dtype)
    res = A.createVecLeft()
    form = GoldenForm(sp, g["r_el"], g["j_el"])
    asm = nf.SequentialAssembler(sp, A, res)
    alpha = np.arange(sp.n_dof, dtype=np.float64)
    asm.form_to_input_list = {"w": ["form", range(sp.n_cells), form, alpha]}
    asm.scatter_forms()
    A.assemble()
    # each element saw its own slice of alpha (ScatterFormData.py:36-40)
    for i, a in form.calls[:5]:
        np.testing.assert_array_equal(a, alpha[g["cell_dofs"][i]])
    O, ro = assembly.assemble_csr(g["cell_dofs"], g["j_el"], g["r_el"], int(g["n_dof"]))
    tol = 1e-13 if dtype == torch.float64 else 2e-6
    got = dense_of(A)
    scale = np.abs(O.toarray()).max()
    assert np.abs(got - O.toarray()).max() <= tol * scale
    np.testing.assert_allclose(res.double().cpu().numpy(), ro, atol=tol * max(np.abs(ro).max(), 1.0))


def test_device_form_then_host_bc_form(cuda_lib):
    """A device Darcy form followed by a host-evaluated boundary form in one
    pass: the second adds to the first."""
    mk, fields = CASES["darcy3d_n2"]
    g = golden("darcy3d_n2")
    sp = product_space(mk(), fields, b_tags=(2, 3, 4, 5, 6, 7))
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"rhs": lambda x, y, z: np.array([x * 0 + 1.0]), "kappa": lambda x, y, z: np.array([x * 0 + 2.0])}
    A = nf.CSRMatrix(sp)
    res = A.createVecLeft()
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"d": ["form", range(sp.n_cells), wf, None]}
    asm.scatter_forms()
    base = dense_of(A)
    base_r = res.double().cpu().numpy().copy()

    n_bc = len(sp.discrete_spaces["u"].bc_elements)
    rng = np.random.default_rng(3)
    dests = [sp.bc_destination_indexes(i) for i in range(n_bc)]
    rs = [rng.standard_normal(len(d)) for d in dests]
    js = [rng.standard_normal((len(d), len(d))) for d in dests]

    class BC:
        def evaluate_form(self, i, alpha_l):
            return rs[i], js[i]
    A.zeroEntries()
    res.zero_()
    asm.form_to_input_list = {"d": ["form", range(sp.n_cells), wf, None],
                              "bc": ["bc_form", range(n_bc), BC(), np.zeros(sp.n_dof)]}
    asm.scatter_forms()
    O, ro = coo(dests, rs, js, sp.n_dof)
    np.testing.assert_allclose(dense_of(A), base + O.toarray(), rtol=0, atol=1e-13)
    np.testing.assert_allclose(res.double().cpu().numpy(), base_r + ro, rtol=0, atol=1e-13)
    assert g["bc_dest"].shape[0] == n_bc


def interior_pairs(sp):
    """(facet index, (cell p, cell n)) for every interior facet."""
    cd = sp.all_destination_indexes()
    u = sp.field_slices["u"]
    flux = cd[:, u]
    flat = flux.ravel()
    order = np.argsort(flat, kind="stable")
    sflat = flat[order]
    same = np.flatnonzero(sflat[1:] == sflat[:-1])
    cells = order // flux.shape[1]
    return [(k, (int(cells[s]), int(cells[s + 1]))) for k, s in enumerate(same)]


def test_interface_and_bc_interface_forms(cuda_lib):
    mk, fields = CASES["darcy2d_n4"]
    sp = product_space(mk(), fields)
    dest = sp.all_destination_indexes()
    pairs = interior_pairs(sp)
    assert len(pairs) > 0
    rng = np.random.default_rng(5)
    k2 = 2 * dest.shape[1]
    J = rng.standard_normal((len(pairs), k2, k2))
    Rv = rng.standard_normal((len(pairs), k2))
    alpha = rng.standard_normal(sp.n_dof)
    seen = []

    class Interface:
        def evaluate_form(self, idx, idx_pair, alpha_pair):
            p, n = idx_pair
            np.testing.assert_array_equal(alpha_pair[0], alpha[dest[p]])
            np.testing.assert_array_equal(alpha_pair[1], alpha[dest[n]])
            seen.append(idx)
            return Rv[idx], J[idx]

    bc_cells = [(k, int(c)) for k, c in enumerate(rng.choice(sp.n_cells, 5, replace=False))]
    Jb = rng.standard_normal((5, k2 // 2, k2 // 2))
    Rb = rng.standard_normal((5, k2 // 2))

    class BCInterface:
        def evaluate_form(self, idx, idx_p, alpha_l):
            np.testing.assert_array_equal(alpha_l, alpha[dest[idx_p]])
            return Rb[idx], Jb[idx]

    cliques = [np.concatenate([dest[p], dest[n]])[None, :] for _, (p, n) in pairs]
    extra = np.concatenate(cliques)
    A = nf.CSRMatrix(sp, extra_cliques=[extra])
    assert A.extended and A.codes is None
    res = A.createVecLeft()
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"i": ["interface_form", pairs, Interface(), alpha],
                              "b": ["bc_interface_form", bc_cells, BCInterface(), alpha]}
    asm.scatter_forms()
    assert sorted(seen) == list(range(len(pairs)))
    dests = [np.concatenate([dest[p], dest[n]]) for _, (p, n) in pairs] + [dest[c] for _, c in bc_cells]
    O, ro = coo(dests, list(Rv) + list(Rb), list(J) + list(Jb), sp.n_dof)
    np.testing.assert_allclose(dense_of(A), O.toarray(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(res.double().cpu().numpy(), ro, rtol=0, atol=1e-12)
    # the device Darcy form refuses a matrix with extra cliques
    wf = nf.LaplaceDualWeakForm(sp)
    wf.functions = {"rhs": lambda x, y, z: np.array([x * 0]), "kappa": lambda x, y, z: np.array([x * 0 + 1.0])}
    with pytest.raises(NotImplementedError):
        wf.assemble(A, res)


def test_interface_form_outside_pattern_sets_status(cuda_lib):
    """Couplings between two cells' DoFs are not in the cell-clique pattern:
    the scatter reports NFEM_ERR_PATTERN (entries skipped, no fault)."""
    mk, fields = CASES["darcy2d_n4"]
    sp = product_space(mk(), fields)
    dest = sp.all_destination_indexes()
    far = (0, (0, sp.n_cells - 1))
    k2 = 2 * dest.shape[1]

    class Interface:
        def evaluate_form(self, idx, idx_pair, alpha_pair):
            return np.ones(k2), np.ones((k2, k2))
    A = nf.CSRMatrix(sp)
    res = A.createVecLeft()
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"i": ["interface_form", [far], Interface(), None]}
    with pytest.raises(_lib.NfemError) as e:
        asm.scatter_forms()
    assert _lib.STATUS_NAMES[e.value.status] == "NFEM_ERR_PATTERN"


def test_time_dependent_forms(cuda_lib):
    mk, fields = CASES["elast2d_n3"]
    g = golden("elast2d_n3")
    sp = product_space(mk(), fields, b_tags=tuple(int(t) for t in g["bc_tags"]))
    dest = sp.all_destination_indexes()
    rng = np.random.default_rng(7)
    alpha_n = rng.standard_normal(sp.n_dof)
    alpha = rng.standard_normal(sp.n_dof)
    t = 0.25

    class TD:
        def evaluate_form(self, i, a_n, a, tt):
            np.testing.assert_array_equal(a_n, alpha_n[dest[i]])
            np.testing.assert_array_equal(a, alpha[dest[i]])
            return (a - a_n) / tt, tt * np.eye(len(a)) + np.outer(a, a_n)

    class TDBC:
        def evaluate_form(self, i, a, tt):
            # the reference slices alpha_n for the boundary term (ScatterFormData.py:43-49)
            np.testing.assert_array_equal(a, alpha_n[g["bc_dest"][i]])
            return tt * a, np.outer(a, a)

    n_bc = g["bc_dest"].shape[0]
    A = nf.CSRMatrix(sp)
    res = A.createVecLeft()
    asm = nf.SequentialAssembler(sp, A, res)
    asm.form_to_input_list = {"td": ["time_dependent_form", range(sp.n_cells), TD(), (alpha_n, alpha), t],
                              "bc": ["time_dependent_bc_form", range(n_bc), TDBC(), (alpha_n, alpha), t]}
    asm.scatter_forms()
    dests = [dest[i] for i in range(sp.n_cells)] + [g["bc_dest"][i] for i in range(n_bc)]
    rs = [(alpha[d] - alpha_n[d]) / t for d in dests[:sp.n_cells]] + [t * alpha_n[d] for d in dests[sp.n_cells:]]
    js = ([t * np.eye(len(d)) + np.outer(alpha[d], alpha_n[d]) for d in dests[:sp.n_cells]]
          + [np.outer(alpha_n[d], alpha_n[d]) for d in dests[sp.n_cells:]])
    O, ro = coo(dests, rs, js, sp.n_dof)
    np.testing.assert_allclose(dense_of(A), O.toarray(), rtol=0, atol=1e-12)
    np.testing.assert_allclose(res.double().cpu().numpy(), ro, rtol=0, atol=1e-12)
    # a host residual array is updated in place, like the reference's numpy residual
    A.zeroEntries()
    host = np.zeros(sp.n_dof)
    asm2 = nf.SequentialAssembler(sp, A, host)
    asm2.form_to_input_list = asm.form_to_input_list
    asm2.scatter_forms()
    np.testing.assert_allclose(host, ro, rtol=0, atol=1e-12)


def test_set_value_like_the_reference_scatter(cuda_lib):
    """The reference's own scatter loop (ScatterFormData.py:5-11: one
    Mat.setValue(addv=True) per entry) against a CSRMatrix: buffered on the
    host, added on the device at assemble()."""
    mk, fields = CASES["darcy2d_n4"]
    g = golden("darcy2d_n4")
    sp = product_space(mk(), fields)
    A = nf.CSRMatrix(sp)
    for i in range(sp.n_cells):
        d = g["cell_dofs"][i]
        data = g["j_el"][i].ravel()
        row = np.repeat(d, len(d))
        col = np.tile(d, len(d))
        for k in range(len(data)):
            A.setValue(row=row[k], col=col[k], value=data[k], addv=True)
    A.assemble()
    O, _ = assembly.assemble_csr(g["cell_dofs"], g["j_el"], g["r_el"], int(g["n_dof"]))
    np.testing.assert_allclose(dense_of(A), O.toarray(), rtol=0, atol=1e-14 * np.abs(O.data).max())
    assert A.getValue(int(g["cell_dofs"][0][0]), int(g["cell_dofs"][0][1])) == pytest.approx(
        O[int(g["cell_dofs"][0][0]), int(g["cell_dofs"][0][1])], abs=1e-14)
    # a coupling outside the pattern is reported at assemble()
    A.setValue(0, sp.n_dof - 1, 1.0)
    with pytest.raises(_lib.NfemError):
        A.assemble()
