"""Device CSR pattern (element-clique union) vs the reference fixtures and the oracle."""
import numpy as np
import pytest
import torch

import nfempy_gb300 as nf
from oracle import assembly, mesh_gen, topology
from tests.cases import CASES, golden
from tests.gpu_helpers import product_space

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(CASES))
def test_pattern_matches_reference(cuda_lib, name):
    mk, fields = CASES[name]
    g = golden(name)
    sp = product_space(mk(), fields)
    A = nf.CSRMatrix(sp)
    rp = A.row_ptr.cpu().numpy()
    rows = np.repeat(np.arange(A.n_rows), np.diff(rp))
    np.testing.assert_array_equal(rows, g["pattern_rows"])
    np.testing.assert_array_equal(A.col_idx[: A.nnz].cpu().numpy(), g["pattern_cols"])
    # incidence lists: every (cell, local) occurrence once, sorted per row
    inc_ptr = A.inc_ptr.cpu().numpy()
    inc = A.inc.cpu().numpy()
    cd = g["cell_dofs"]
    n_loc = cd.shape[1]
    for r in range(0, A.n_rows, max(1, A.n_rows // 50)):
        seg = inc[inc_ptr[r]:inc_ptr[r + 1]]
        assert np.all(np.diff(seg) > 0)
        assert np.all(cd[seg // n_loc, seg % n_loc] == r)
    assert inc_ptr[-1] == cd.size


@pytest.mark.parametrize("gen,n", [("square", 32), ("cube", 8)])
def test_pattern_and_slots_match_oracle(cuda_lib, gen, n):
    m = getattr(mesh_gen, gen)(n)
    for fields in ([("u", "RT", 1, 1, False), ("p", "P", 0, 1, True)], [("u", "P", 2, m["dim"], False)]):
        sp = product_space(m, fields)
        A = nf.CSRMatrix(sp)
        cd = sp.all_destination_indexes()
        ip, ix = assembly.pattern_csr(cd, sp.n_dof)
        np.testing.assert_array_equal(A.row_ptr.cpu().numpy(), ip)
        np.testing.assert_array_equal(A.col_idx[: A.nnz].cpu().numpy(), ix)
        T, n_loc = cd.shape
        slots = torch.empty((T, n_loc, n_loc), dtype=torch.int32, device="cuda")
        nf._lib.call("nfem_pattern_slots", nf._lib.ptr(sp.cell_dofs), T, n_loc, n_loc, nf._lib.ptr(A.row_ptr),
                     nf._lib.ptr(A.col_idx), nf._lib.ptr(slots), nf._lib.ptr(A.status), nf._lib.stream_ptr())
        A.check_status("slots")
        s = slots.cpu().numpy()
        rows = np.repeat(cd, n_loc, axis=1).reshape(T, n_loc, n_loc)
        cols = np.tile(cd, (1, n_loc)).reshape(T, n_loc, n_loc)
        np.testing.assert_array_equal(ix[s], cols)
        assert np.all(s >= ip[rows]) and np.all(s < ip[rows + 1])


def test_scan_matches_cumsum(cuda_lib):
    for n in (1, 5, 4096, 4097, 1_000_003):
        x = torch.randint(0, 50, (n,), dtype=torch.int32, device="cuda")
        out = torch.empty(n + 1, dtype=torch.int64, device="cuda")
        b = nf._lib.C.c_size_t(0)
        nf._lib.call("nfem_scan_workspace_bytes", n, nf._lib.C.byref(b))
        ws = torch.empty(int(b.value), dtype=torch.uint8, device="cuda")
        nf._lib.call("nfem_exclusive_scan", nf._lib.ptr(x), n, nf._lib.ptr(out), nf._lib.ptr(ws), ws.numel(),
                     nf._lib.stream_ptr())
        ref = torch.zeros(n + 1, dtype=torch.int64)
        ref[1:] = torch.cumsum(x.cpu().long(), 0)
        assert torch.equal(out.cpu(), ref)
