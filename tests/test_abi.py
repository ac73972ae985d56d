"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU calls)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from nfempy_gb300 import _lib, build, meshes, quadrature
from oracle import mesh_gen
from oracle import quadrature as oquad

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        syms |= set(re.findall(r"\b(nfem_[a-z0-9_]+)\s*\(", txt))
    return syms


@pytest.fixture(scope="module")
def lib_path():
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.LIB_PATH


def test_library_exports_header(lib_path):
    h = ctypes.CDLL(lib_path)
    syms = header_symbols()
    assert len(syms) >= 10
    missing = [s for s in sorted(syms) if not hasattr(h, s)]
    assert not missing, missing
    # every symbol bound in ctypes is declared in the header and vice versa
    assert set(_lib.exported_symbols()) == syms


def test_status_strings(lib_path):
    lib = _lib.lib()
    assert lib.nfem_abi_version() >= 1
    assert lib.nfem_status_string(0) == b"ok"
    assert lib.nfem_status_string(6).startswith(b"assembled row")


def test_workspace_queries(lib_path):
    lib = _lib.lib()
    b = ctypes.c_size_t(0)
    assert lib.nfem_scan_workspace_bytes(1000, ctypes.byref(b)) == 0 and b.value > 0
    assert lib.nfem_numbering_workspace_bytes(100, 3, 2, 50, 10, ctypes.byref(b)) == 0 and b.value > 0
    assert lib.nfem_numbering_workspace_bytes(100, 3, 3, 50, 10, ctypes.byref(b)) == 1  # entity_dim == cell_dim
    assert lib.nfem_pattern_workspace_bytes(100, 5, 300, ctypes.byref(b)) == 0 and b.value > 0
    assert lib.nfem_pattern_workspace_bytes(-1, 5, 300, ctypes.byref(b)) == 1


@pytest.mark.parametrize("dim,order", [(1, 3), (2, 3), (2, 5), (3, 3), (3, 5)])
def test_product_quadrature_matches_oracle(dim, order):
    a = quadrature.make_quadrature(dim, order)
    b = oquad.make_quadrature(dim, order)
    np.testing.assert_allclose(a[0], b[0], atol=1e-15)
    np.testing.assert_allclose(a[1], b[1], atol=1e-15)


@pytest.mark.parametrize("gen,n", [("square", 3), ("square", 8), ("cube", 2), ("cube", 3)])
def test_product_meshes_match_oracle(gen, n):
    a = getattr(meshes, gen)(n)
    b = getattr(mesh_gen, gen)(n)
    np.testing.assert_array_equal(a["points"], b["points"])
    assert len(a["blocks"]) == len(b["blocks"])
    for (ta, ca, pa), (tb, cb, pb) in zip(a["blocks"], b["blocks"]):
        assert ta == tb
        np.testing.assert_array_equal(ca, cb)
        np.testing.assert_array_equal(pa, pb)


def test_grf_is_seeded():
    x = np.random.default_rng(0).random((100, 3))
    a = meshes.grf_log_field(x, 0.1, 1.0, 7, device="cpu")
    b = meshes.grf_log_field(x, 0.1, 1.0, 7, device="cpu")
    c = meshes.grf_log_field(x, 0.1, 1.0, 8, device="cpu")
    # the same seed gives the same field (up to the summation order a
    # multi-threaded host matmul may pick)
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-12)
    assert np.abs(a - c).max() > 1e-3
    big = meshes.grf_log_field(np.random.default_rng(1).random((20000, 3)) * 50, 0.1, 2.0, 3, device="cpu")
    assert abs(big.std() - 2.0) < 0.15


def test_new_workspace_queries_and_argument_checks(lib_path):
    """Host-side checks of the entry points added for the P2 elasticity and
    Cosserat geometry workspaces, the copy helper and the chunk table: sizes,
    and invalid arguments refused before any device work."""
    lib = _lib.lib()
    b = ctypes.c_size_t(0)
    assert lib.nfem_elasticity_p2_workspace_bytes(_lib.NFEM_F32, 1000, ctypes.byref(b)) == 0 and b.value == 48000
    assert lib.nfem_elasticity_p2_workspace_bytes(_lib.NFEM_F64, 1000, ctypes.byref(b)) == 0 and b.value == 96000
    assert lib.nfem_cosserat_workspace_bytes(_lib.NFEM_F32, 10, ctypes.byref(b)) == 0 and b.value == 480
    assert lib.nfem_elasticity_p2_workspace_bytes(7, 10, ctypes.byref(b)) == 1
    assert lib.nfem_cosserat_workspace_bytes(_lib.NFEM_F32, -1, ctypes.byref(b)) == 1
    assert lib.nfem_copy_bytes(None, None, 0, None) == 0          # nothing to copy
    assert lib.nfem_copy_bytes(None, None, 16, None) == 1         # null pointers
    # chunk table: a layout that is not flux rows + one pressure row per cell
    assert lib.nfem_pattern_darcy_chunks(None, 10, 5, 4, 7, None, None, None) == 1     # null table
    dummy = ctypes.c_void_p(64)
    rc = lib.nfem_pattern_darcy_chunks(dummy, 10, 5, 4, 7, dummy, None, None)  # p_base + n_cells != n_rows
    assert _lib.STATUS_NAMES[rc] == "NFEM_ERR_UNSUPPORTED"
    # Darcy assembly: bad dimension, value type, and a chunk table that does not fit the rows
    args = [0] * 26
    assert lib.nfem_darcy_rt1p0_assemble(4, 1, *args[2:]) == 1
    assert lib.nfem_darcy_rt1p0_assemble(3, 9, *args[2:]) == 1
    # record workspace of the two-pass form: 8 FP32 words per cell and the list of badly shaped
    # cells (a count, one index per cell), 11 / 8 FP64 words (3-D / 2-D)
    assert lib.nfem_darcy_workspace_bytes(3, _lib.NFEM_F32, 1000, ctypes.byref(b)) == 0 and b.value == 32000 + 4016
    assert lib.nfem_darcy_workspace_bytes(3, _lib.NFEM_F64, 1000, ctypes.byref(b)) == 0 and b.value == 88000
    assert lib.nfem_darcy_workspace_bytes(2, _lib.NFEM_F64, 1000, ctypes.byref(b)) == 0 and b.value == 64000
    assert lib.nfem_darcy_workspace_bytes(4, _lib.NFEM_F32, 10, ctypes.byref(b)) == 1
    # fused FP64 form: plan size (header, one word per 32-row chunk, the schedule, one flag
    # per 32-cell chunk), and its checks before any device work
    T, p_base = 1000, 2100
    rec_chunks, row_chunks = -(-T // 32), -(-p_base // 32)
    sync_word = (4 + row_chunks + rec_chunks + row_chunks + 3) // 4 * 4
    assert lib.nfem_darcy_fused_plan_bytes(T, p_base, ctypes.byref(b)) == 0
    assert b.value == 4 * (sync_word + rec_chunks)
    assert lib.nfem_darcy_fused_plan_bytes(-1, p_base, ctypes.byref(b)) == 1
    assert _lib.STATUS_NAMES[lib.nfem_darcy_fused_plan_bytes(2 ** 31, p_base, ctypes.byref(b))] == "NFEM_ERR_OVERFLOW"
    assert lib.nfem_darcy_fused_plan(None, T, p_base, 0, None, 0, None) == 1             # no plan buffer
    assert lib.nfem_darcy_fused_plan(dummy, T, p_base, -1, dummy, b.value, None) == 1    # negative lead
    fused = [0] * 24
    assert lib.nfem_darcy_rt1p0_assemble_fused(T, T + p_base + 1, *fused[2:]) == 1       # n_rows != p_base + T


def test_two_level_ap_queries_and_argument_checks(lib_path):
    """Host-side checks of the A P pattern entry points: the workspace size
    grows with the rows, and missing structures are refused before any device
    work."""
    lib = _lib.lib()
    b = ctypes.c_size_t(0)
    assert lib.nfem_two_level_ap_workspace_bytes(1000, ctypes.byref(b)) == 0
    small = b.value
    assert lib.nfem_two_level_ap_workspace_bytes(100000, ctypes.byref(b)) == 0 and b.value > small > 12000
    assert lib.nfem_two_level_ap_workspace_bytes(-1, ctypes.byref(b)) == 1
    nnz = ctypes.c_int64(0)
    csr = _lib.Csr(10, None, None, None, _lib.NFEM_F32)
    tl = _lib.TwoLevel()
    # no P aggregates, then no CSR arrays
    assert lib.nfem_two_level_ap_pattern(ctypes.byref(csr), ctypes.byref(tl), None, 0, ctypes.c_void_p(64), None,
                                         ctypes.byref(nnz), None, None) == 1
    tl.p_agg = 64
    assert lib.nfem_two_level_ap_pattern(ctypes.byref(csr), ctypes.byref(tl), None, 0, ctypes.c_void_p(64), None,
                                         ctypes.byref(nnz), None, None) == 1
    csr2 = _lib.Csr(10, 64, 64, None, _lib.NFEM_F32)
    assert lib.nfem_two_level_ap_pattern(ctypes.byref(csr2), ctypes.byref(tl), None, 0, ctypes.c_void_p(64), None,
                                         ctypes.byref(nnz), None, None) == 3  # NFEM_ERR_WORKSPACE


def test_precond_setup_checks_arguments_before_launching(lib_path):
    """nfem_precond_setup refuses bad arguments before any device work: a
    smoother matrix that does not share A's pattern, an unsupported block
    size, an FP32 matrix where the FP64 one is needed."""
    lib = _lib.lib()
    fake = 64
    A64 = _lib.Csr(100, fake, fake, fake, _lib.NFEM_F64)
    pc = _lib.Precond(_lib.PC_CELL_BLOCK, 5, 20, fake, fake, fake, fake, None, None, None, None)
    other = _lib.Csr(100, fake + 16, fake, fake, _lib.NFEM_F32)
    pc.smoother = ctypes.pointer(other)
    assert lib.nfem_precond_setup(ctypes.byref(pc), ctypes.byref(A64), None, None) == 1
    pc.smoother = None
    pc.n_loc = 33  # cell blocks of 4 to 32 DoFs
    assert lib.nfem_precond_setup(ctypes.byref(pc), ctypes.byref(A64), None, None) == 7  # NFEM_ERR_UNSUPPORTED
    pc.n_loc = 3
    assert lib.nfem_precond_setup(ctypes.byref(pc), ctypes.byref(A64), None, None) == 7
    A32 = _lib.Csr(100, fake, fake, fake, _lib.NFEM_F32)
    assert lib.nfem_precond_setup(ctypes.byref(pc), ctypes.byref(A32), None, None) == 1


def test_status_string_for_every_code(lib_path):
    lib = _lib.lib()
    for code, name in _lib.STATUS_NAMES.items():
        s = lib.nfem_status_string(code)
        assert s and s != b"unknown status", name
    assert lib.nfem_status_string(999) == b"unknown status"
