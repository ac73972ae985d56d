"""ctypes binding of libnfem_gb300.so (the C ABI declared in include/nfem_gb300.h).

The library is required: every compute entry point of the package goes
through it, and importing a function from here raises when the library is
missing.  There is no CPU fallback.
"""
import ctypes as C
import os

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("NFEM_GB300_LIB", os.path.join(HERE, "libnfem_gb300.so"))

NFEM_OK = 0
NFEM_F64 = 0
NFEM_F32 = 1
NFEM_BF16 = 2
COEF_NONE, COEF_CELL, COEF_QPOINT = 0, 1, 2
DARCY_CHUNK_CELLS = 32  # NFEM_DARCY_CHUNK_CELLS
COARSE_BLOCK_MAX = 1024  # NFEM_COARSE_BLOCK_MAX

STATUS_NAMES = {
    0: "NFEM_OK", 1: "NFEM_ERR_INVALID_ARG", 2: "NFEM_ERR_CUDA", 3: "NFEM_ERR_WORKSPACE",
    4: "NFEM_ERR_OVERFLOW", 5: "NFEM_ERR_CAPACITY", 6: "NFEM_ERR_PATTERN", 7: "NFEM_ERR_UNSUPPORTED",
    8: "NFEM_ERR_NOT_CONVERGED", 9: "NFEM_ERR_BREAKDOWN", 10: "NFEM_ERR_NONFINITE",
    11: "NFEM_ERR_DEGENERATE", 12: "NFEM_ERR_DOMAIN", 13: "NFEM_ERR_TIMEOUT",
}


class NfemError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = int(status)
        name = STATUS_NAMES.get(self.status, str(status))
        super().__init__(f"{where}: {name}" if where else name)


class DofBlock(C.Structure):
    _fields_ = [("occ_rank", C.c_void_p), ("n_ent", C.c_int32), ("width", C.c_int32), ("base", C.c_int64)]


class DarcySlices(C.Structure):
    _fields_ = [("slice_shift", C.c_int32), ("lookahead_cells", C.c_int32), ("record_quarters", C.c_int32),
                ("flux_row_begin", C.c_void_p)]


class Csr(C.Structure):
    _fields_ = [("n_rows", C.c_int64), ("row_ptr", C.c_void_p), ("col_idx", C.c_void_p), ("values", C.c_void_p),
                ("value_type", C.c_int)]


class TwoLevel(C.Structure):
    _fields_ = [("p_base", C.c_int64), ("n_agg", C.c_int32), ("cell_agg", C.c_void_p), ("w", C.c_void_p),
                ("p_agg", C.c_void_p), ("p_val", C.c_void_p), ("pt_nnz", C.c_int64), ("pt_ptr", C.c_void_p),
                ("pt_row", C.c_void_p), ("pt_slot", C.c_void_p), ("pt_val", C.c_void_p), ("ac", C.c_void_p),
                ("gj", C.c_void_p), ("ac_inv", C.c_void_p), ("work", C.c_void_p), ("n_blocks", C.c_int32),
                ("blk_max", C.c_int32), ("ac_entries", C.c_int64), ("blk_ptr", C.c_void_p), ("blk_off", C.c_void_p),
                ("agg_blk", C.c_void_p), ("ap_nnz", C.c_int64), ("ap_ptr", C.c_void_p), ("ap_col", C.c_void_p),
                ("ap_val", C.c_void_p), ("omega", C.c_float), ("post_smooth", C.c_int32)]


class Precond(C.Structure):
    _fields_ = [("kind", C.c_int), ("n_loc", C.c_int), ("n_cells", C.c_int64), ("cell_dofs", C.c_void_p),
                ("inc_ptr", C.c_void_p), ("inc", C.c_void_p), ("block_inv", C.c_void_p), ("diag_inv", C.c_void_p),
                ("wsqrt", C.c_void_p), ("winvsqrt", C.c_void_p), ("setup_scratch", C.c_void_p),
                ("two_level", C.POINTER(TwoLevel)), ("a32", C.POINTER(Csr)), ("smoother", C.POINTER(Csr))]


class SolveParams(C.Structure):
    _fields_ = [("rtol", C.c_double), ("inner_rtol", C.c_double), ("restart", C.c_int), ("max_inner", C.c_int),
                ("max_outer", C.c_int), ("snapshots", C.c_void_p), ("max_snapshots", C.c_int),
                ("no_graphs", C.c_int), ("schedule", C.c_void_p), ("schedule_capacity", C.c_int),
                ("schedule_mode", C.c_int), ("relres_out", C.c_void_p)]


class SolveInfo(C.Structure):
    _fields_ = [("inner_iterations", C.c_int), ("outer_iterations", C.c_int), ("initial_relres", C.c_double),
                ("final_relres", C.c_double), ("status", C.c_int), ("n_snapshots", C.c_int)]


PC_NONE, PC_JACOBI, PC_CELL_BLOCK, PC_TWO_LEVEL, PC_NODE_BLOCK = 0, 1, 2, 3, 4

_P = C.c_void_p
_I = C.c_int
_I64 = C.c_int64
_SZ = C.c_size_t

_SIGS = {
    "nfem_abi_version": ([], _I),
    "nfem_status_string": ([_I], C.c_char_p),
    "nfem_scan_workspace_bytes": ([_I64, C.POINTER(_SZ)], _I),
    "nfem_exclusive_scan": ([_P, _I64, _P, _P, _SZ, _P], _I),
    "nfem_exclusive_scan_noalloc": ([_P, _I64, _P, _P], _I),
    "nfem_numbering_workspace_bytes": ([_I64, _I, _I, _I64, _I64, C.POINTER(_SZ)], _I),
    "nfem_number_entities": ([_P, _I64, _I, _I, _I64, _P, _I64, _I, _P, _SZ, _P, _P, _P, _P], _I),
    "nfem_rt1_sign_mask": ([_P, _I64, _I, _P, _P], _I),
    "nfem_compose_cell_dofs": ([_I64, _I, C.POINTER(DofBlock), _P, _I, _P], _I),
    "nfem_pattern_workspace_bytes": ([_I64, _I, _I64, C.POINTER(_SZ)], _I),
    "nfem_pattern_rows": ([_P, _I64, _I, _I, _I64, _P, _SZ, _P, _P, _P, C.POINTER(_I64), _P, _P], _I),
    "nfem_pattern_cols": ([_P, _I64, _I, _I, _I64, _P, _P, _P, _P, _P, _P], _I),
    "nfem_pattern_slots": ([_P, _I64, _I, _I, _P, _P, _P, _P, _P], _I),
    "nfem_pattern_local_codes": ([_P, _I64, _I, _I, _I64, _P, _P, _P, _P, _P, _P, _P], _I),
    "nfem_points_split": ([_P, _I64, _P, _P], _I),
    "nfem_points_fixed64": ([_P, _I64, _P, _P], _I),
    "nfem_knob_set": ([_I, _I], _I),
    "nfem_mlp_infer_tc": ([_P, _P, _P, _I64, _P, _P, _P, _P], _I),
    "nfem_csr_add_entries": ([_I, _I64, _P, _P, _P, _P, _P, _I64, _P, _P, _P], _I),
    "nfem_pcg_setup": ([_I, _P, _P, _P, _P], _I),
    "nfem_pcg_workspace_bytes": ([_I64, C.POINTER(_SZ)], _I),
    "nfem_solve_ir_pcg": ([_P, _P, _I, _P, _P, _P, C.c_double, C.c_double, _I, _I, _P, _SZ, _P, _P, _P], _I),
    "nfem_darcy_rt1p0_assemble_pass": ([_I, _I, _I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _I, C.c_void_p, _I, _P, _P,
                                        _P, _P, _P, _I, _P, _SZ, _I, _I64, _I64, _I64, _I64, _I64, _I64, _P, _P], _I),
    "nfem_scatter_elements": ([_I, _I64, _I, _P, _P, _P, _P, _P, _I64, _P, _P, _P, _P], _I),
    "nfem_rt1_dirichlet_rows": ([_I, _I, _I64, _P, _P, _P, _I, _I, _I, C.c_double, _P, C.POINTER(C.c_double), _I,
                                 _P, _P], _I),
    "nfem_knob_get": ([_I, C.POINTER(_I)], _I),
    "nfem_field_error_workspace_bytes": ([_P], _I),
    "nfem_field_error": ([_I, _I, _I, _I64, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _I,
                          _P, _P, _SZ, _P], _I),
    "nfem_pattern_pairs": ([_P, _P, _P, _I64, _P, _P, _P, _P], _I),
    "nfem_darcy_rt1p0_assemble": ([_I, _I, _I64, _I64, _P, _P, _P, _P, _I64, _P, _P, _P, _I,
                                   _P, _I, _P, _P, _P, _P, _P, _P, _I, _P, _SZ, _P, _P], _I),
    "nfem_darcy_workspace_bytes": ([_I, _I, _I64, C.POINTER(_SZ)], _I),
    "nfem_darcy_ring_bytes": ([_I, _I, C.POINTER(_SZ)], _I),
    "nfem_darcy_rt1p0_assemble_sliced": ([_I, _I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _I, _P, _I, _P, _P, _P,
                                          C.POINTER(DarcySlices), _P, _P, _I, _P, _SZ, _P, _P], _I),
    "nfem_darcy_fused_plan_bytes": ([_I64, _I64, C.POINTER(_SZ)], _I),
    "nfem_darcy_fused_plan": ([_P, _I64, _I64, _I, _P, _SZ, _P], _I),
    "nfem_darcy_rt1p0_assemble_fused": ([_I64, _I64, _P, _P, _P, _I64, _P, _P, _P, _I, _P, _I, _P, _P, _P, _P, _SZ,
                                         _P, _P, _I, _P, _SZ, _P, _P], _I),
    "nfem_pattern_darcy_chunks": ([_P, _I64, _I, _I64, _I64, _P, _P, _P], _I),
    "nfem_copy_bytes": ([_P, _P, _SZ, _P], _I),
    "nfem_spmv": ([_I, _I64, _P, _P, _P, _P, _P, _P], _I),
    "nfem_residual_f64": ([_I64, _P, _P, _P, _P, _P, _P, _P], _I),
    "nfem_precond_setup": ([C.POINTER(Precond), C.POINTER(Csr), _P, _P], _I),
    "nfem_precond_apply": ([C.POINTER(Precond), _I64, _P, _P, _P], _I),
    "nfem_two_level_ap_workspace_bytes": ([_I64, C.POINTER(_SZ)], _I),
    "nfem_two_level_ap_pattern": ([C.POINTER(Csr), C.POINTER(TwoLevel), _P, _SZ, _P, _P, C.POINTER(_I64), _P, _P],
                                  _I),
    "nfem_solve_workspace_bytes": ([_I64, _I, C.POINTER(_SZ)], _I),
    "nfem_solve_ir_fgmres": ([C.POINTER(Csr), C.POINTER(Csr), C.POINTER(Precond), _P, _P, C.POINTER(SolveParams),
                              _P, _SZ, C.POINTER(SolveInfo), _P], _I),
    "nfem_mlp_param_count": ([_P, C.POINTER(_I64)], _I),
    "nfem_mlp_forward": ([_P, _I, _P, _P, _I64, _P, _P, _P, _P, _P], _I),
    "nfem_mlp_backward_workspace_bytes": ([_P, _I64, C.POINTER(_SZ)], _I),
    "nfem_mlp_backward": ([_P, _I, _P, _I64, _P, _P, _P, _P, _P, _P, _P, _SZ, _P, _P], _I),
    "nfem_adam_step": ([_I64, _P, _P, _P, _P, C.c_float, C.c_float, C.c_float, C.c_float, _I, _P, _P], _I),
    "nfem_to_bf16": ([_I64, _P, _P, _P], _I),
    "nfem_pattern_node_codes": ([_P, _I64, _I, _I, _I64, _I64, _P, _P, _P, _P, _P, _P, _P], _I),
    "nfem_elasticity_p2_assemble": ([_I, _I64, _I64, _I64, _P, _P, _P, _P, _P, _P, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), _P, _P, _P, _P, _I, _P, _P, _I, _P, _SZ, _P, _P], _I),
    "nfem_elasticity_p2_workspace_bytes": ([_I, _I64, C.POINTER(C.c_size_t)], _I),
    "nfem_elasticity_p2_penalty": ([_I, _I64, _P, _P, _P, C.c_double, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double), _P, _P, _P, _P, _P], _I),
    "nfem_cosserat_assemble": ([_I, _I64, _I64, _I64, _P, _P, _P, _P, C.POINTER(C.c_double), _P,
                                C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), _P, _P, _P,
                                _P, _P, _P, _I, _P, _SZ, _P, _P], _I),
    "nfem_cosserat_riesz_assemble": ([_I, _I64, _I64, _I64, _P, _P, _P, _P, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), _P, _P, _P,
                                      _P, _P, _I, _P, _SZ, _P, _P], _I),
    "nfem_cosserat_workspace_bytes": ([_I, _I64, C.POINTER(C.c_size_t)], _I),
    "nfem_le_dual_assemble": ([_I, _I64, _I64, _I64, _P, _P, _P, _P, C.c_double, C.c_double, _P,
                               C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double), _P, _P, _P, _P,
                               _P, _P, _I, _P, _SZ, _P, _P], _I),
    "nfem_le_riesz_assemble": ([_I, _I64, _I64, _I64, _P, _P, _P, _P, C.c_double, C.c_double, C.POINTER(C.c_double),
                                C.POINTER(C.c_double), C.POINTER(C.c_double), _P, _P, _P, _P, _P, _I, _P, _SZ, _P,
                                _P], _I),
    "nfem_darcy_rt1_dirichlet": ([_I, _I, _I64, _P, _P, _P, _I, _P, C.POINTER(C.c_double), _I, _P, _P], _I),
    "nfem_darcy_l2_error": ([_I, _I64, _P, _P, _P, _P, _I, _P, _P, _P, C.POINTER(C.c_double),
                             C.POINTER(C.c_double), _I, _P, _P, _SZ, _P], _I),
}

_lib = None


def lib():
    """Load the CUDA library once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NfemError(-1, f"{LIB_PATH} is missing: run nfempy_gb300.build.build() (nvcc, sm_103a)")
        h = C.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            f = getattr(h, name)
            f.argtypes = args
            f.restype = res
        _lib = h
    return _lib


def exported_symbols():
    return sorted(_SIGS)


def call(name, *args):
    rc = getattr(lib(), name)(*args)
    if rc != NFEM_OK:
        raise NfemError(rc, name)
    return rc


def ptr(t):
    """Raw device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return C.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def require_cuda(t, what):
    if not t.is_cuda:
        raise ValueError(f"{what} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{what} must be contiguous")
