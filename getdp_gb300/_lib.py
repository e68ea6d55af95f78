"""ctypes binding of ``libgetdp_gb300.so`` (the C ABI in include/getdp_gb300.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when the shared library is missing, and every call that needs a GPU fails
with the CUDA error the library reports.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

GB300_OK = 0
ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "unsupported option",
          4: "solver did not converge", 5: "zero pivot in ILU",
          6: "capacity exceeded", 7: "zero row in matrix"}

TERM_TRI3_MAGNETOSTATIC = 1
TERM_TRI3_EDDY_COMPLEX = 2
TERM_TET10_ELASTICITY = 3
TERM_TET4_EDGE_CURLCURL = 4
TERM_TRI3_MAGNETOSTATIC_NL = 5


class GetDPError(RuntimeError):
    """An error reported by the backend (GetDP's Message::Error)."""

    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class SolverParams(ctypes.Structure):
    _fields_ = [
        ("matrix_format", ctypes.c_int), ("matrix_printing", ctypes.c_int),
        ("matrix_storage", ctypes.c_int), ("scaling", ctypes.c_int),
        ("renumbering_technique", ctypes.c_int), ("preconditioner", ctypes.c_int),
        ("preconditioner_position", ctypes.c_int), ("nb_fill", ctypes.c_int),
        ("permutation_tolerance", ctypes.c_double),
        ("dropping_tolerance", ctypes.c_double),
        ("diagonal_compensation", ctypes.c_double), ("re_use_ilu", ctypes.c_int),
        ("algorithm", ctypes.c_int), ("krylov_size", ctypes.c_int),
        ("ic_acceleration", ctypes.c_double), ("re_use_lu", ctypes.c_int),
        ("iterative_improvement", ctypes.c_int), ("nb_iter_max", ctypes.c_int),
        ("stopping_test", ctypes.c_double), ("precision", ctypes.c_int),
        ("inner_tolerance", ctypes.c_double), ("inner_iter_max", ctypes.c_int),
        ("batch_kernel", ctypes.c_int),
    ]


class SolveInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int),
                ("residual_estimate", ctypes.c_double),
                ("true_residual", ctypes.c_double), ("rhs_norm", ctypes.c_double),
                ("refinement_steps", ctypes.c_int),
                ("inner_iterations", ctypes.c_int), ("ilu_factorized", ctypes.c_int),
                ("batch_form", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class TermBatch(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("n_nodes", ctypes.c_int),
                ("n_elems", ctypes.c_int), ("nodes", ctypes.c_void_p),
                ("elems", ctypes.c_void_p), ("elem_dofs", ctypes.c_void_p),
                ("elem_sign", ctypes.c_void_p), ("coef", ctypes.c_void_p),
                ("source", ctypes.c_void_p), ("coef2", ctypes.c_void_p),
                ("coef3", ctypes.c_void_p), ("p0", ctypes.c_double), ("p1", ctypes.c_double),
                ("p2", ctypes.c_double), ("on_device", ctypes.c_int),
                ("fixed_values", ctypes.c_void_p), ("n_fixed", ctypes.c_int),
                ("scatter", ctypes.c_int)]


# gb300_term_batch.scatter
SCATTER_DEFAULT, SCATTER_SEARCH, SCATTER_TABLE, SCATTER_COLOURED = 0, 1, 2, 3


# every symbol of include/getdp_gb300.h with (restype, argtypes)
_P, _I, _D, _LL, _SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, \
    ctypes.c_longlong, ctypes.c_size_t
_PP = ctypes.POINTER(ctypes.c_void_p)
SIGNATURES = {
    "gb300_last_error": (ctypes.c_char_p, []),
    "gb300_version": (_I, []),
    "gb300_ctx_create": (_I, [_I, _PP]),
    "gb300_ctx_destroy": (_I, [_P]),
    "gb300_ctx_synchronize": (_I, [_P]),
    "gb300_host_alloc": (_I, [_SZ, _PP]),
    "gb300_host_free": (_I, [_P]),
    "gb300_device_alloc": (_I, [_P, _SZ, _PP]),
    "gb300_device_free": (_I, [_P, _P]),
    "gb300_copy_to_device": (_I, [_P, _P, _P, _SZ]),
    "gb300_copy_to_host": (_I, [_P, _P, _P, _SZ]),
    "gb300_solver_params_default": (None, [ctypes.POINTER(SolverParams)]),
    "gb300_solver_params_set": (_I, [ctypes.POINTER(SolverParams), ctypes.c_char_p, ctypes.c_char_p]),
    "gb300_solver_params_read": (_I, [ctypes.POINTER(SolverParams), ctypes.c_char_p]),
    "gb300_vector_create": (_I, [_P, _I, _PP]),
    "gb300_vector_destroy": (_I, [_P]),
    "gb300_vector_zero": (_I, [_P]),
    "gb300_vector_set": (_I, [_P, _P]),
    "gb300_vector_get": (_I, [_P, _P]),
    "gb300_vector_size": (_I, [_P, ctypes.POINTER(_I)]),
    "gb300_vector_norm2": (_I, [_P, ctypes.POINTER(_D)]),
    "gb300_vector_axpby": (_I, [_D, _P, _D, _P]),
    "gb300_vector_add_values": (_I, [_P, _I, _P, _P]),
    "gb300_matrix_create": (_I, [_P, _I, _PP]),
    "gb300_matrix_destroy": (_I, [_P]),
    "gb300_matrix_reset": (_I, [_P]),
    "gb300_matrix_zero": (_I, [_P]),
    "gb300_matrix_add_double": (_I, [_P, _D, _I, _I]),
    "gb300_matrix_add_complex": (_I, [_P, _D, _D, _I, _I, _I, _I]),
    "gb300_matrix_add_coo": (_I, [_P, _LL, _P, _P, _P]),
    "gb300_matrix_assemble": (_I, [_P]),
    "gb300_matrix_size": (_I, [_P, ctypes.POINTER(_I)]),
    "gb300_matrix_nnz": (_I, [_P, ctypes.POINTER(_LL)]),
    "gb300_matrix_get_csr": (_I, [_P, _P, _P, _P]),
    "gb300_matrix_set_csr": (_I, [_P, _LL, _P, _P, _P]),
    "gb300_matrix_mult": (_I, [_P, _P, _P]),
    "gb300_generate_pattern": (_I, [_P, ctypes.POINTER(TermBatch)]),
    "gb300_generate_values": (_I, [_P, _P, ctypes.POINTER(TermBatch)]),
    "gb300_generate_values_at": (_I, [_P, _P, ctypes.POINTER(TermBatch), _P]),
    "gb300_solve": (_I, [_P, _P, ctypes.POINTER(SolverParams), _P, ctypes.POINTER(SolveInfo)]),
    "gb300_msh_read": (_I, [ctypes.c_char_p, _PP]),
    "gb300_msh_free": (_I, [_P]),
    "gb300_msh_nodes": (_I, [_P, ctypes.POINTER(_LL), _PP, _PP]),
    "gb300_msh_group_count": (_I, [_P, ctypes.POINTER(_I)]),
    "gb300_msh_group": (_I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_LL),
                             ctypes.POINTER(_I), ctypes.POINTER(_I), _PP, _PP, _PP]),
    "gb300_matrix_set_correction": (_I, [_P, _P, _I]),
    "gb300_matrix_set_aggregates": (_I, [_P, _P, _I]),
    "gb300_matrix_aggregate_graph": (_I, [_P, _I]),
    "gb300_matrix_coarse_energy": (_I, [_P, _P, _P]),
    "gb300_matrix_scale_correction": (_I, [_P, ctypes.c_double]),
    "gb300_precond_apply": (_I, [_P, ctypes.POINTER(SolverParams), _P, _P]),
    "gb300_mpnn_param_count": (_I, []),
    "gb300_mpnn_create": (_I, [_P, ctypes.c_uint, _PP]),
    "gb300_mpnn_destroy": (_I, [_P]),
    "gb300_mpnn_set_params": (_I, [_P, _P]),
    "gb300_mpnn_get_params": (_I, [_P, _P]),
    "gb300_mpnn_infer": (_I, [_P, _P]),
    "gb300_mpnn_loss_grad": (_I, [_P, _P, _P, _P, _I, ctypes.POINTER(_D), _P]),
    "gb300_mpnn_adam_step": (_I, [_P, ctypes.c_float, ctypes.c_float]),
    "gb300_mpnn_set_loss": (_I, [_P, _I]),
    "gb300_post_elements": (_I, [ctypes.POINTER(TermBatch), _P, _P]),
    "gb300_post_points": (_I, [ctypes.POINTER(TermBatch), _P, _I, _P, _P, _P, _P]),
    "gb300_rcmk_order": (_I, [_I, _P, _P, _P]),
    "gb300_format_dof_records": (_I, [ctypes.c_longlong, _P, _P, _P, ctypes.c_longlong,
                                      ctypes.POINTER(ctypes.c_longlong)]),
    "gb300_format_int_rows": (_I, [ctypes.c_longlong, _I, _P, ctypes.c_longlong, _P,
                                   ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]),
    "gb300_solve_batch": (_I, [_P, _P, ctypes.POINTER(SolverParams), _P, _I,
                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(SolveInfo)]),
    "gb300_event_record": (_I, [_P, _I]),
    "gb300_event_elapsed": (_I, [_P, _I, _I, ctypes.POINTER(ctypes.c_float)]),
    "gb300_bench_spmv": (_I, [_P, _I, _I, ctypes.POINTER(_D)]),
    "gb300_bench_fp64_peak": (_I, [_P, ctypes.POINTER(_D)]),
    "gb300_bench_dmma_peak": (_I, [_P, ctypes.POINTER(_D)]),
    "gb300_residual_noalloc": (_I, [_P, _P, _P, _P, ctypes.POINTER(_D)]),
}

_LIB = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load the CUDA library (raises if it is missing: no CPU fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(
                f"CUDA backend not built: {path} is missing "
                "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def check(rc: int) -> None:
    if rc != GB300_OK:
        msg = _LIB.gb300_last_error().decode(errors="replace") if _LIB else ""
        raise GetDPError(rc, msg)
