"""GetDP's LinAlg interface, backed by the GB300 library.

The functions carry the names and argument meaning of src/kernel/LinAlg.h
:90-213 as implemented for Sparskit in src/kernel/LinAlg_SPARSKIT.cpp; errors
raise :class:`GetDPError` where the reference calls Message::Error.  Objects
(``gSolver``, ``gVector``, ``gMatrix``) wrap device-resident data; scalar
adds to vectors and matrices are staged on the host in call order and merged
on the device when the object is next used, so per-entry semantics (sums of
duplicates in call order) are those of the reference.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import GetDPError, SolveInfo, SolverParams, check

_CTX = None
_SOLVER_OPTIONS: list = []
_SOLVER_FILE: Optional[str] = None


def context():
    """The process-wide context on device 0 (one GPU, one stream)."""
    global _CTX
    if _CTX is None:
        L = _lib.load()
        h = ctypes.c_void_p()
        check(L.gb300_ctx_create(0, ctypes.byref(h)))
        _CTX = h
    return _CTX


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


# ---------------------------------------------------------------- solver
class gSolver:
    """Solver_Params (contrib/Sparskit/Sparskit.h:83-103)."""

    def __init__(self):
        self.params = SolverParams()
        _lib.load().gb300_solver_params_default(ctypes.byref(self.params))

    def set(self, name: str, value) -> None:
        check(_lib.load().gb300_solver_params_set(
            ctypes.byref(self.params), name.encode(), str(value).encode()))

    def read(self, path: str) -> None:
        check(_lib.load().gb300_solver_params_read(ctypes.byref(self.params),
                                                   path.encode()))

    def __getitem__(self, field):
        return getattr(self.params, field)

    def __setitem__(self, field, value):
        setattr(self.params, field, value)


def LinAlg_InitializeSolver(argv: Sequence[str]) -> None:
    """Collect ``-solver file`` and ``-Name value`` options
    (LinAlg_SPARSKIT.cpp:29-66)."""
    global _SOLVER_FILE
    _SOLVER_OPTIONS.clear()
    i = 1
    while i < len(argv):
        a = argv[i]
        if a.startswith("-"):
            if a[1:] in ("solver", "s"):
                i += 1
                if i < len(argv) and not argv[i].startswith("-"):
                    _SOLVER_FILE = argv[i]
                    i += 1
                else:
                    raise GetDPError(1, "Missing file name")
            else:
                i += 1
                if i < len(argv) and not argv[i].startswith("-"):
                    _SOLVER_OPTIONS.append((a[1:], argv[i]))
                    i += 1
                else:
                    raise GetDPError(1, "Missing number")
        else:
            i += 1


def LinAlg_CreateSolver(SolverDataFileName: Optional[str] = None,
                        path: str = "") -> gSolver:
    """Defaults, then the parameter file, then command-line overrides
    (LinAlg_SPARSKIT.cpp:72-113).  A missing file keeps the defaults (the
    reference would prompt for values interactively)."""
    S = gSolver()
    name = SolverDataFileName or _SOLVER_FILE or os.path.join(path, "solver.par")
    if name and os.path.exists(name):
        S.read(name)
    for k, v in _SOLVER_OPTIONS:
        S.set(k, v)
    return S


# ---------------------------------------------------------------- vectors
class gVector:
    def __init__(self, n: int):
        L = _lib.load()
        self.n = int(n)
        self.h = ctypes.c_void_p()
        check(L.gb300_vector_create(context(), self.n, ctypes.byref(self.h)))
        self._idx: list = []
        self._val: list = []

    def _flush(self):
        if self._idx:
            idx = np.ascontiguousarray(self._idx, np.int32)
            val = np.ascontiguousarray(self._val, np.float64)
            self._idx, self._val = [], []
            check(_lib.load().gb300_vector_add_values(self.h, len(idx), _ptr(idx), _ptr(val)))

    def set(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, np.float64)
        if a.shape != (self.n,):
            raise GetDPError(1, f"vector of size {self.n} expected")
        self._idx, self._val = [], []
        check(_lib.load().gb300_vector_set(self.h, _ptr(a)))

    def numpy(self) -> np.ndarray:
        self._flush()
        out = np.empty(self.n, np.float64)
        check(_lib.load().gb300_vector_get(self.h, _ptr(out)))
        return out

    def destroy(self):
        if self.h:
            _lib.load().gb300_vector_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def LinAlg_CreateVector(Solver: Optional[gSolver], n: int) -> gVector:
    return gVector(n)


def LinAlg_DestroyVector(V: gVector) -> None:
    V.destroy()


def LinAlg_ZeroVector(V: gVector) -> None:
    V._idx, V._val = [], []
    check(_lib.load().gb300_vector_zero(V.h))


def LinAlg_SetVector(V: gVector, v: float) -> None:
    V.set(np.full(V.n, float(v)))


def LinAlg_CopyVector(V1: gVector, V2: gVector) -> None:
    V2.set(V1.numpy())


def LinAlg_AddDoubleInVector(d: float, V: gVector, i: int) -> None:
    V._idx.append(i)
    V._val.append(d)


LinAlg_AddScalarInVector = LinAlg_AddDoubleInVector


def LinAlg_AddComplexInVector(d1: float, d2: float, V: gVector, i: int, j: int) -> None:
    V._idx += [i, j]
    V._val += [d1, d2]


def LinAlg_GetDoubleInVector(V: gVector, i: int) -> float:
    return float(V.numpy()[i])


def LinAlg_GetVectorSize(V: gVector) -> int:
    return V.n


def LinAlg_SubVectorVector(V1: gVector, V2: gVector, V3: gVector) -> None:
    """V3 = V1 - V2 with V3 one of V1, V2 (sub_vector_vector_1/2)."""
    if V3 is not V1 and V3 is not V2:
        raise GetDPError(1, "Wrong arguments in 'LinAlg_SubVectorVector'")
    V3.set(V1.numpy() - V2.numpy())


def LinAlg_VectorNorm2(V: gVector) -> float:
    V._flush()
    out = ctypes.c_double()
    check(_lib.load().gb300_vector_norm2(V.h, ctypes.byref(out)))
    return out.value


def LinAlg_AssembleVector(V: gVector) -> None:
    V._flush()


# --------------------------------------------------------------- matrices
class gMatrix:
    def __init__(self, n: int):
        L = _lib.load()
        self.n = int(n)
        self.h = ctypes.c_void_p()
        check(L.gb300_matrix_create(context(), self.n, ctypes.byref(self.h)))

    def nnz(self) -> int:
        v = ctypes.c_longlong()
        check(_lib.load().gb300_matrix_nnz(self.h, ctypes.byref(v)))
        return v.value

    def assemble(self) -> None:
        check(_lib.load().gb300_matrix_assemble(self.h))

    def csr(self):
        """(indptr, indices, data) of the assembled matrix, on the host."""
        self.assemble()
        nnz = self.nnz()
        ip = np.empty(self.n + 1, np.int32)
        ix = np.empty(max(nnz, 1), np.int32)
        dv = np.empty(max(nnz, 1), np.float64)
        check(_lib.load().gb300_matrix_get_csr(self.h, _ptr(ip), _ptr(ix), _ptr(dv)))
        return ip, ix[:nnz], dv[:nnz]

    def set_csr(self, indptr, indices, data) -> None:
        ip = np.ascontiguousarray(indptr, np.int32)
        ix = np.ascontiguousarray(indices, np.int32)
        dv = np.ascontiguousarray(data, np.float64)
        check(_lib.load().gb300_matrix_set_csr(self.h, len(dv), _ptr(ip), _ptr(ix), _ptr(dv)))

    def set_aggregates(self, agg, n_agg: Optional[int] = None) -> None:
        """Aggregates of the unknowns for the two-level preconditioners
        (Preconditioner 21, 22): agg[i] in 0 .. n_agg - 1 for every row."""
        a = np.ascontiguousarray(agg, np.int32)
        if n_agg is None:
            n_agg = int(a.max()) + 1 if len(a) else 0
        check(_lib.load().gb300_matrix_set_aggregates(self.h, _ptr(a), int(n_agg)))

    def aggregate_graph(self, n_agg: int = 1024) -> None:
        """Aggregates from the matrix graph alone (no mesh needed)."""
        check(_lib.load().gb300_matrix_aggregate_graph(self.h, int(n_agg)))

    def add_coo(self, i, j, v) -> None:
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        v = np.ascontiguousarray(v, np.float64)
        check(_lib.load().gb300_matrix_add_coo(self.h, len(v), _ptr(i), _ptr(j), _ptr(v)))

    def destroy(self):
        if self.h:
            _lib.load().gb300_matrix_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def LinAlg_CreateMatrix(Solver: Optional[gSolver], n: int, m: Optional[int] = None) -> gMatrix:
    return gMatrix(n)


def LinAlg_DestroyMatrix(M: gMatrix) -> None:
    M.destroy()


def LinAlg_ZeroMatrix(M: gMatrix) -> None:
    check(_lib.load().gb300_matrix_zero(M.h))


def LinAlg_AddDoubleInMatrix(d: float, M: gMatrix, i: int, j: int) -> None:
    check(_lib.load().gb300_matrix_add_double(M.h, float(d), int(i), int(j)))


LinAlg_AddScalarInMatrix = LinAlg_AddDoubleInMatrix


def LinAlg_AddComplexInMatrix(d1: float, d2: float, M: gMatrix, i: int, j: int,
                              k: int, l: int) -> None:
    check(_lib.load().gb300_matrix_add_complex(M.h, float(d1), float(d2), i, j, k, l))


def LinAlg_AssembleMatrix(M: gMatrix) -> None:
    M.assemble()


def LinAlg_GetMatrixSize(M: gMatrix):
    return M.n, M.n


def LinAlg_ProdMatrixVector(M: gMatrix, V1: gVector, V2: gVector) -> None:
    if V1 is V2:
        raise GetDPError(1, "Wrong arguments in 'LinAlg_ProdMatrixVector'")
    V1._flush()
    check(_lib.load().gb300_matrix_mult(M.h, V1.h, V2.h))


# ----------------------------------------------------------------- solve
def LinAlg_Solve(A: gMatrix, B: gVector, Solver: gSolver, X: gVector,
                 solverIndex: int = 0) -> dict:
    """solve_matrix (Sparskit.cpp:108-634) on the GPU; returns the solve
    information (status, iterations, residuals)."""
    B._flush()
    info = SolveInfo()
    rc = _lib.load().gb300_solve(A.h, B.h, ctypes.byref(Solver.params), X.h,
                                 ctypes.byref(info))
    if rc != 0 and rc != 4:
        check(rc)
    d = info.as_dict()
    if rc == 4:  # the reference only warns when the iteration fails
        d["warning"] = _lib.load().gb300_last_error().decode()
    return d


def LinAlg_SolveBatch(A: gMatrix, B: gVector, Solver: gSolver, X: gVector,
                      offsets) -> list:
    """LinAlg_Solve over independent systems held as A's diagonal blocks
    (system k: rows offsets[k]..offsets[k+1]); one information dict per
    system.  A system that fails only warns, as LinAlg_Solve does."""
    B._flush()
    off = np.ascontiguousarray(offsets, np.int32)
    nsys = len(off) - 1
    infos = (SolveInfo * max(nsys, 1))()
    rc = _lib.load().gb300_solve_batch(
        A.h, B.h, ctypes.byref(Solver.params), X.h, nsys,
        off.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), infos)
    if rc != 0 and rc != 4:
        check(rc)
    out = [infos[k].as_dict() for k in range(nsys)]
    if rc == 4:
        msg = _lib.load().gb300_last_error().decode()
        for d in out:
            if d["status"] != 0:
                d["warning"] = msg
    return out


def LinAlg_SolveAgain(A: gMatrix, B: gVector, Solver: gSolver, X: gVector,
                      solverIndex: int = 0) -> dict:
    """LinAlg_Solve reusing the previous solve's ILU(0) factorisation of A
    (Re_Use_LU set for this call, LinAlg_SPARSKIT.cpp:578-585)."""
    keep = Solver["re_use_lu"]
    Solver["re_use_lu"] = 1
    try:
        return LinAlg_Solve(A, B, Solver, X, solverIndex)
    finally:
        Solver["re_use_lu"] = keep
