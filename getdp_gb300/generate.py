"""The batched Generate hook: one call assembles a whole formulation.

It stands where GetDP's Treatment_FemFormulation element loop
(src/kernel/Treatment_Formulation.cpp:413-618) calls
Cal_GalerkinTermOfFemEquation for each element: the host gathers the element
tables once (element -> unknown numbers in GetDP's numbering, edge signs,
per-element coefficients) and the GPU evaluates and scatters every element
matrix.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import TermBatch, check
from .linalg import context, gMatrix, gVector
from .workloads import DofMap, Problem

TWO_PI = 6.2831853071795865  # the reference's TWO_PI (SolvingAnalyse.cpp:23)


def term_arrays(p: Problem, dm: DofMap) -> dict:
    """Host arrays of the term batch for problem p, contiguous."""
    f = p.formulation
    m = p.mesh
    a = {"nodes": np.ascontiguousarray(m.nodes, np.float64),
         "elems": np.ascontiguousarray(m.elems, np.int32),
         "elem_dofs": np.ascontiguousarray(dm.elem_dofs, np.int32),
         "coef": np.ascontiguousarray(p.coef, np.float64)}
    p0 = p1 = p2 = 0.0
    if f == "magnetostatics2d":
        kind = _lib.TERM_TRI3_MAGNETOSTATIC
        a["source"] = np.ascontiguousarray(p.source, np.float64)
    elif f == "eddy2d":
        kind = _lib.TERM_TRI3_EDDY_COMPLEX
        a["source"] = np.ascontiguousarray(p.source, np.float64)
        a["coef2"] = np.ascontiguousarray(p.params["sigma"], np.float64)
        if "omega_e" in p.params:  # a batch: each problem's own frequency
            a["coef3"] = np.ascontiguousarray(p.params["omega_e"], np.float64)
        else:
            p0 = p.params["freq"] * TWO_PI
    elif f == "elasticity":
        kind = _lib.TERM_TET10_ELASTICITY
        p0 = p.params["poisson"]
        p1 = -p.params["rho"] * p.params["g"]
    elif f == "nonlinear2d":
        kind = _lib.TERM_TRI3_MAGNETOSTATIC_NL
        a["source"] = np.ascontiguousarray(p.source, np.float64)
        p0 = p.params["k_sat"]
        p1 = p.params["b_sat2"]
    elif f == "curlcurl":
        kind = _lib.TERM_TET4_EDGE_CURLCURL
        a["elem_sign"] = np.ascontiguousarray(dm.elem_sign, np.int8)
        a["source"] = np.ascontiguousarray(p.source, np.float64).reshape(-1, 3)
        p0 = p.params["reg"]
    else:
        raise ValueError(f)
    if dm.fixed_values is not None:
        a["fixed_values"] = np.ascontiguousarray(dm.fixed_values, np.float64)
    a["_kind"] = kind
    a["_p"] = (p0, p1, p2)
    return a


def _batch(arrays: dict, ptrs: dict, on_device: int) -> TermBatch:
    t = TermBatch()
    t.kind = arrays["_kind"]
    t.n_nodes = arrays["nodes"].shape[0]
    t.n_elems = arrays["elems"].shape[0]
    for k in ("nodes", "elems", "elem_dofs", "elem_sign", "coef", "source", "coef2",
              "coef3", "fixed_values"):
        setattr(t, k, ptrs.get(k))
    fv = arrays.get("fixed_values")
    t.n_fixed = 0 if fv is None else fv.shape[0]
    t.p0, t.p1, t.p2 = arrays["_p"]
    t.on_device = on_device
    return t


class DeviceTerms:
    """The term batch of a problem, copied once into device memory (the
    element tables stay resident between Generate calls)."""

    def __init__(self, p: Problem, dm: DofMap):
        L = _lib.load()
        self.arrays = term_arrays(p, dm)
        self.ptrs = {}
        self.bytes = 0
        ctx = context()
        for k, v in self.arrays.items():
            if k.startswith("_"):
                continue
            h = ctypes.c_void_p()
            check(L.gb300_device_alloc(ctx, v.nbytes, ctypes.byref(h)))
            check(L.gb300_copy_to_device(ctx, h, ctypes.c_void_p(v.ctypes.data), v.nbytes))
            self.ptrs[k] = h.value
            self.bytes += v.nbytes
        self.batch = _batch(self.arrays, self.ptrs, 1)

    def free(self):
        L = _lib.load()
        for v in self.ptrs.values():
            L.gb300_device_free(context(), ctypes.c_void_p(v))
        self.ptrs = {}

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def host_batch(arrays: dict) -> TermBatch:
    ptrs = {k: v.ctypes.data for k, v in arrays.items() if not k.startswith("_")}
    return _batch(arrays, ptrs, 0)


def generate(A: gMatrix, b: gVector, batch: TermBatch, pattern: bool = True,
             solution: gVector = None, scatter: int = None) -> None:
    """Generate[A]: (re)build A's pattern if asked (a pattern this context
    built from the same element table is reused), zero A and b, assemble (at
    the current solution, for a formulation that depends on it).  scatter:
    one of _lib.SCATTER_* (default: the batch's own setting)."""
    L = _lib.load()
    if scatter is not None:
        batch.scatter = int(scatter)
    if pattern:
        check(L.gb300_generate_pattern(A.h, ctypes.byref(batch)))
    else:
        A.assemble()
    check(L.gb300_vector_zero(b.h))
    b._idx, b._val = [], []
    if not pattern:
        # values only: zero the existing pattern's values
        check(L.gb300_matrix_zero(A.h))
    if solution is None:
        check(L.gb300_generate_values(A.h, b.h, ctypes.byref(batch)))
    else:
        solution._flush()
        check(L.gb300_generate_values_at(A.h, b.h, ctypes.byref(batch), solution.h))


def generate_problem(p: Problem, dm: DofMap, A: gMatrix = None, b: gVector = None):
    """Convenience: assemble problem p into a new (or given) A and b."""
    if A is None:
        A = gMatrix(dm.n_dof)
    if b is None:
        b = gVector(dm.n_dof)
    arrays = term_arrays(p, dm)
    generate(A, b, host_batch(arrays))
    return A, b
