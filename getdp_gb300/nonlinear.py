"""The Newton loop of a nonlinear resolution, on the GPU end to end.

GetDP runs it from the .pro file's Operation block; for the a_z
magnetostatic templates (templates/Lib_Magnetostatics_a_phi.pro:220-240):

    InitSolution[A]; Generate[A]; Solve[A];
    Generate[A]; GetResidual[A, $res0]; $res = $res0; $iter = 0;
    While[$res > tol_abs && $res / $res0 > tol_rel && $res / $res0 <= 1 &&
          $iter < iter_max] { Solve[A]; Generate[A]; GetResidual[A, $res]; }

Generate assembles the Newton-Raphson terms at the current solution
(gb300_generate_values_at, pattern built once), Solve is LinAlg_Solve, and
GetResidual is ||b - A x||_2 (SolvingOperations.cpp:1318-1341: product,
difference, norm), formed on the GPU in one pass (gb300_residual_noalloc).
Nothing leaves the GPU but the residual norms and the solver's status.
"""
from __future__ import annotations

import dataclasses

import ctypes

from . import _lib
from . import generate as G
from . import linalg as LA


@dataclasses.dataclass
class NewtonResult:
    x: LA.gVector
    history: list          # GetResidual after each Generate (res0 first)
    solves: list           # LinAlg_Solve information of every Solve
    converged: bool


def newton(terms: G.DeviceTerms, n: int, solver, tol_rel: float = 1e-8,
           tol_abs: float = 1e-300, iter_max: int = 50, A: LA.gMatrix = None,
           b: LA.gVector = None, relaxation=(1.0,)) -> NewtonResult:
    """With several relaxation factors the step dx of each Solve is relaxed
    as SolveJac_AdaptRelax does with CheckAll 0 (SolvingOperations.cpp:
    1593-1700): the factors are tried in order, x + f dx regenerated and its
    residual ||b - A x|| / N kept while it decreases; the best is taken.
    `solver` is a gSolver for LinAlg_Solve, or a callable (A, b, x) -> info
    dict that solves A x = b in its place (the learned preconditioner's
    solve, for one)."""
    A = A if A is not None else LA.gMatrix(n)
    b = b if b is not None else LA.gVector(n)
    x = LA.gVector(n)  # InitSolution: zero
    r = LA.gVector(n)
    x_save = LA.gVector(n) if len(relaxation) > 1 else None
    dx = LA.gVector(n) if len(relaxation) > 1 else None
    L = _lib.load()
    solves = []
    first = [True]

    def generate():
        G.generate(A, b, terms.batch, pattern=first[0], solution=x)
        first[0] = False

    def linear(x_):
        if callable(solver):
            return solver(A, b, x_)
        return LA.LinAlg_Solve(A, b, solver, x_)

    def solve():
        if x_save is None:
            solves.append(linear(x))
            generate()
            return
        _lib.check(L.gb300_vector_axpby(1.0, x.h, 0.0, x_save.h))
        solves.append(linear(x))
        _lib.check(L.gb300_vector_axpby(1.0, x.h, 0.0, dx.h))
        _lib.check(L.gb300_vector_axpby(-1.0, x_save.h, 1.0, dx.h))  # dx = x_new - x
        err_prev, f_opt = 1e99, relaxation[0]
        for k, f in enumerate(relaxation):
            _lib.check(L.gb300_vector_axpby(1.0, x_save.h, 0.0, x.h))
            _lib.check(L.gb300_vector_axpby(f, dx.h, 1.0, x.h))
            generate()
            e = residual() / n
            if e < err_prev:
                err_prev, f_opt = e, f
            elif k > 0:
                break
        if f != f_opt or e >= err_prev:  # the last trial was not the best
            _lib.check(L.gb300_vector_axpby(1.0, x_save.h, 0.0, x.h))
            _lib.check(L.gb300_vector_axpby(f_opt, dx.h, 1.0, x.h))
            generate()

    def residual():
        b._flush()
        out = ctypes.c_double()
        _lib.check(_lib.load().gb300_residual_noalloc(A.h, x.h, b.h, r.h,
                                                      ctypes.byref(out)))
        return out.value

    generate()
    solve()  # Solve, then Generate at the (relaxed) new solution
    res0 = residual()
    hist = [res0]
    res, it = res0, 0
    while (res > tol_abs and res / res0 > tol_rel and res / res0 <= 1 and
           it < iter_max):
        solve()
        res = residual()
        it += 1
        hist.append(res)
    return NewtonResult(x, hist, solves, bool(res <= tol_abs or res / res0 <= tol_rel))
