"""Learned correction of the ILU(0) preconditioner (Preconditioner 20).

The network (getdp_gb300/csrc/learned.cu, 3 message-passing layers of
width 32 over the matrix graph, BF16 weights) predicts a sparse matrix G on
A's pattern; the preconditioner is z = ILU^-1 v, z += G (v - A z).  It is
trained on the GPU with its own forward and backward kernels and Adam, on
systems assembled by Generate and solutions from the plain solver: for
each, z1 = ILU^-1 b, r1 = b - A z1, e1 = x* - z1, and the loss is
||G r1 - e1||^2 / ||e1||^2.  solve() runs FGMRES with the correction and
falls back to the plain ILU(0)-GMRES when that does not converge or takes
more steps than the cap allows; the FP64 residual decides either way.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np

from . import _lib
from . import linalg as LA
from ._lib import check


class MPNN:
    def __init__(self, seed: int = 1):
        L = _lib.load()
        self.L = L
        self.h = ctypes.c_void_p()
        check(L.gb300_mpnn_create(LA.context(), seed, ctypes.byref(self.h)))
        self.n_params = L.gb300_mpnn_param_count()

    def __del__(self):
        try:
            if self.h:
                self.L.gb300_mpnn_destroy(self.h)
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        check(self.L.gb300_mpnn_get_params(self.h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_params(self, w) -> None:
        w = np.ascontiguousarray(w, np.float32)
        check(self.L.gb300_mpnn_set_params(self.h, w.ctypes.data_as(ctypes.c_void_p)))

    def infer(self, A: LA.gMatrix) -> None:
        """Predict G for A and attach it as A's correction."""
        A.assemble()
        check(self.L.gb300_mpnn_infer(self.h, A.h))

    def loss_grad(self, A: LA.gMatrix, r1: LA.gVector, e1,
                  accumulate: bool = False, want_grad: bool = False):
        loss = ctypes.c_double()
        g = np.zeros(self.n_params, np.float32) if want_grad else None
        check(self.L.gb300_mpnn_loss_grad(
            self.h, A.h, r1.h, e1.h if e1 is not None else None, int(accumulate),
            ctypes.byref(loss),
            g.ctypes.data_as(ctypes.c_void_p) if want_grad else None))
        return loss.value, g

    def adam_step(self, lr: float, grad_scale: float = 1.0) -> None:
        check(self.L.gb300_mpnn_adam_step(self.h, ctypes.c_float(lr),
                                          ctypes.c_float(grad_scale)))


def ilu_params(renumbering: int = 1) -> LA.gSolver:
    S = LA.LinAlg_CreateSolver(None)
    S.set("Preconditioner", 6)
    S.set("Renumbering_Technique", renumbering)
    return S


@dataclasses.dataclass
class Sample:
    A: LA.gMatrix
    b: LA.gVector
    r1: LA.gVector
    e1: object  # gVector, or None for a probe without solution


def make_sample(A: LA.gMatrix, b: LA.gVector, x_star: LA.gVector,
                renumbering: int = 1) -> Sample:
    """Training targets for one system: z1 = ILU^-1 b, r1 = b - A z1,
    e1 = x* - z1 (all on the GPU)."""
    L = _lib.load()
    n = A.n
    z1 = LA.gVector(n)
    r1 = LA.gVector(n)
    e1 = LA.gVector(n)
    b._flush()
    x_star._flush()
    check(L.gb300_precond_apply(A.h, ctypes.byref(ilu_params(renumbering).params), b.h, z1.h))
    check(L.gb300_matrix_mult(A.h, z1.h, r1.h))          # r1 = A z1
    check(L.gb300_vector_axpby(1.0, b.h, -1.0, r1.h))     # r1 = b - A z1
    check(L.gb300_vector_axpby(1.0, x_star.h, 0.0, e1.h))
    check(L.gb300_vector_axpby(-1.0, z1.h, 1.0, e1.h))    # e1 = x* - z1
    return Sample(A, b, r1, e1)


def make_probes(A: LA.gMatrix, count: int, seed: int, renumbering: int = 1) -> list:
    """Random probes v (no solution needed): r1 = v - A ILU^-1 v, with
    ILU^-1 r1 standing in for A^-1 r1 in the loss's normalisation."""
    L = _lib.load()
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        v = LA.gVector(A.n)
        v.set(rng.standard_normal(A.n))
        v._flush()
        z1 = LA.gVector(A.n)
        r1 = LA.gVector(A.n)
        check(L.gb300_precond_apply(A.h, ctypes.byref(ilu_params(renumbering).params),
                                    v.h, z1.h))
        check(L.gb300_matrix_mult(A.h, z1.h, r1.h))
        check(L.gb300_vector_axpby(1.0, v.h, -1.0, r1.h))
        e1 = LA.gVector(A.n)
        check(L.gb300_precond_apply(A.h, ctypes.byref(ilu_params(renumbering).params),
                                    r1.h, e1.h))
        out.append(Sample(A, v, r1, e1))
    return out


def train(net: MPNN, samples: list, epochs: int = 20, lr: float = 3e-3,
          batch: int = 8, seed: int = 0) -> list:
    """Adam on mini-batches of systems; returns the mean loss per epoch."""
    rng = np.random.default_rng(seed)
    hist = []
    for _ in range(epochs):
        order = rng.permutation(len(samples))
        tot = 0.0
        for s0 in range(0, len(order), batch):
            idx = order[s0:s0 + batch]
            for k, i in enumerate(idx):
                s = samples[i]
                loss, _ = net.loss_grad(s.A, s.r1, s.e1, accumulate=k > 0)
                tot += loss
            net.adam_step(lr, 1.0 / len(idx))
        hist.append(tot / len(samples))
    return hist


def solve(A: LA.gMatrix, b: LA.gVector, x: LA.gVector, net: MPNN,
          stopping_test: float = 1e-8, krylov: int = 50, nb_iter_max: int = 20000,
          renumbering: int = 1, precision: int = 0, cap: int = None) -> dict:
    """FGMRES with the learned correction; the plain ILU(0)-GMRES if that
    stagnates (no convergence within `cap` steps)."""
    net.infer(A)
    S = LA.LinAlg_CreateSolver(None)
    for k, v in dict(Algorithm=9, Preconditioner=20, Krylov_Size=krylov,
                     Nb_Iter_Max=cap or nb_iter_max, Renumbering_Technique=renumbering,
                     Precision=precision).items():
        S.set(k, v)
    S["stopping_test"] = stopping_test
    info = LA.LinAlg_Solve(A, b, S, x)
    info["preconditioner"] = "learned"
    if info["status"] == 0:
        return info
    P = LA.LinAlg_CreateSolver(None)
    for k, v in dict(Algorithm=8, Preconditioner=6, Krylov_Size=krylov,
                     Nb_Iter_Max=nb_iter_max, Renumbering_Technique=renumbering,
                     Precision=precision).items():
        P.set(k, v)
    P["stopping_test"] = stopping_test
    plain = LA.LinAlg_Solve(A, b, P, x)
    plain["preconditioner"] = "ilu0 (fallback)"
    plain["learned_attempt_iterations"] = info["iterations"]
    return plain
