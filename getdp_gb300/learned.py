"""Learned correction of the ILU(0) preconditioner (Preconditioner 20).

The network (getdp_gb300/csrc/learned.cu, 3 message-passing layers of
width 32 over the matrix graph, BF16 weights) predicts a sparse matrix G on
A's pattern; the preconditioner is z = ILU^-1 v, z += G (v - A z).  It is
trained on the GPU with its own forward and backward kernels and Adam, on
systems assembled by Generate and solutions from the plain solver: for
each, z1 = ILU^-1 b, r1 = b - A z1, e1 = x* - z1, and the loss is the
energy norm of the error left, (G r1 - e1)^T A (G r1 - e1) / e1^T A e1
(random probes without a solution stand in with ILU^-1 r1 for e1).
solve() scales the correction by the energy-optimal step on random probes
(step_length), runs FGMRES with it, and falls back to the plain
ILU(0)-GMRES when the step is too small, or when FGMRES does not converge
within the cap; the FP64 residual decides either way.
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

    def set_loss(self, mode: int) -> None:
        """0: the one-level energy loss; 1: the energy left after the coarse
        correction of the two-level cycle (the matrices need aggregates)."""
        check(self.L.gb300_mpnn_set_loss(self.h, int(mode)))

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
                renumbering: int = 1, ilu: bool = True) -> Sample:
    """Training targets for one system: z1 = ILU^-1 b, r1 = b - A z1,
    e1 = x* - z1 (all on the GPU); without ilu, z1 = 0 (r1 = b, e1 = x*:
    G then stands alone, as in Preconditioner 24)."""
    L = _lib.load()
    n = A.n
    z1 = LA.gVector(n)
    r1 = LA.gVector(n)
    e1 = LA.gVector(n)
    b._flush()
    x_star._flush()
    if ilu:
        check(L.gb300_precond_apply(A.h, ctypes.byref(ilu_params(renumbering).params),
                                    b.h, z1.h))
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


def make_error_probes(A: LA.gMatrix, count: int, seed: int, renumbering: int = 1,
                      ilu: bool = True) -> list:
    """Random probes with a known solution: e0 random, b = A e0, then as
    make_sample (z1 = ILU^-1 b, r1 = b - A z1 = A e1, e1 = e0 - z1), so
    that r1 = A e1 holds exactly, as the two-level loss needs."""
    L = _lib.load()
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        e0 = LA.gVector(A.n)
        e0.set(rng.standard_normal(A.n))
        e0._flush()
        b = LA.gVector(A.n)
        check(L.gb300_matrix_mult(A.h, e0.h, b.h))
        out.append(make_sample(A, b, e0, renumbering, ilu))
    return out


def copy_matrix(A: LA.gMatrix) -> LA.gMatrix:
    """A new matrix with A's CSR (through the host): training keeps the
    Jacobians of every Newton step while the solver reuses A."""
    ip, ix, dv = A.csr()
    B = LA.gMatrix(A.n)
    B.set_csr(ip, ix, dv)
    return B


def copy_vector(v: LA.gVector) -> LA.gVector:
    w = LA.gVector(v.n)
    v._flush()
    check(_lib.load().gb300_vector_axpby(1.0, v.h, 0.0, w.h))
    return w


def step_length(A: LA.gMatrix, probes: int = 2, seed: int = 0, renumbering: int = 1,
                precision: int = 0) -> float:
    """The step along the attached correction that minimises the energy norm
    of the error left after the ILU step, averaged over random probes v:
    with z1 = ILU^-1 v, r1 = v - A z1 and g = G r1, the error after
    z1 + w g is smallest in the A-norm at w = r1.g / g.Ag (A symmetric
    positive definite).  A value <= 0 means the correction does not help."""
    L = _lib.load()
    rng = np.random.default_rng(seed)
    n = A.n
    S6 = ilu_params(renumbering)
    S6.set("Precision", precision)
    S20 = ilu_params(renumbering)
    S20.set("Preconditioner", 20)
    S20.set("Precision", precision)
    v, z1, z2, r1, ag = (LA.gVector(n) for _ in range(5))
    num = den = 0.0
    for _ in range(probes):
        v.set(rng.standard_normal(n))
        check(L.gb300_precond_apply(A.h, ctypes.byref(S6.params), v.h, z1.h))
        check(L.gb300_precond_apply(A.h, ctypes.byref(S20.params), v.h, z2.h))
        check(L.gb300_vector_axpby(-1.0, z1.h, 1.0, z2.h))    # g = z2 - z1
        check(L.gb300_matrix_mult(A.h, z1.h, r1.h))
        check(L.gb300_vector_axpby(1.0, v.h, -1.0, r1.h))     # r1 = v - A z1
        check(L.gb300_matrix_mult(A.h, z2.h, ag.h))           # A g
        g, r, a = z2.numpy(), r1.numpy(), ag.numpy()
        num += float(r @ g)
        den += float(g @ a)
    return num / den if den > 0 else 0.0


def coarse_energy(A: LA.gMatrix, u: LA.gVector) -> float:
    """u^T C u, C = P0 Ac^-1 P0^T on A's aggregates (its own values)."""
    out = ctypes.c_double()
    u._flush()
    check(_lib.load().gb300_matrix_coarse_energy(A.h, u.h, ctypes.byref(out)))
    return out.value


def step_length_two_level(A: LA.gMatrix, probes: int = 1, seed: int = 0,
                          renumbering: int = 1, precision: int = 0,
                          rhs: LA.gVector = None) -> float:
    """step_length for the correction inside the two-level cycle: the step
    w that minimises the energy of the error left after the coarse
    correction, (e1 - w g)^T (A - A C A) (e1 - w g), over the probes:
    w = (g.r1 - (Ag)^T C r1) / (g.Ag - (Ag)^T C Ag), the cross term by
    polarisation, 2 u^T C v = (u+v)^T C (u+v) - u^T C u - v^T C v (no
    solution needed: e1^T A g = r1^T g).  With rhs, the probe is the
    system's own right-hand side, whose error after the ILU(0) step is the
    one the solve meets (random probes are white noise, which a local
    correction removes far better: they overstate the step about twofold);
    otherwise `probes` random vectors.  A needs aggregates and the
    correction."""
    L = _lib.load()
    rng = np.random.default_rng(seed)
    n = A.n
    S6 = ilu_params(renumbering)
    S6.set("Precision", precision)
    S20 = ilu_params(renumbering)
    S20.set("Preconditioner", 20)
    S20.set("Precision", precision)
    S20["re_use_lu"] = 1  # the factor the first application made
    v, z1, z2, r1, ag, sm = (LA.gVector(n) for _ in range(6))
    num = den = 0.0
    for k in range(1 if rhs is not None else probes):
        if rhs is not None:
            rhs._flush()
            check(L.gb300_vector_axpby(1.0, rhs.h, 0.0, v.h))
        else:
            v.set(rng.standard_normal(n))
        S6["re_use_lu"] = 1 if k else 0  # factor A's current values once
        check(L.gb300_precond_apply(A.h, ctypes.byref(S6.params), v.h, z1.h))
        check(L.gb300_precond_apply(A.h, ctypes.byref(S20.params), v.h, z2.h))
        check(L.gb300_vector_axpby(-1.0, z1.h, 1.0, z2.h))    # g = z2 - z1
        check(L.gb300_matrix_mult(A.h, z1.h, r1.h))
        check(L.gb300_vector_axpby(1.0, v.h, -1.0, r1.h))     # r1 = v - A z1
        check(L.gb300_matrix_mult(A.h, z2.h, ag.h))           # A g
        check(L.gb300_vector_axpby(1.0, ag.h, 0.0, sm.h))
        check(L.gb300_vector_axpby(1.0, r1.h, 1.0, sm.h))     # A g + r1
        q_ag, q_r, q_s = coarse_energy(A, ag), coarse_energy(A, r1), coarse_energy(A, sm)
        g, r, a = z2.numpy(), r1.numpy(), ag.numpy()
        num += float(r @ g) - 0.5 * (q_s - q_ag - q_r)
        den += float(g @ a) - q_ag
    return num / den if den > 0 else 0.0


def train(net: MPNN, samples: list, epochs: int = 20, lr: float = 3e-3,
          batch: int = 8, seed: int = 0) -> list:
    """Adam on mini-batches of systems; returns the mean loss per epoch."""
    rng = np.random.default_rng(seed)
    hist = []
    skipped = [0]
    for _ in range(epochs):
        order = rng.permutation(len(samples))
        tot = 0.0
        ep_used = 0
        for s0 in range(0, len(order), batch):
            idx = order[s0:s0 + batch]
            used = 0
            for i in idx:
                ep_used += 1
                s = samples[i]
                try:
                    loss, _ = net.loss_grad(s.A, s.r1, s.e1, accumulate=used > 0)
                except _lib.GetDPError:
                    # a sample whose energy normalisation is not positive
                    # (zero error): nothing to learn from it
                    skipped[0] += 1
                    ep_used -= 1
                    continue
                tot += loss
                used += 1
            if used:
                net.adam_step(lr, 1.0 / used)
        hist.append(tot / max(ep_used, 1))
    net.skipped = skipped[0]
    return hist


def solve(A: LA.gMatrix, b: LA.gVector, x: LA.gVector, net: MPNN,
          stopping_test: float = 1e-8, krylov: int = 50, nb_iter_max: int = 20000,
          renumbering: int = 1, precision: int = 0, cap: int = None,
          line_search: bool = True, min_step: float = 0.05) -> dict:
    """FGMRES with the learned correction; the plain ILU(0)-GMRES if that
    stagnates (no convergence within `cap` steps).  With line_search the
    correction is first scaled by step_length(A), and not used at all when
    that step is below min_step."""
    net.infer(A)
    omega = None
    if line_search:
        omega = step_length(A, renumbering=renumbering, precision=precision)
        if omega < min_step:
            return _plain(A, b, x, stopping_test, krylov, nb_iter_max, renumbering,
                          precision, dict(learned_attempt_iterations=0, step=omega,
                                          preconditioner="ilu0 (correction rejected)"))
        check(_lib.load().gb300_matrix_scale_correction(A.h, ctypes.c_double(omega)))
    S = LA.LinAlg_CreateSolver(None)
    for k, v in dict(Algorithm=9, Preconditioner=20, Krylov_Size=krylov,
                     Nb_Iter_Max=cap or nb_iter_max, Renumbering_Technique=renumbering,
                     Precision=precision).items():
        S.set(k, v)
    S["stopping_test"] = stopping_test
    info = LA.LinAlg_Solve(A, b, S, x)
    info["preconditioner"] = "learned"
    info["step"] = omega
    if info["status"] == 0:
        return info
    return _plain(A, b, x, stopping_test, krylov, nb_iter_max, renumbering, precision,
                  dict(learned_attempt_iterations=info["iterations"], step=omega,
                       preconditioner="ilu0 (fallback)"))


def _plain(A, b, x, stopping_test, krylov, nb_iter_max, renumbering, precision, extra):
    """The method without the network: ILU(0)-GMRES, or FGMRES with the
    FP32 factor (Precision 1)."""
    P = LA.LinAlg_CreateSolver(None)
    for k, v in dict(Algorithm=8 if precision == 0 else 9, Preconditioner=6,
                     Krylov_Size=krylov, Nb_Iter_Max=nb_iter_max,
                     Renumbering_Technique=renumbering, Precision=precision).items():
        P.set(k, v)
    P["stopping_test"] = stopping_test
    plain = LA.LinAlg_Solve(A, b, P, x)
    plain.update(extra)
    return plain


class NewtonSolver:
    """The linear solve of each Newton step with the learned correction, as
    a callable for nonlinear.newton: the learned FGMRES is capped at the
    step count of the last plain solve (iterations not reduced = fallback),
    the first attempt at `first_cap`; after `max_failures` failed attempts
    the remaining steps use the plain method directly."""

    def __init__(self, net: MPNN, stopping_test: float = 1e-10, krylov: int = 50,
                 nb_iter_max: int = 20000, renumbering: int = 1, precision: int = 1,
                 first_cap: int = 2000, max_failures: int = 1):
        self.net = net
        self.kw = dict(stopping_test=stopping_test, krylov=krylov,
                       nb_iter_max=nb_iter_max, renumbering=renumbering,
                       precision=precision)
        self.first_cap = first_cap
        self.max_failures = max_failures
        self.failures = 0
        self.last_plain = None
        self.log = []

    def __call__(self, A: LA.gMatrix, b: LA.gVector, x: LA.gVector) -> dict:
        if self.failures >= self.max_failures:
            info = _plain(A, b, x, self.kw["stopping_test"], self.kw["krylov"],
                          self.kw["nb_iter_max"], self.kw["renumbering"],
                          self.kw["precision"], dict(preconditioner="ilu0 (learned off)"))
        else:
            cap = self.last_plain if self.last_plain else self.first_cap
            info = solve(A, b, x, self.net, cap=cap, **self.kw)
            if info["preconditioner"] != "learned":
                self.failures += 1
        if info["preconditioner"] != "learned":
            self.last_plain = info["iterations"]
        self.log.append({k: info.get(k) for k in ("preconditioner", "iterations",
                                                  "learned_attempt_iterations", "step")})
        return info


class TwoLevelNewtonSolver:
    """The linear solve of each Newton step with the learned correction
    inside the two-level cycle (Preconditioner 22, FGMRES), as a callable
    for nonlinear.newton.  The correction is used at the scale it was
    trained for (step 1: the training loss is the energy the cycle leaves);
    step=None scales it by step_length_two_level on the right-hand side,
    which measured 7-9 on the nonlinear Jacobians and made FGMRES fail.
    The method without the network is the same cycle with plain ILU(0)
    smoothing (Preconditioner 21): it is used when the step is below
    min_step, when the learned solve does not converge within cap_margin
    times the last plain step count, and for good after max_failures such
    attempts; the first solve runs it to set that count.  The FP64 residual decides in
    every case."""

    def __init__(self, net: MPNN, agg, n_agg: int, stopping_test: float = 1e-10,
                 krylov: int = 50, nb_iter_max: int = 20000, precision: int = 1,
                 max_failures: int = 1, min_step: float = 0.05, step: float = 1.0,
                 preconditioner: int = 22, cap_margin: float = 1.25):
        self.net = net
        self.agg = np.ascontiguousarray(agg, np.int32)
        self.n_agg = int(n_agg)
        self.stop = stopping_test
        self.krylov = krylov
        self.nb_iter_max = nb_iter_max
        self.precision = precision
        self.max_failures = max_failures
        self.min_step = min_step
        self.step = step
        # 22; 23: the correction in the first smoothing only; 24: G alone
        self.preconditioner = preconditioner
        self.cap_margin = cap_margin
        self.failures = 0
        self.last_plain = None
        self.seen = None
        self.log = []

    def _params(self, prec: int, cap: int) -> LA.gSolver:
        S = LA.LinAlg_CreateSolver(None)
        # 24 is a fixed linear operator (no FP32 factor): GMRES suffices
        alg = 8 if prec == 24 else 9
        for k, v in dict(Algorithm=alg, Preconditioner=prec, Krylov_Size=self.krylov,
                         Nb_Iter_Max=cap, Renumbering_Technique=1,
                         Precision=self.precision).items():
            S.set(k, v)
        S["stopping_test"] = self.stop
        return S

    def _plain(self, A, b, x, why: str, extra: dict) -> dict:
        info = LA.LinAlg_Solve(A, b, self._params(21, self.nb_iter_max), x)
        info["preconditioner"] = why
        info.update(extra)
        self.last_plain = info["iterations"]
        return info

    def __call__(self, A: LA.gMatrix, b: LA.gVector, x: LA.gVector) -> dict:
        if self.seen is not A:
            A.set_aggregates(self.agg, self.n_agg)
            self.seen = A
        if self.last_plain is None:
            # the first solve sets the step count the learned attempts must beat
            info = self._plain(A, b, x, "two-level ilu0 (reference count)", {})
        elif self.failures >= self.max_failures:
            info = self._plain(A, b, x, "two-level ilu0 (learned off)", {})
        else:
            self.net.infer(A)
            omega = self.step
            if omega is None and self.preconditioner != 24:
                omega = step_length_two_level(A, precision=self.precision, rhs=b)
            if omega < self.min_step:
                info = self._plain(A, b, x, "two-level ilu0 (correction rejected)",
                                   dict(step=omega, learned_attempt_iterations=0))
                self.failures += 1
            else:
                if omega != 1.0:
                    check(_lib.load().gb300_matrix_scale_correction(A.h,
                                                                    ctypes.c_double(omega)))
                # Newton's later systems take more steps than the one that
                # set the count: a quarter of margin before the attempt is
                # called stagnant
                cap = int(np.ceil(self.cap_margin * self.last_plain))
                info = LA.LinAlg_Solve(A, b, self._params(self.preconditioner, cap), x)
                info["preconditioner"] = "two-level learned"
                info["step"] = omega
                if info["status"] != 0:
                    self.failures += 1
                    info = self._plain(A, b, x, "two-level ilu0 (fallback)",
                                       dict(step=omega,
                                            learned_attempt_iterations=info["iterations"]))
        self.log.append({k: info.get(k) for k in ("preconditioner", "iterations",
                                                  "learned_attempt_iterations", "step")})
        return info
