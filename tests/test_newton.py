"""Nonlinear (Newton) path: the Newton-Raphson element terms and the Newton
loop of the reference's nonlinear resolution, against fixtures of the
reference itself (tests/golden/newton_*.npz, make_nl_golden.py) and the
oracle.

Tolerances: matrix and RHS of a Generate within 1e-12 relative plus 1e-13
of the entry's rounding scale (tests/tolerances.py); the residual history within 1e-9 of res0 plus 1e-6 of
each value (the linear solves stop at 1e-13, so iterates differ by that
much, amplified by the problem's conditioning); the same number of Newton
steps; final solutions within 1e-7 relative.
"""
import os

import numpy as np
import pytest

import oracle
from getdp_gb300 import workloads as W
from tests import tolerances as TOL
from tests.golden_cases import GOLDEN

NAMES = ["newton_nl2d_n12", "newton_nl2d_n16"]


def load(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    kw = {str(k): int(v) for k, v in zip(d["gen_kw_keys"], d["gen_kw_vals"])}
    p = W.nonlinear_2d(**kw)
    assert abs(float(np.sum(p.mesh.nodes * np.arange(1, 4))) -
               float(d["node_checksum"])) < 1e-9, "mesh generator drifted"
    return d, p, W.dofmap_for(p)


def solve_kw(d):
    par = {str(k): v for k, v in zip(d["par_keys"], d["par_vals"])}
    return dict(algorithm=int(par["Algorithm"]), preconditioner=int(par["Preconditioner"]),
                krylov_size=int(par["Krylov_Size"]),
                stopping_test=float(np.float32(par["Stopping_Test"])),
                nb_iter_max=int(par["Nb_Iter_Max"]),
                renumbering=int(par["Renumbering_Technique"]))


def close_history(h, ref):
    return len(h) == len(ref) and np.all(np.abs(np.asarray(h) - ref) <=
                                         1e-9 * ref[0] + 1e-6 * np.abs(ref))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_first_generate_matches_reference(name):
    d, p, dm = load(name)
    ip, ix, dv, b, sabs, babs = oracle.assemble(p, dm, with_abs=True)
    assert np.array_equal(ip, d["indptr"]) and np.array_equal(ix, d["indices"])
    # exp() of the host's libm against the reference's build: last bits
    sabs = TOL.matrix_scale(ip, ix, dv, sabs)
    assert TOL.values_close(dv, d["data"], sabs)
    assert TOL.values_close(b, d["b"], babs)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_newton_matches_reference(name):
    d, p, dm = load(name)
    x, hist, its = oracle.newton(p, dm, tol=1e-8, iter_max=50, **solve_kw(d))
    assert close_history(hist, d["history"]), (hist, d["history"])
    assert np.linalg.norm(x - d["x"]) <= 1e-7 * np.linalg.norm(d["x"])


# ----------------------------------------------------------------- GPU
def _gpu_terms(p, dm):
    from getdp_gb300 import build
    build.build()
    from getdp_gb300 import generate as G_
    return G_.DeviceTerms(p, dm)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_generate_matches_reference_and_oracle(name):
    d, p, dm = load(name)
    terms = _gpu_terms(p, dm)
    from getdp_gb300 import generate as G_
    from getdp_gb300 import linalg as LA
    A = LA.gMatrix(dm.n_dof)
    b = LA.gVector(dm.n_dof)
    x = LA.gVector(dm.n_dof)
    G_.generate(A, b, terms.batch, pattern=True, solution=x)  # x = 0
    ip, ix, dv = A.csr()
    assert np.array_equal(ip, d["indptr"]) and np.array_equal(ix, d["indices"])
    _, _, _, _, sabs, babs = oracle.assemble(p, dm, with_abs=True)
    sabs = TOL.matrix_scale(d["indptr"], d["indices"], d["data"], sabs)
    assert TOL.values_close(dv, d["data"], sabs)
    bb = b.numpy()
    assert TOL.values_close(bb, d["b"], babs)
    # at a field deep in the nonlinear range: the reference's final solution
    x.set(d["x"])
    G_.generate(A, b, terms.batch, pattern=False, solution=x)
    oip, oix, odv, ob, sabs, babs = oracle.assemble(p, dm, solution=d["x"], with_abs=True)
    ip, ix, dv = A.csr()
    sabs = TOL.matrix_scale(oip, oix, odv, sabs)
    assert np.array_equal(ip, oip) and TOL.values_close(dv, odv, sabs)
    bb = b.numpy()
    assert TOL.values_close(bb, ob, babs)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("renumbering", [0, 1])
def test_gpu_newton_matches_reference(name, renumbering):
    d, p, dm = load(name)
    terms = _gpu_terms(p, dm)
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import nonlinear as NL
    kw = solve_kw(d)
    S = LA.LinAlg_CreateSolver(None)
    S.set("Algorithm", kw["algorithm"])
    S.set("Preconditioner", kw["preconditioner"])
    S.set("Krylov_Size", kw["krylov_size"])
    S.set("Stopping_Test", "1e-13")
    S.set("Nb_Iter_Max", kw["nb_iter_max"])
    S.set("Renumbering_Technique", renumbering)
    r = NL.newton(terms, dm.n_dof, S, tol_rel=1e-8, iter_max=50)
    assert r.converged
    assert close_history(r.history, d["history"]), (r.history, d["history"])
    assert np.linalg.norm(r.x.numpy() - d["x"]) <= 1e-7 * np.linalg.norm(d["x"])


RELAX = (1.0, 0.5, 0.25, 0.125, 0.0625, 0.03125)


def test_oracle_relaxed_newton_converges():
    p = W.nonlinear_2d(n=24, seed=5)
    dm = W.dofmap_for(p)
    kw = dict(algorithm=8, preconditioner=6, renumbering=1, krylov_size=50,
              stopping_test=float(np.float32(1e-12)), nb_iter_max=5000)
    _, hist, _ = oracle.newton(p, dm, tol=1e-8, iter_max=25, relaxation=RELAX, **kw)
    assert hist[-1] / hist[0] <= 1e-8 and len(hist) <= 12


@pytest.mark.gpu
def test_gpu_relaxed_newton_matches_oracle():
    p = W.nonlinear_2d(n=24, seed=5)
    dm = W.dofmap_for(p)
    terms = _gpu_terms(p, dm)
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import nonlinear as NL
    S = LA.LinAlg_CreateSolver(None)
    for k, v in dict(Algorithm=8, Preconditioner=6, Krylov_Size=50, Nb_Iter_Max=5000,
                     Renumbering_Technique=0).items():
        S.set(k, v)
    S.set("Stopping_Test", "1e-12")
    r = NL.newton(terms, dm.n_dof, S, tol_rel=1e-8, iter_max=25, relaxation=RELAX)
    xo, hist, _ = oracle.newton(p, dm, tol=1e-8, iter_max=25, relaxation=RELAX,
                                algorithm=8, preconditioner=6, renumbering=0,
                                krylov_size=50, stopping_test=float(np.float32(1e-12)),
                                nb_iter_max=5000)
    assert r.converged
    assert close_history(r.history, hist), (r.history, hist)
    assert np.linalg.norm(r.x.numpy() - xo) <= 1e-7 * np.linalg.norm(xo)
