"""Parity at the full sizes of the benchmark configurations.

The golden fixtures pin the GPU path against the reference itself on small
meshes; these tests pin it against the oracle (the reference's element loop
and Sparskit solves restated, bit-exact against the reference on every
golden fixture) at the sizes the measurements use:

* Generate (pattern bit-exact; values and RHS within the per-entry bound of
  tests/tolerances.py: 1e-12 relative, or 1e-13 of the Jacobi-scaled matrix):
  - 2D P1 magnetostatics, 256^2 cells (131,072 triangles);
  - 3D P2 elasticity, 48^3 x 6 tets (663,552 tets, 228,911,580 nonzeros);
  - 3D Whitney-edge curl-curl, 40^3 x 6 tets (384,000 tets);
  - 2D nonlinear magnetostatics, 1024^2 cells (2,097,152 triangles), at
    a = 0 and at a state where the saturating law is far from linear
    (|b| up to ~2 T).
* Solve:
  - magnetostatics 256^2, ILU(0)-GMRES(50) in GetDP's order at
    Stopping_Test 1e-14: solution within 1e-10 of the oracle's;
  - curl-curl 40^3, ILU(0)-FGMRES(40) to 1e-8 in GetDP's order, FP64 and with
    the FP32 factor: converged, true residual at the target, step count
    within 25 % of the oracle's, solution within 1e-6 of the oracle's;
  - elasticity 48^3, Jacobi-CG: the FP64 iterate after 10 steps (status -1,
    Sparskit's partial solution) within 1e-12 of the oracle's;
  - elasticity 16^3, the mixed FP32/FP64 CG to a 1e-11 FP64 residual (the
    FP32 inner iterations stall near 1e-12 there) against the oracle's FP64
    CG solution at 1e-12: within 1e-8 (the forward error bound, condition
    number ~7e3 from the oracle's 1,178 CG steps times 1e-11, is 7e-8).
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from getdp_gb300 import generate as G_
from getdp_gb300 import linalg as LA
from getdp_gb300 import workloads as W
from tests import tolerances as TOL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from getdp_gb300 import build
    build.build()
    oracle.build()


def _gpu_generate(p, dm, solution=None):
    A = LA.gMatrix(dm.n_dof)
    b = LA.gVector(dm.n_dof)
    batch = G_.host_batch(G_.term_arrays(p, dm))
    x = None
    if solution is not None:
        x = LA.gVector(dm.n_dof)
        x.set(solution)
    G_.generate(A, b, batch, pattern=True, solution=x)
    ip, ix, dv = A.csr()
    return A, b, ip, ix, dv, b.numpy()


def _check_generate(p, dm, solution=None):
    A, b, ip, ix, dv, bb = _gpu_generate(p, dm, solution)
    oip, oix, odv, ob, sabs, babs = oracle.assemble(p, dm, solution=solution, with_abs=True)
    assert np.array_equal(ip, oip), "row pointers differ"
    assert np.array_equal(ix, oix), "column indices differ"
    scale = TOL.matrix_scale(oip, oix, odv, sabs, p.formulation == "eddy2d")
    worst, beyond = TOL.report(dv, odv, scale)
    assert TOL.values_close(dv, odv, scale), (worst, beyond)
    worst_b, _ = TOL.report(bb, ob, babs)
    if not TOL.values_close(bb, ob, babs):
        r = np.abs(bb - ob) / np.maximum(TOL.bound(ob, babs), 1e-300)
        top = np.argsort(r)[-5:]
        raise AssertionError(f"rhs worst {worst_b}: rows {top.tolist()} gpu {bb[top].tolist()} "
                             f"oracle {ob[top].tolist()} scale {np.asarray(babs)[top].tolist()}")
    print(f"{p.name}: n={dm.n_dof} nnz={len(odv)} worst/bound values {worst:.3f} "
          f"({beyond} entries beyond 1e-12 relative) rhs {worst_b:.3f}")
    return A, b, (oip, oix, odv, ob)


def test_generate_magnetostatics_256():
    p = W.magnetostatics_2d(256, seed=1)
    _check_generate(p, W.dofmap_for(p))


def test_generate_elasticity_48():
    p = W.elasticity_p2(48, seed=2)
    dm = W.dofmap_for(p)
    assert dm.n_dof == 2709792
    A, _, _ = _check_generate(p, dm)
    assert A.nnz() == 228911580


def test_generate_curlcurl_40():
    p = W.curlcurl_edge(40, seed=3)
    dm = W.dofmap_for(p)
    assert dm.n_dof == 433720
    _check_generate(p, dm)


def _saturating_state(p, dm):
    """a on the unknowns: a smooth field whose curl reaches ~2 T, where
    nu(|b|) of the saturating law varies by orders of magnitude."""
    m = p.mesh
    used = np.zeros(m.n_nodes, bool)
    used[m.elems.ravel()] = True
    fixed = np.zeros(m.n_nodes, bool)
    fixed[m.bnd.ravel()] = True
    xy = m.nodes[used & ~fixed]
    a = 0.4 * np.sin(np.pi * xy[:, 0]) * np.sin(np.pi * xy[:, 1]) * \
        (1.0 + 0.3 * np.sin(9.0 * xy[:, 0] + 5.0 * xy[:, 1]))
    assert len(a) == dm.n_dof
    return a


@pytest.mark.parametrize("state", ["zero", "saturating"])
def test_generate_nonlinear_1024(state):
    p = W.nonlinear_2d(1024, seed=5)
    dm = W.dofmap_for(p)
    x = np.zeros(dm.n_dof) if state == "zero" else _saturating_state(p, dm)
    _check_generate(p, dm, solution=x)


def _solve_gpu(A, b, par):
    S = LA.LinAlg_CreateSolver(None)
    for k, v in par.items():
        S.set(k, v)
    x = LA.gVector(A.n)
    info = LA.LinAlg_Solve(A, b, S, x)
    return x.numpy(), info


def test_solve_magnetostatics_256_matches_oracle():
    p = W.magnetostatics_2d(256, seed=1)
    dm = W.dofmap_for(p)
    A, b, (oip, oix, odv, ob) = _check_generate(p, dm)
    par = {"Algorithm": 8, "Preconditioner": 6, "Krylov_Size": 50,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-14", "Nb_Iter_Max": 20000}
    xg, info = _solve_gpu(A, b, par)
    xo, st, its, _ = oracle.solve(oip, oix, odv, ob, algorithm=8, preconditioner=6,
                                  krylov_size=50, renumbering=0, nb_iter_max=20000,
                                  stopping_test=float(np.float32(1e-14)))
    assert st == 0 and info["status"] == 0, (info, st)
    err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    print(f"magnetostatics 256^2: gpu {info['iterations']} oracle {its} steps, "
          f"solution difference {err:.2e}")
    assert err <= 1e-10, err


@pytest.mark.parametrize("precision", [0, 1])
def test_solve_curlcurl_40_matches_oracle(precision):
    p = W.curlcurl_edge(40, seed=3)
    dm = W.dofmap_for(p)
    A, b, (oip, oix, odv, ob) = _check_generate(p, dm)
    par = {"Algorithm": 9, "Preconditioner": 6, "Krylov_Size": 40,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-8", "Nb_Iter_Max": 5000,
           "Precision": precision}
    xg, info = _solve_gpu(A, b, par)
    xo, st, its, _ = oracle.solve(oip, oix, odv, ob, algorithm=9, preconditioner=6,
                                  krylov_size=40, renumbering=0, nb_iter_max=5000,
                                  stopping_test=float(np.float32(1e-8)))
    assert st == 0 and info["status"] == 0, (info, st)
    M = sp.csr_matrix((odv, oix, oip))
    bn = np.linalg.norm(ob)
    res_g = np.linalg.norm(ob - M @ xg) / bn
    res_o = np.linalg.norm(ob - M @ xo) / bn
    err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    print(f"curl-curl 40^3 precision {precision}: gpu {info['iterations']} steps "
          f"(res {res_g:.2e}), oracle {its} (res {res_o:.2e}), difference {err:.2e}")
    assert res_g <= 2e-8 and abs(info["iterations"] - its) <= 0.25 * its + 2
    assert err <= 1e-6, err


def test_cg_elasticity_48_first_steps_match_oracle():
    p = W.elasticity_p2(48, seed=2)
    dm = W.dofmap_for(p)
    A, b, (oip, oix, odv, ob) = _check_generate(p, dm)
    k = 10
    par = {"Algorithm": 1, "Preconditioner": 0, "Scaling": 1,
           "Stopping_Test": "1e-8", "Nb_Iter_Max": k, "Precision": 0}
    S = LA.LinAlg_CreateSolver(None)
    for kk, v in par.items():
        S.set(kk, v)
    x = LA.gVector(A.n)
    info = LA.LinAlg_Solve(A, b, S, x)
    xo, st, its, _ = oracle.solve(oip, oix, odv, ob, algorithm=1, preconditioner=0,
                                  scaling=1, renumbering=0, nb_iter_max=k,
                                  stopping_test=float(np.float32(1e-8)))
    assert st == -1 and info["status"] == -1 and info["iterations"] == its, (info, st, its)
    xg = x.numpy()
    err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    print(f"elasticity 48^3: {its} CG steps, iterate difference {err:.2e}")
    assert err <= 1e-12, err


def test_mixed_cg_elasticity_16_matches_oracle_fp64():
    p = W.elasticity_p2(16, seed=2)
    dm = W.dofmap_for(p)
    A, b, (oip, oix, odv, ob) = _check_generate(p, dm)
    par = {"Algorithm": 1, "Preconditioner": 0, "Scaling": 1,
           "Stopping_Test": "1e-11", "Nb_Iter_Max": 20000, "Precision": 1}
    S = LA.LinAlg_CreateSolver(None)
    for kk, v in par.items():
        S.set(kk, v)
    S["stopping_test"] = 1e-11
    x = LA.gVector(A.n)
    info = LA.LinAlg_Solve(A, b, S, x)
    xo, st, its, _ = oracle.solve(oip, oix, odv, ob, algorithm=1, preconditioner=0,
                                  scaling=1, renumbering=0, nb_iter_max=20000,
                                  stopping_test=1e-12)
    assert st == 0 and info["status"] == 0, (info, st)
    xg = x.numpy()
    err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    print(f"elasticity 16^3 mixed CG: {info['iterations']} steps "
          f"({info['refinement_steps']} FP64 updates), oracle FP64 {its}; "
          f"difference {err:.2e}")
    assert err <= 1e-8, err
