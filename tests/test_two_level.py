"""Two-level preconditioning on aggregates (Preconditioners 21 and 22).

No counterpart in the reference: Sparskit's preconditioners are one-level.
What is checked:
* one application of the cycle z = S v; z += P0 Ac^-1 P0^T (v - A z);
  z += S (v - A z) against the same cycle written out in numpy (Ac = P0^T A
  P0 inverted by numpy in FP64) around the GPU's own ILU(0) applications, in
  GetDP's order and in the multicolour order;
* the solution of GMRES/FGMRES with it against the oracle's solution
  (Sparskit's ILU(0)-GMRES) at Stopping_Test 1e-14, and the step counts
  against the plain ILU(0) solve on the same system;
* repeated solves give bit-identical solutions (the coarse matrix is summed
  in fixed point);
* invalid aggregates and a coarse matrix that is not positive definite are
  errors, not faults.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from getdp_gb300 import _lib
from getdp_gb300 import generate as G
from getdp_gb300 import linalg as LA
from getdp_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _system(n, seed=5, state_scale=None):
    """The nonlinear 2D magnetostatics system at a = 0, or at a saturating
    state (state_scale times a fixed smooth field)."""
    p = W.nonlinear_2d(n=n, seed=seed)
    dm = W.dofmap_for(p)
    terms = G.DeviceTerms(p, dm)
    A = LA.gMatrix(dm.n_dof)
    b = LA.gVector(dm.n_dof)
    sol = None
    if state_scale is not None:
        node_of = np.full(dm.n_dof, 0)
        m = dm.elem_dofs >= 0
        node_of[dm.elem_dofs[m]] = p.mesh.elems[m]
        c = p.mesh.nodes[node_of]
        s = state_scale * np.sin(np.pi * c[:, 0]) * np.sin(np.pi * c[:, 1])
        sol = LA.gVector(dm.n_dof)
        sol.set(s)
    G.generate(A, b, terms.batch, pattern=True, solution=sol)
    return p, dm, A, b, terms


def _params(prec, renumbering=1, algorithm=8, precision=0, stop=1e-10, maxit=20000):
    S = LA.LinAlg_CreateSolver(None)
    for k, v in dict(Algorithm=algorithm, Preconditioner=prec, Krylov_Size=50,
                     Nb_Iter_Max=maxit, Renumbering_Technique=renumbering,
                     Precision=precision).items():
        S.set(k, v)
    S["stopping_test"] = stop
    return S


def _apply(A, S, v):
    L = _lib.load()
    vv = LA.gVector(A.n)
    vv.set(v)
    z = LA.gVector(A.n)
    _lib.check(L.gb300_precond_apply(A.h, ctypes.byref(S.params), vv.h, z.h))
    return z.numpy()


@pytest.mark.parametrize("renumbering", [0, 1])
def test_cycle_matches_its_definition(renumbering):
    p, dm, A, b, _ = _system(40, state_scale=0.02)
    agg, nc = W.cell_aggregates(p, dm, 6)
    A.set_aggregates(agg, nc)
    ip, ix, dv = A.csr()
    Am = sp.csr_matrix((dv, ix, ip), shape=(A.n, A.n))
    P = sp.csr_matrix((np.ones(A.n), (np.arange(A.n), agg)), shape=(A.n, nc))
    Ac = (P.T @ Am @ P).toarray()
    Aci = np.linalg.inv(Ac)
    S6 = _params(6, renumbering)
    v = np.random.default_rng(1).standard_normal(A.n)
    z = _apply(A, S6, v)
    z = z + P @ (Aci @ (P.T @ (v - Am @ z)))
    z = z + _apply(A, S6, v - Am @ z)
    got = _apply(A, _params(21, renumbering), v)
    err = np.linalg.norm(got - z) / np.linalg.norm(z)
    # Ac is summed in fixed point (each term within 2^-40 of max|a|) and
    # inverted without pivoting: ~cond(Ac) x 1e-15
    assert err < 1e-9, err


def _solve(A, b, S):
    x = LA.gVector(A.n)
    info = LA.LinAlg_Solve(A, b, S, x)
    return x.numpy(), info


def test_solution_matches_the_oracle_and_takes_fewer_steps():
    p, dm, A, b, _ = _system(128, state_scale=0.02)
    agg, nc = W.cell_aggregates(p, dm, 8)
    A.set_aggregates(agg, nc)
    ip, ix, dv = A.csr()
    bh = b.numpy()
    xo, st, its_o, _ = oracle.solve(ip, ix, dv, bh, algorithm=8, preconditioner=6,
                                    renumbering=0, krylov_size=50, nb_iter_max=20000,
                                    stopping_test=1e-14)
    assert st == 0
    x2, i2 = _solve(A, b, _params(21, 1, stop=1e-14))
    x1, i1 = _solve(A, b, _params(6, 1, stop=1e-14))
    assert i2["status"] == 0 and i1["status"] == 0
    err = np.linalg.norm(x2 - xo) / np.linalg.norm(xo)
    print(f"two-level {i2['iterations']} steps, ILU(0) {i1['iterations']}, "
          f"oracle {its_o}; difference {err:.2e}")
    assert err < 1e-10, err
    assert i2["iterations"] * 3 < i1["iterations"]


def test_mixed_precision_fgmres_with_the_cycle():
    # FGMRES (FP64 basis) with the FP32 ILU(0) inside the cycle, to 1e-10
    p, dm, A, b, _ = _system(128, state_scale=0.02)
    agg, nc = W.cell_aggregates(p, dm, 8)
    A.set_aggregates(agg, nc)
    x2, i2 = _solve(A, b, _params(21, 1, 9, 1))
    x1, i1 = _solve(A, b, _params(6, 1, 9, 1))
    assert i2["status"] == 0 and i1["status"] == 0
    assert i2["true_residual"] <= 1.05e-10 * i2["rhs_norm"]
    print(f"mixed two-level {i2['iterations']} steps, ILU(0) {i1['iterations']}")
    assert i2["iterations"] * 3 < i1["iterations"]


def test_repeated_solves_are_bit_identical():
    p, dm, A, b, _ = _system(96, state_scale=0.02)
    agg, nc = W.cell_aggregates(p, dm, 12)
    A.set_aggregates(agg, nc)
    S = _params(21, 1, 9, 1)
    xa, ia = _solve(A, b, S)
    xb, ib = _solve(A, b, S)
    assert ia["iterations"] == ib["iterations"]
    assert np.array_equal(xa, xb)


def test_reuse_keeps_the_coarse_inverse():
    p, dm, A, b, _ = _system(64)
    agg, nc = W.cell_aggregates(p, dm, 8)
    A.set_aggregates(agg, nc)
    S = _params(21, 1)
    x1, i1 = _solve(A, b, S)
    S["re_use_lu"] = 1
    x2, i2 = _solve(A, b, S)
    assert i2["ilu_factorized"] == 0
    assert i1["iterations"] == i2["iterations"] and np.array_equal(x1, x2)


def test_invalid_aggregates_are_errors():
    p, dm, A, b, _ = _system(16)
    n = A.n
    with pytest.raises(LA.GetDPError, match="outside"):
        A.set_aggregates(np.full(n, 3), 2)
    with pytest.raises(LA.GetDPError, match="has no row"):
        A.set_aggregates(np.zeros(n), 2)
    with pytest.raises(LA.GetDPError, match="supported"):
        A.set_aggregates(np.arange(n) % 3000, 3000)
    with pytest.raises(LA.GetDPError, match="supported"):
        A.aggregate_graph(0)


def test_indefinite_coarse_matrix_is_an_error():
    # -Laplacian: symmetric negative definite, so the first coarse pivot is < 0
    m = 30
    T = sp.diags([-1.0, 2.0, -1.0], [-1, 0, 1], shape=(m, m))
    K = -(sp.kron(T, sp.identity(m)) + sp.kron(sp.identity(m), T)).tocsr()
    K.sort_indices()
    A = LA.gMatrix(m * m)
    A.set_csr(K.indptr, K.indices, K.data)
    A.set_aggregates(np.arange(m * m) // 90, 10)
    b = LA.gVector(m * m)
    b.set(np.ones(m * m))
    x = LA.gVector(m * m)
    with pytest.raises(LA.GetDPError, match="not positive definite"):
        LA.LinAlg_Solve(A, b, _params(21, 0), x)


def test_zero_correction_gives_the_plain_cycle():
    # Preconditioner 22 with G = 0 is Preconditioner 21, step for step
    p, dm, A, b, _ = _system(64, state_scale=0.02)
    agg, nc = W.cell_aggregates(p, dm, 8)
    A.set_aggregates(agg, nc)
    nnz = A.nnz()
    _lib.check(_lib.load().gb300_matrix_set_correction(
        A.h, np.zeros(nnz).ctypes.data_as(ctypes.c_void_p), 0))
    for prec in (0, 1):
        x21, i21 = _solve(A, b, _params(21, 1, 9, prec))
        x22, i22 = _solve(A, b, _params(22, 1, 9, prec))
        assert i21["status"] == 0 and i22["status"] == 0
        assert i21["iterations"] == i22["iterations"]
        assert np.array_equal(x21, x22)


def test_aggregates_from_the_matrix_graph():
    # GetDP's solve has no mesh at hand: Preconditioner 21 on a matrix
    # without aggregates makes them from A's graph, and they serve as well
    p, dm, A, b, _ = _system(128, state_scale=0.02)
    x1, i1 = _solve(A, b, _params(6, 1, stop=1e-12))
    x2, i2 = _solve(A, b, _params(21, 1, stop=1e-12))   # aggregates made here
    agg, nc = W.cell_aggregates(p, dm, 8)
    A.set_aggregates(agg, nc)
    x3, i3 = _solve(A, b, _params(21, 1, stop=1e-12))
    print(f"ILU(0) {i1['iterations']}, graph aggregates {i2['iterations']}, "
          f"cells {i3['iterations']}")
    assert i1["status"] == 0 and i2["status"] == 0 and i3["status"] == 0
    assert i2["iterations"] * 3 < i1["iterations"]
    assert i2["iterations"] <= 1.25 * i3["iterations"]
    assert np.linalg.norm(x2 - x1) <= 1e-7 * np.linalg.norm(x1)
    # explicit: about n / 256 rows each
    A.aggregate_graph(256)
    x4, i4 = _solve(A, b, _params(21, 1, stop=1e-12))
    assert i4["status"] == 0


def _spai1(Am):
    """G with rows argmin ||e_i - A g|| over A's pattern of row i (numpy)."""
    n = Am.shape[0]
    Ac = Am.tocsc()
    G = Am.copy().astype(np.float64).tolil()
    for i in range(n):
        J = Am.indices[Am.indptr[i]:Am.indptr[i + 1]]
        sub = Ac[:, J].toarray()
        e = np.zeros(n)
        e[i] = 1.0
        g, *_ = np.linalg.lstsq(sub, e, rcond=None)
        for j, gj in zip(J, g):
            G[i, j] = gj
    return G.tocsr()


def test_spai_cycle_matches_its_definition():
    # Preconditioner 25: the cycle smoothed by z = G v, G the SPAI-1 of A on
    # its own pattern, made on the device
    p, dm, A, b, _ = _system(24, state_scale=0.02)
    agg, nc = W.cell_aggregates(p, dm, 4)
    A.set_aggregates(agg, nc)
    ip, ix, dv = A.csr()
    Am = sp.csr_matrix((dv, ix, ip), shape=(A.n, A.n))
    Gm = _spai1(Am)
    P = sp.csr_matrix((np.ones(A.n), (np.arange(A.n), agg)), shape=(A.n, nc))
    Aci = np.linalg.inv((P.T @ Am @ P).toarray())
    v = np.random.default_rng(2).standard_normal(A.n)
    z = Gm @ v
    z = z + P @ (Aci @ (P.T @ (v - Am @ z)))
    z = z + Gm @ (v - Am @ z)
    got = _apply(A, _params(25, 0), v)
    err = np.linalg.norm(got - z) / np.linalg.norm(z)
    assert err < 1e-9, err


def test_spai_cycle_solves_to_the_oracle_solution():
    p, dm, A, b, _ = _system(128, state_scale=0.02)
    agg, nc = W.cell_aggregates(p, dm, 8)
    A.set_aggregates(agg, nc)
    ip, ix, dv = A.csr()
    xo, st, _, _ = oracle.solve(ip, ix, dv, b.numpy(), algorithm=8, preconditioner=6,
                                renumbering=0, krylov_size=50, nb_iter_max=20000,
                                stopping_test=1e-14)
    x25, i25 = _solve(A, b, _params(25, 0, stop=1e-14))
    x21, i21 = _solve(A, b, _params(21, 1, stop=1e-14))
    print(f"SPAI-1 cycle {i25['iterations']} steps, ILU(0) cycle {i21['iterations']}")
    assert i25["status"] == 0
    assert np.linalg.norm(x25 - xo) <= 1e-10 * np.linalg.norm(xo)
