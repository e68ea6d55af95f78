"""GPU parity: the CUDA path against the reference's outputs and the oracle.

Tolerances (FP64):
* CSR pattern: identical to the reference's (bit-exact integers);
* matrix and RHS values: |gpu - ref| <= 1e-12 |ref| + 1e-13 S, S the
  entry's rounding scale sqrt(A_ii A_jj) (tests/tolerances.py: the summation
  order differs -- atomics, fused multiply-adds);
* the LinAlg add path (entries added one by one in the reference's call
  order): bit-exact;
* solutions: converged (status 0); with the reference's own tolerance the
  GPU solution is within 1e-6 relative of the oracle's and the iteration
  counts agree within 5 % + 2; with Stopping_Test 1e-14 within 1e-10.
"""
import numpy as np
import pytest

import oracle
from getdp_gb300 import generate as G_
from getdp_gb300 import linalg as LA
from getdp_gb300 import workloads as W
from tests import golden_cases as G
from tests import tolerances as TOL

pytestmark = pytest.mark.gpu

ASSEMBLY_CASES = [n for n in G.names() if not n.endswith("ilu32")]


def _abs_sums(p, dm, indptr, indices, data, solution=None):
    """The rounding scales of tests/tolerances.py for the reference matrix
    (indptr, indices, data): per entry and per RHS row (the oracle's pattern
    is the reference's: checked)."""
    oip, oix, _, _, sabs, babs = oracle.assemble(p, dm, solution=solution, with_abs=True)
    assert np.array_equal(oip, indptr) and np.array_equal(oix, indices)
    return TOL.matrix_scale(indptr, indices, data, sabs, p.formulation == "eddy2d"), babs


@pytest.fixture(scope="module", autouse=True)
def _built():
    from getdp_gb300 import build
    build.build()
    oracle.build()


@pytest.mark.parametrize("name", ASSEMBLY_CASES)
def test_generate_matches_reference(name):
    d, p, dm = G.load(name)
    A, b = G_.generate_problem(p, dm)
    ip, ix, dv = A.csr()
    assert np.array_equal(ip, d["indptr"])
    assert np.array_equal(ix, d["indices"])
    sabs, babs = _abs_sums(p, dm, d["indptr"], d["indices"], d["data"])
    assert TOL.values_close(dv, d["data"], sabs), TOL.report(dv, d["data"], sabs)
    bb = b.numpy()
    assert TOL.values_close(bb, d["b"], babs), TOL.report(bb, d["b"], babs)


@pytest.mark.parametrize("name", ASSEMBLY_CASES)
def test_linalg_add_path_bit_exact(name):
    # the reference's LinAlg_AddDoubleInMatrix sequence, entry by entry
    d, p, dm = G.load(name)
    rr, cc, vv, b = oracle.assemble_coo(p, dm)
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.add_coo(rr, cc, vv)
    LA.LinAlg_AssembleMatrix(A)
    ip, ix, dv = A.csr()
    assert np.array_equal(ip, d["indptr"])
    assert np.array_equal(ix, d["indices"])
    # the same triplets merged by the oracle on this machine: bit-exact
    oip, oix, odv, _ = oracle.assemble(p, dm)
    assert np.array_equal(dv, odv), (
        f"{np.sum(dv != odv)} entries differ, max rel "
        f"{np.max(np.abs(dv - odv) / np.maximum(np.abs(odv), 1e-300)):.2e}")
    # and the reference's values (an element value computed on another
    # architecture can differ in its last bit)
    sabs, _ = _abs_sums(p, dm, d["indptr"], d["indices"], d["data"])
    assert TOL.values_close(dv, d["data"], sabs)


def _solver(params: dict):
    S = LA.LinAlg_CreateSolver(None)
    for k, v in params.items():
        S.set(k, v)
    return S


def _golden_params(d):
    return {str(k): (v if str(k) == "Stopping_Test" else int(v))
            for k, v in zip(d["par_keys"], d["par_vals"])}


@pytest.mark.parametrize("name", ASSEMBLY_CASES)
def test_solve_matches_oracle(name):
    d, p, dm = G.load(name)
    par = _golden_params(d)
    par["Renumbering_Technique"] = 0  # the GPU keeps GetDP's DOF order
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    kw = oracle.params_from_golden(d["par_keys"], d["par_vals"])
    kw["renumbering"] = 0
    kw["stopping_test"] = float(np.float32(kw["stopping_test"]))
    xo, st, its, _ = oracle.solve(d["indptr"], d["indices"], d["data"], d["b"], **kw)
    assert st == 0 and info["status"] == 0, (info, st)
    xg = x.numpy()
    if name in ILL_CONDITIONED:
        # kappa ~ 3e11: iteration counts depend on rounding in the
        # orthogonalisation (classical Gram-Schmidt here, MGS in the
        # reference) and the
        # forward error bound kappa * tol exceeds 1, so the bar is the
        # backward error: the GPU's true residual against the oracle's (the
        # Givens estimate of FGMRES drifts from the true residual on both)
        import scipy.sparse as sp
        Am = sp.csr_matrix((d["data"], d["indices"], d["indptr"]))
        res_oracle = np.linalg.norm(d["b"] - Am @ xo)
        res_gpu = np.linalg.norm(d["b"] - Am @ xg)
        target = kw["stopping_test"] * np.linalg.norm(d["b"])
        assert abs(info["iterations"] - its) <= 0.25 * its, (info["iterations"], its)
        assert res_gpu <= 20 * max(res_oracle, target), (res_gpu, res_oracle, target)
    else:
        assert abs(info["iterations"] - its) <= 0.05 * its + 2, (info["iterations"], its)
        assert np.linalg.norm(xg - xo) <= 1e-6 * np.linalg.norm(xo)


# 2-norm condition numbers of the golden systems that are near singular
# (curl-curl with a 1e-6 mass regularisation), computed with numpy
ILL_CONDITIONED = {"cc_edge_n4": 2.87e11}


def test_fgmres_matches_oracle():
    d, p, dm = G.load("ms2d_n24")
    par = {"Algorithm": 9, "Preconditioner": 6, "Krylov_Size": 50,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-10"}
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    xo, st, its, _ = oracle.solve(d["indptr"], d["indices"], d["data"], d["b"],
                                  algorithm=9, renumbering=0, krylov_size=50,
                                  stopping_test=float(np.float32(1e-10)))
    assert st == 0 and info["status"] == 0
    assert abs(info["iterations"] - its) <= 1, (info["iterations"], its)
    assert np.linalg.norm(x.numpy() - xo) <= 1e-8 * np.linalg.norm(xo)


# (the regularised curl-curl case, kappa ~ 3e11, cannot reach 1e-14 in FP64:
# the oracle stops at its iteration cap as well)
@pytest.mark.parametrize("name", ["ms2d_n24", "el_p2_n3", "eddy_n8"])
def test_tight_solve_within_1e10(name):
    d, p, dm = G.load(name)
    par = _golden_params(d)
    par.update(Renumbering_Technique=0, Stopping_Test="1e-14", Nb_Iter_Max=20000)
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    kw = oracle.params_from_golden(d["par_keys"], d["par_vals"])
    kw.update(renumbering=0, stopping_test=float(np.float32(1e-14)), nb_iter_max=20000)
    xo, st, its, _ = oracle.solve(d["indptr"], d["indices"], d["data"], d["b"], **kw)
    assert info["status"] == 0 and st == 0, (info, st)
    # the forward error attainable in FP64 is ~ kappa * 1e-16
    bound = max(1e-10, ILL_CONDITIONED.get(name, 0.0) * 1e-15)
    assert np.linalg.norm(x.numpy() - xo) <= bound * np.linalg.norm(xo)


def test_mixed_precision_cg_reaches_1e8():
    p = W.elasticity_p2(n=4, seed=3)
    dm = W.dofmap_for(p)
    A, b = G_.generate_problem(p, dm)
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    S = _solver({"Algorithm": 1, "Preconditioner": 0, "Scaling": 1,
                 "Stopping_Test": "1e-8", "Nb_Iter_Max": 100000, "Precision": 1})
    info = LA.LinAlg_Solve(A, b, S, x)
    assert info["status"] == 0
    assert info["true_residual"] <= 1e-8 * info["rhs_norm"] * 1.0000001
    assert info["refinement_steps"] >= 1
    # same answer as the FP64 solve
    x64 = LA.LinAlg_CreateVector(None, dm.n_dof)
    S64 = _solver({"Algorithm": 1, "Preconditioner": 0, "Scaling": 1,
                   "Stopping_Test": "1e-8", "Nb_Iter_Max": 100000})
    LA.LinAlg_Solve(A, b, S64, x64)
    assert np.linalg.norm(x.numpy() - x64.numpy()) <= 1e-5 * np.linalg.norm(x64.numpy())


def test_mixed_precision_fgmres_ilu32():
    p = W.magnetostatics_2d(n=48, seed=7)
    dm = W.dofmap_for(p)
    A, b = G_.generate_problem(p, dm)
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    S = _solver({"Algorithm": 9, "Preconditioner": 6, "Krylov_Size": 50,
                 "Renumbering_Technique": 0, "Stopping_Test": "1e-10",
                 "Precision": 1})
    info = LA.LinAlg_Solve(A, b, S, x)
    assert info["status"] == 0
    assert info["true_residual"] <= 2e-10 * info["rhs_norm"]


def test_zero_rhs_gives_zero_solution():
    d, p, dm = G.load("ms2d_n8")
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    x.set(np.ones(dm.n_dof))
    info = LA.LinAlg_Solve(A, b, _solver({"Algorithm": 8, "Preconditioner": 6,
                                          "Renumbering_Technique": 0}), x)
    assert info["status"] == 0
    assert not np.any(x.numpy())


def test_zero_pivot_is_reported():
    A = LA.LinAlg_CreateMatrix(None, 2)
    A.set_csr([0, 2, 4], [0, 1, 0, 1], [0.0, 1.0, 1.0, 1.0])
    b = LA.LinAlg_CreateVector(None, 2)
    b.set(np.ones(2))
    x = LA.LinAlg_CreateVector(None, 2)
    with pytest.raises(LA.GetDPError) as e:
        LA.LinAlg_Solve(A, b, _solver({"Algorithm": 8, "Preconditioner": 6,
                                       "Renumbering_Technique": 0}), x)
    assert e.value.code == 5 and "Zero pivot on line 1" in str(e.value)


def test_zero_row_is_reported():
    A = LA.LinAlg_CreateMatrix(None, 3)
    A.set_csr([0, 1, 1, 2], [0, 2], [1.0, 1.0])
    b = LA.LinAlg_CreateVector(None, 3)
    x = LA.LinAlg_CreateVector(None, 3)
    with pytest.raises(LA.GetDPError) as e:
        LA.LinAlg_Solve(A, b, _solver({"Algorithm": 8}), x)
    assert e.value.code == 7


def test_iteration_cap_is_a_warning():
    d, p, dm = G.load("el_p2_n3")
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver({"Algorithm": 1, "Preconditioner": 0,
                                          "Scaling": 1, "Nb_Iter_Max": 10}), x)
    assert info["status"] == -1 and info["iterations"] == 10 and "warning" in info


def test_missing_pattern_entry_is_an_error():
    p = W.magnetostatics_2d(n=4, seed=1)
    dm = W.dofmap_for(p)
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    ident = np.arange(dm.n_dof + 1, dtype=np.int32)
    A.set_csr(ident, np.arange(dm.n_dof, dtype=np.int32), np.ones(dm.n_dof))
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    arrays = G_.term_arrays(p, dm)
    import ctypes
    from getdp_gb300 import _lib
    with pytest.raises(LA.GetDPError):
        _lib.check(_lib.load().gb300_generate_values(
            A.h, b.h, ctypes.byref(G_.host_batch(arrays))))


def test_empty_system():
    A = LA.LinAlg_CreateMatrix(None, 0)
    A.set_csr([0], [], [])
    b = LA.LinAlg_CreateVector(None, 0)
    x = LA.LinAlg_CreateVector(None, 0)
    info = LA.LinAlg_Solve(A, b, _solver({}), x)
    assert info["status"] == 0


def test_linalg_product_and_norm():
    d, p, dm = G.load("cc_edge_n4")
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    v = LA.LinAlg_CreateVector(None, dm.n_dof)
    rng = np.random.default_rng(0)
    xv = rng.standard_normal(dm.n_dof)
    v.set(xv)
    y = LA.LinAlg_CreateVector(None, dm.n_dof)
    LA.LinAlg_ProdMatrixVector(A, v, y)
    import scipy.sparse as sp
    ref = sp.csr_matrix((d["data"], d["indices"], d["indptr"])) @ xv
    assert np.allclose(y.numpy(), ref, rtol=1e-13, atol=1e-13 * np.max(np.abs(ref)))
    assert abs(LA.LinAlg_VectorNorm2(v) - np.linalg.norm(xv)) <= 1e-13 * np.linalg.norm(xv)


def test_complex_adds_skip_zero_parts():
    A = LA.LinAlg_CreateMatrix(None, 4)
    LA.LinAlg_AddComplexInMatrix(2.0, 0.0, A, 0, 0, 1, 1)
    LA.LinAlg_AddComplexInMatrix(0.0, 3.0, A, 2, 0, 3, 1)
    LA.LinAlg_AddComplexInMatrix(1.0, 1.0, A, 2, 2, 3, 3)
    LA.LinAlg_AddComplexInMatrix(1.0, 1.0, A, 0, 2, 1, 3)
    ip, ix, dv = A.csr()
    dense = np.zeros((4, 4))
    for i in range(4):
        for k in range(ip[i], ip[i + 1]):
            dense[i, ix[k]] = dv[k]
    # (0,0),(1,1) real 2; rows 2/3 to cols 0/1 imaginary only
    assert dense[0, 0] == 2 and dense[1, 1] == 2 and dense[0, 1] == 0
    assert dense[2, 1] == -3 and dense[3, 0] == 3
    assert ip[-1] == 2 + 2 + 4 + 4


# Renumbering_Technique 1: the backend's multicolour ordering for the
# ILU(0) (Sparskit uses RCMK there).  The preconditioner differs from the
# oracle's, so the iteration count does; the solution is the same system's.
@pytest.mark.parametrize("name", ["ms2d_n24", "eddy_n8", "ms2d_n8"])
def test_multicolour_ilu_solution_matches_oracle(name):
    d, p, dm = G.load(name)
    par = _golden_params(d)
    par.update(Renumbering_Technique=1, Stopping_Test="1e-14", Nb_Iter_Max=20000)
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    assert info["status"] == 0, info
    kw = oracle.params_from_golden(d["par_keys"], d["par_vals"])
    kw.update(renumbering=1, stopping_test=float(np.float32(1e-14)), nb_iter_max=20000)
    xo, st, its, _ = oracle.solve(d["indptr"], d["indices"], d["data"], d["b"], **kw)
    assert st == 0
    assert np.linalg.norm(x.numpy() - xo) <= 1e-10 * np.linalg.norm(xo)
    # the same solve again: the ordering and every reduction are deterministic
    x2 = LA.LinAlg_CreateVector(None, dm.n_dof)
    info2 = LA.LinAlg_Solve(A, b, _solver(par), x2)
    assert info2["iterations"] == info["iterations"]
    assert np.array_equal(x.numpy(), x2.numpy())


def test_multicolour_ilu_at_reference_tolerance():
    # the reference's own parameters (RCMK on, 1e-10): the GPU's solution is
    # within the tolerance's reach of the oracle's, and the true residual
    # meets the stopping test
    d, p, dm = G.load("ms2d_n24")
    par = _golden_params(d)
    assert par.get("Renumbering_Technique", 1) == 1
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    assert info["status"] == 0, info
    # GMRES stops on its Givens estimate of the residual, which drifts
    # from the true residual in rounding (in the reference's RCMK order the
    # GPU's true residual is within 1.01x the stopping test,
    # test_reference_order_reproduces_the_reference_run)
    print(f"true residual / (stopping test * ||b||): "
          f"{info['true_residual'] / (1e-10 * info['rhs_norm']):.3f}")
    assert info["true_residual"] <= 1.01e-10 * info["rhs_norm"], info
    assert np.linalg.norm(x.numpy() - d["x"]) <= 1e-6 * np.linalg.norm(d["x"])


@pytest.mark.parametrize("name", ["ms2d_n8", "ms2d_n12_dir", "ms2d_n24", "ms2d_n24_ilu32",
                                  "eddy_n8", "eddy_n8_dir"])
def test_reference_order_reproduces_the_reference_run(name):
    # the golden runs of the reference binary itself, with its default RCMK
    # order: in the same order (Renumbering_Technique 2) the GPU takes the
    # reference's step count (+-1: classical against modified Gram-Schmidt),
    # its true residual meets the stopping test, and the solution is the
    # reference's within the tolerance's reach
    d, p, dm = G.load(name)
    par = _golden_params(d)
    assert par["Renumbering_Technique"] == 1
    par["Renumbering_Technique"] = 2
    if str(d["exe"]) == "getdp_ilu32":
        par["Precision"] = 2  # the reference built with HAVE_ILU_FLOAT
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    assert info["status"] == 0, info
    assert abs(info["iterations"] - int(d["iterations"])) <= 1, (info, int(d["iterations"]))
    rtol = float(np.float32(par["Stopping_Test"]))
    assert info["true_residual"] <= 1.01 * rtol * info["rhs_norm"], info
    assert np.linalg.norm(x.numpy() - d["x"]) <= 1e-6 * np.linalg.norm(d["x"])


def test_multicolour_fgmres_curlcurl_backward_error():
    d, p, dm = G.load("cc_edge_n4")
    par = _golden_params(d)
    par.update(Renumbering_Technique=1)
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    assert info["status"] == 0, info
    # kappa ~ 3e11: the Givens estimate of FGMRES drifts from the true
    # residual (on the oracle too), so the bar is the oracle's own true
    # residual with its RCMK ordering
    kw = oracle.params_from_golden(d["par_keys"], d["par_vals"])
    kw.update(renumbering=1, stopping_test=float(np.float32(kw["stopping_test"])))
    xo, st, its, _ = oracle.solve(d["indptr"], d["indices"], d["data"], d["b"], **kw)
    import scipy.sparse as sp
    Am = sp.csr_matrix((d["data"], d["indices"], d["indptr"]))
    res = np.linalg.norm(d["b"] - Am @ x.numpy())
    res_oracle = np.linalg.norm(d["b"] - Am @ xo)
    target = kw["stopping_test"] * np.linalg.norm(d["b"])
    assert res <= 20 * max(res_oracle, target), (res, res_oracle, target)


# ---- wide levels: the sliced-ELL sweeps ---------------------------------
# The golden systems are small: every level of their triangular solves fits
# the one-block kernel.  A 5-point Laplacian with its rows in red-black
# order has two levels per sweep of m^2 / 2 rows each, so the wide-level
# (sliced-ELL) kernels run, in GetDP's order the oracle also follows.
def _red_black_laplacian(m, shift=1e-2):
    import scipy.sparse as sp
    T = sp.diags([-np.ones(m - 1), 2 * np.ones(m), -np.ones(m - 1)], [-1, 0, 1])
    A = (sp.kron(sp.identity(m), T) + sp.kron(T, sp.identity(m)) +
         shift * sp.identity(m * m)).tocsr()
    ii, jj = np.divmod(np.arange(m * m), m)
    perm = np.concatenate([np.flatnonzero((ii + jj) % 2 == 0),
                           np.flatnonzero((ii + jj) % 2 == 1)])
    P = A[perm][:, perm].tocsr()
    P.sort_indices()
    return P


@pytest.mark.parametrize("algorithm,precision,ilu", [(8, 0, "64"), (9, 1, "32")])
def test_wide_levels_match_oracle(algorithm, precision, ilu):
    A = _red_black_laplacian(90)  # two levels of 4,050 rows per sweep
    n = A.shape[0]
    rng = np.random.default_rng(11)
    bv = rng.standard_normal(n)
    G2 = LA.LinAlg_CreateMatrix(None, n)
    G2.set_csr(A.indptr, A.indices, A.data)
    b = LA.LinAlg_CreateVector(None, n)
    b.set(bv)
    x = LA.LinAlg_CreateVector(None, n)
    par = {"Algorithm": algorithm, "Preconditioner": 6, "Krylov_Size": 30,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-12", "Nb_Iter_Max": 5000,
           "Precision": precision}
    info = LA.LinAlg_Solve(G2, b, _solver(par), x)
    xo, st, its, _ = oracle.solve(A.indptr, A.indices, A.data, bv, algorithm=algorithm,
                                  preconditioner=6, renumbering=0, krylov_size=30,
                                  stopping_test=float(np.float32(1e-12)),
                                  nb_iter_max=5000, ilu=ilu)
    assert st == 0 and info["status"] == 0, (info, st)
    assert abs(info["iterations"] - its) <= 0.05 * its + 2, (info, its)
    assert np.linalg.norm(x.numpy() - xo) <= 1e-9 * np.linalg.norm(xo)


def test_wide_levels_batched_match_single():
    import scipy.sparse as sp
    A1 = _red_black_laplacian(72)
    A2 = _red_black_laplacian(66, shift=5e-2)  # levels of 2,592 and 2,178 rows
    A = sp.block_diag([A1, A2]).tocsr()
    A.sort_indices()
    n1, n = A1.shape[0], A.shape[0]
    rng = np.random.default_rng(5)
    bv = rng.standard_normal(n)
    G2 = LA.LinAlg_CreateMatrix(None, n)
    G2.set_csr(A.indptr, A.indices, A.data)
    b = LA.LinAlg_CreateVector(None, n)
    b.set(bv)
    x = LA.LinAlg_CreateVector(None, n)
    par = {"Algorithm": 8, "Preconditioner": 6, "Krylov_Size": 20,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-12", "Nb_Iter_Max": 5000}
    infos = LA.LinAlg_SolveBatch(G2, b, _solver(par), x, np.array([0, n1, n]))
    xs = x.numpy()
    for k, (Ak, lo, hi) in enumerate([(A1, 0, n1), (A2, n1, n)]):
        xo, st, its, _ = oracle.solve(Ak.indptr, Ak.indices, Ak.data, bv[lo:hi],
                                      algorithm=8, preconditioner=6, renumbering=0,
                                      krylov_size=20, stopping_test=float(np.float32(1e-12)),
                                      nb_iter_max=5000)
        assert st == 0 and infos[k]["status"] == 0, (k, infos[k], st)
        assert abs(infos[k]["iterations"] - its) <= 0.05 * its + 2, (k, infos[k], its)
        assert np.linalg.norm(xs[lo:hi] - xo) <= 1e-9 * np.linalg.norm(xo)


# ---- the multicolour ordering itself ------------------------------------
def _first_fit_from_last(indptr, indices, bs):
    """The colouring the backend computes: sequential first fit over the
    vertices (bs consecutive rows each) from the last to the first."""
    nv = (len(indptr) - 1) // bs
    col = -np.ones(nv, np.int64)
    for v in range(nv - 1, -1, -1):
        nb = indices[indptr[v * bs]:indptr[v * bs + bs]] // bs
        used = set(col[nb[nb != v]].tolist())
        c = 0
        while c in used:
            c += 1
        col[v] = c
    order = np.argsort(col, kind="stable")
    return (order[:, None] * bs + np.arange(bs)[None, :]).ravel()


@pytest.mark.parametrize("name,bs", [("ms2d_n24", 1), ("eddy_n8", 2), ("cc_edge_n4", 1)])
def test_multicolour_ordering_is_first_fit_from_last(name, bs):
    # the GPU's multicolour solve takes the steps the oracle takes on the
    # system permuted by the first-fit colouring from the last vertex
    import scipy.sparse as sp
    d, p, dm = G.load(name)
    par = _golden_params(d)
    par.update(Renumbering_Technique=1, Nb_Iter_Max=5000)
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    perm = _first_fit_from_last(d["indptr"], d["indices"], bs)
    M = sp.csr_matrix((d["data"], d["indices"], d["indptr"]))[perm][:, perm].tocsr()
    M.sort_indices()
    kw = oracle.params_from_golden(d["par_keys"], d["par_vals"])
    kw.update(renumbering=0, nb_iter_max=5000,
              stopping_test=float(np.float32(kw["stopping_test"])))
    xo, st, its, _ = oracle.solve(M.indptr, M.indices, M.data, d["b"][perm], **kw)
    assert st == 0 and info["status"] == 0, (info, st, its)
    xg = x.numpy()[perm]
    if name in ILL_CONDITIONED:
        # counts depend on rounding there (see test_solve_matches_oracle):
        # the bar is the step count within 25 % and the backward error
        assert abs(info["iterations"] - its) <= 0.25 * its, (info["iterations"], its)
        res_gpu = np.linalg.norm(d["b"][perm] - M @ xg)
        res_oracle = np.linalg.norm(d["b"][perm] - M @ xo)
        target = kw["stopping_test"] * np.linalg.norm(d["b"])
        assert res_gpu <= 20 * max(res_oracle, target), (res_gpu, res_oracle, target)
        return
    assert abs(info["iterations"] - its) <= 0.05 * its + 2, (info["iterations"], its)
    assert np.linalg.norm(xg - xo) <= 1e-6 * np.linalg.norm(xo)


# ---- abnormal right-hand sides --------------------------------------------
@pytest.mark.parametrize("kind", ["zero", "nan", "inf"])
@pytest.mark.parametrize("algorithm,precond,precision", [(1, 0, 0), (1, 0, 1), (8, 6, 0),
                                                         (9, 6, 0), (9, 6, 1)])
def test_abnormal_rhs_status_matches_oracle(kind, algorithm, precond, precision):
    # what the reference returns for a zero, NaN or infinite right-hand side
    # (status code, products counted, x = 0): CG stops at its first brkdn,
    # GMRES at the restart test or at mgsro's norm check
    d, p, dm = G.load("ms2d_n8")
    bv = np.zeros(dm.n_dof)
    if kind != "zero":
        bv[:] = 1.0
        bv[3] = np.nan if kind == "nan" else np.inf
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(bv)
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    par = {"Algorithm": algorithm, "Preconditioner": precond, "Krylov_Size": 10,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-10", "Nb_Iter_Max": 100,
           "Precision": precision}
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    xo, st, its, _ = oracle.solve(d["indptr"], d["indices"], d["data"], bv,
                                  algorithm=algorithm, preconditioner=precond,
                                  renumbering=0, krylov_size=10, nb_iter_max=100,
                                  stopping_test=float(np.float32(1e-10)))
    assert info["status"] == st, (info, st, its)
    assert info["iterations"] == its, (info, its)
    assert not np.any(x.numpy()) and not np.any(xo)


@pytest.mark.parametrize("algorithm,precond", [(1, 0), (8, 6), (9, 6)])
@pytest.mark.parametrize("cap", [1, 2, 5, 17])
def test_iteration_cap_matches_oracle(algorithm, precond, cap):
    # Nb_Iter_Max reached: status -1, the products counted as Sparskit
    # counts them, and the partial solution of that many steps
    d, p, dm = G.load("ms2d_n24")
    A = LA.LinAlg_CreateMatrix(None, dm.n_dof)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    b = LA.LinAlg_CreateVector(None, dm.n_dof)
    b.set(d["b"])
    x = LA.LinAlg_CreateVector(None, dm.n_dof)
    par = {"Algorithm": algorithm, "Preconditioner": precond, "Krylov_Size": 10,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-10", "Nb_Iter_Max": cap}
    info = LA.LinAlg_Solve(A, b, _solver(par), x)
    xo, st, its, _ = oracle.solve(d["indptr"], d["indices"], d["data"], d["b"],
                                  algorithm=algorithm, preconditioner=precond,
                                  renumbering=0, krylov_size=10, nb_iter_max=cap,
                                  stopping_test=float(np.float32(1e-10)))
    assert st == -1 and info["status"] == -1, (info, st)
    assert info["iterations"] == its, (info, its)
    assert np.linalg.norm(x.numpy() - xo) <= 1e-9 * np.linalg.norm(xo)


@pytest.mark.parametrize("n", [1, 5])
@pytest.mark.parametrize("algorithm,precond", [(1, 0), (8, 6), (9, 6), (8, 0)])
def test_tiny_systems_match_oracle(n, algorithm, precond):
    # one and five unknowns with a restart length of 50: on one unknown
    # GMRES's first Arnoldi vector is a multiple of the basis, which the
    # reference reports as a break-down (-3) with the exact solution
    import scipy.sparse as sp
    if n == 1:
        A = sp.csr_matrix(np.array([[2.0]]))
    else:
        A = sp.diags([-np.ones(n - 1), 2.5 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1]).tocsr()
    A.sort_indices()
    bv = np.arange(1, n + 1, dtype=float)
    G2 = LA.LinAlg_CreateMatrix(None, n)
    G2.set_csr(A.indptr, A.indices, A.data)
    b = LA.LinAlg_CreateVector(None, n)
    b.set(bv)
    x = LA.LinAlg_CreateVector(None, n)
    par = {"Algorithm": algorithm, "Preconditioner": precond, "Krylov_Size": 50,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-10", "Nb_Iter_Max": 100}
    info = LA.LinAlg_Solve(G2, b, _solver(par), x)
    xo, st, its, _ = oracle.solve(A.indptr, A.indices, A.data, bv, algorithm=algorithm,
                                  preconditioner=precond, renumbering=0, krylov_size=50,
                                  nb_iter_max=100, stopping_test=float(np.float32(1e-10)))
    assert info["status"] == st and info["iterations"] == its, (info, st, its)
    assert np.linalg.norm(x.numpy() - xo) <= 1e-12 * np.linalg.norm(xo)


@pytest.mark.parametrize("renumbering", [0, 1])
@pytest.mark.parametrize("algorithm", [8, 9])
def test_solve_again_reuses_the_factorisation(renumbering, algorithm):
    # LinAlg_SolveAgain keeps the ILU(0) factor of the previous solve of A
    # (Re_Use_LU, LinAlg_SPARSKIT.cpp:578-585): a second right-hand side is
    # solved without factoring again, with the same iterates as a solve that
    # factors; a Generate makes a new matrix, whose first solve factors
    p = W.magnetostatics_2d(24, seed=12)
    dm = W.dofmap_for(p)
    par = {"Algorithm": algorithm, "Preconditioner": 6, "Krylov_Size": 50,
           "Renumbering_Technique": renumbering, "Stopping_Test": "1e-12"}
    S = _solver(par)
    n = dm.n_dof
    A, b = G_.generate_problem(p, dm)
    x = LA.LinAlg_CreateVector(None, n)
    info0 = LA.LinAlg_Solve(A, b, S, x)
    assert info0["status"] == 0 and info0["ilu_factorized"] == 1
    b2 = LA.LinAlg_CreateVector(None, n)
    b2.set(b.numpy() * 0.5 + 1e-3 * np.cos(np.arange(n)))
    xa = LA.LinAlg_CreateVector(None, n)
    ia = LA.LinAlg_SolveAgain(A, b2, S, xa)
    assert ia["status"] == 0 and ia["ilu_factorized"] == 0
    assert S["re_use_lu"] == 0  # restored after the call
    xf = LA.LinAlg_CreateVector(None, n)
    fresh = LA.LinAlg_Solve(A, b2, S, xf)
    assert fresh["ilu_factorized"] == 1
    # the same factor either way: the same iterates
    assert ia["iterations"] == fresh["iterations"]
    assert np.array_equal(xa.numpy(), xf.numpy())
    # after a Generate: a new matrix, factored on its first solve
    G_.generate(A, b, G_.host_batch(G_.term_arrays(p, dm)), pattern=True)
    xg = LA.LinAlg_CreateVector(None, n)
    ig = LA.LinAlg_SolveAgain(A, b, S, xg)
    assert ig["status"] == 0 and ig["ilu_factorized"] == 1
