"""Batched sweep of independent problems: one Generate and one batched solve
over the diagonal blocks, checked problem by problem against the oracle run
on each problem alone.

Tolerances as in test_gpu_parity: values within 1e-12 relative (plus 1e-13
of the row maximum); solutions within 1e-6 of the oracle's at the
reference tolerance with iteration counts within 5 % + 2, within 1e-10 at
Stopping_Test 1e-14.
"""
import numpy as np
import pytest

import oracle
from tests import tolerances as TOL
from getdp_gb300 import workloads as W

SIZES = [6, 9, 4, 12, 7]


def small_sweep():
    return [W.eddy_2d(n, seed=500 + k) for k, n in enumerate(SIZES)]


def test_concat_numbering_and_offsets():
    probs = small_sweep()
    bt = W.concat_problems(probs)
    assert bt.offsets[0] == 0 and bt.offsets[-1] == bt.dofmap.n_dof
    e0 = 0
    for k, (p, dm) in enumerate(zip(probs, bt.dofmaps)):
        ne = p.mesh.n_elems
        got = bt.dofmap.elem_dofs[e0:e0 + ne]
        want = np.where(dm.elem_dofs >= 0, dm.elem_dofs + bt.offsets[k], -1)
        assert np.array_equal(got, want)
        assert bt.offsets[k + 1] - bt.offsets[k] == dm.n_dof
        om = bt.problem.params["omega_e"][e0:e0 + ne]
        assert np.all(om == p.params["freq"] * 6.2831853071795865)
        e0 += ne


def test_sweep_sizes_and_seeds():
    probs = W.eddy_sweep(n_problems=6, seed=3, n_min=4, n_max=9)
    assert all(4 <= p.params["n"] <= 9 for p in probs)
    assert len({p.params["seed"] for p in probs}) == 6


# ----------------------------------------------------------------- GPU
def _gpu_setup():
    from getdp_gb300 import build
    build.build()
    oracle.build()
    from getdp_gb300 import generate as G_
    from getdp_gb300 import linalg as LA
    probs = small_sweep()
    bt = W.concat_problems(probs)
    A = LA.gMatrix(bt.dofmap.n_dof)
    b = LA.gVector(bt.dofmap.n_dof)
    terms = G_.DeviceTerms(bt.problem, bt.dofmap)
    G_.generate(A, b, terms.batch, pattern=True)
    return probs, bt, A, b, LA


def _solver(LA, par):
    S = LA.LinAlg_CreateSolver(None)
    for k, v in par.items():
        S.set(k, v)
    return S


@pytest.mark.gpu
def test_batched_generate_matches_oracle_blocks():
    probs, bt, A, b, LA = _gpu_setup()
    ip, ix, dv = A.csr()
    bb = b.numpy()
    for k, (p, dm) in enumerate(zip(probs, bt.dofmaps)):
        r0, r1 = bt.offsets[k], bt.offsets[k + 1]
        oip, oix, odv, ob, sabs, babs = oracle.assemble(p, dm, with_abs=True)
        s, e = ip[r0], ip[r1]
        assert np.array_equal(ip[r0:r1 + 1] - s, oip)
        assert np.array_equal(ix[s:e] - r0, oix)
        assert TOL.values_close(dv[s:e], odv, TOL.matrix_scale(oip, oix, odv, sabs, True))
        assert TOL.values_close(bb[r0:r1], ob, babs)


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", [8, 9])
def test_batched_solve_matches_oracle_per_problem(algorithm):
    probs, bt, A, b, LA = _gpu_setup()
    par = {"Algorithm": algorithm, "Preconditioner": 6, "Krylov_Size": 20,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-10", "Nb_Iter_Max": 2000}
    x = LA.gVector(bt.dofmap.n_dof)
    infos = LA.LinAlg_SolveBatch(A, b, _solver(LA, par), x, bt.offsets)
    xs = x.numpy()
    for k, (p, dm) in enumerate(zip(probs, bt.dofmaps)):
        oip, oix, odv, ob = oracle.assemble(p, dm)
        xo, st, its, _ = oracle.solve(oip, oix, odv, ob, algorithm=algorithm,
                                      preconditioner=6, renumbering=0, krylov_size=20,
                                      stopping_test=float(np.float32(1e-10)),
                                      nb_iter_max=2000)
        assert st == 0 and infos[k]["status"] == 0, (k, infos[k], st)
        assert abs(infos[k]["iterations"] - its) <= 0.05 * its + 2, (k, infos[k], its)
        xk = xs[bt.offsets[k]:bt.offsets[k + 1]]
        assert np.linalg.norm(xk - xo) <= 1e-6 * np.linalg.norm(xo), k


@pytest.mark.gpu
def test_batched_solve_equals_single_solves():
    # each system of the batch runs the single-system iteration: same
    # iteration counts, solutions within rounding of the reductions
    probs, bt, A, b, LA = _gpu_setup()
    par = {"Algorithm": 8, "Preconditioner": 6, "Krylov_Size": 20,
           "Renumbering_Technique": 0, "Stopping_Test": "1e-12", "Nb_Iter_Max": 2000}
    x = LA.gVector(bt.dofmap.n_dof)
    infos = LA.LinAlg_SolveBatch(A, b, _solver(LA, par), x, bt.offsets)
    xs = x.numpy()
    from getdp_gb300 import generate as G_
    for k, (p, dm) in enumerate(zip(probs, bt.dofmaps)):
        A1, b1 = G_.generate_problem(p, dm)
        x1 = LA.gVector(dm.n_dof)
        info1 = LA.LinAlg_Solve(A1, b1, _solver(LA, par), x1)
        assert abs(info1["iterations"] - infos[k]["iterations"]) <= 1, (k, info1, infos[k])
        xk = xs[bt.offsets[k]:bt.offsets[k + 1]]
        assert np.linalg.norm(xk - x1.numpy()) <= 1e-9 * np.linalg.norm(x1.numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_batched_multicolour_tight(precision):
    probs, bt, A, b, LA = _gpu_setup()
    par = {"Algorithm": 9, "Preconditioner": 6, "Krylov_Size": 30,
           "Renumbering_Technique": 1, "Stopping_Test": "1e-14", "Nb_Iter_Max": 5000,
           "Precision": precision}
    x = LA.gVector(bt.dofmap.n_dof)
    infos = LA.LinAlg_SolveBatch(A, b, _solver(LA, par), x, bt.offsets)
    xs = x.numpy()
    for k, (p, dm) in enumerate(zip(probs, bt.dofmaps)):
        assert infos[k]["status"] == 0, (k, infos[k])
        oip, oix, odv, ob = oracle.assemble(p, dm)
        xo, st, its, _ = oracle.solve(oip, oix, odv, ob, algorithm=9, preconditioner=6,
                                      renumbering=1, krylov_size=30,
                                      stopping_test=float(np.float32(1e-14)),
                                      nb_iter_max=5000)
        assert st == 0
        xk = xs[bt.offsets[k]:bt.offsets[k + 1]]
        assert np.linalg.norm(xk - xo) <= 1e-10 * np.linalg.norm(xo), k


@pytest.mark.gpu
def test_batched_rejects_coupled_blocks_and_bad_offsets():
    probs, bt, A, b, LA = _gpu_setup()
    from getdp_gb300._lib import GetDPError
    x = LA.gVector(bt.dofmap.n_dof)
    par = {"Algorithm": 8, "Preconditioner": 6}
    off = bt.offsets.copy()
    off[2] += 1  # a block boundary inside a problem: its entries cross it
    with pytest.raises(GetDPError, match="couples two systems"):
        LA.LinAlg_SolveBatch(A, b, _solver(LA, par), x, off)
    off = bt.offsets.copy()
    off[-1] -= 1
    with pytest.raises(GetDPError, match="offsets"):
        LA.LinAlg_SolveBatch(A, b, _solver(LA, par), x, off)


# ------------------------------------------ one launch, a cluster per system
def _solve_form(LA, A, b, bt, par, form):
    x = LA.gVector(bt.dofmap.n_dof)
    S = _solver(LA, dict(par, Batch_Kernel=form))
    infos = LA.LinAlg_SolveBatch(A, b, S, x, bt.offsets)
    return infos, x.numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm,precision,renumbering",
                         [(8, 0, 1), (9, 0, 1), (9, 1, 1), (8, 1, 1), (9, 0, 0)])
def test_cluster_form_follows_the_per_kernel_form(algorithm, precision, renumbering):
    # the same iteration per system: step counts within 1 (the sums are
    # formed in another order), solutions within rounding of the reductions
    probs, bt, A, b, LA = _gpu_setup()
    par = {"Algorithm": algorithm, "Preconditioner": 6, "Krylov_Size": 20,
           "Renumbering_Technique": renumbering, "Stopping_Test": "1e-12",
           "Nb_Iter_Max": 3000, "Precision": precision}
    i0, x0 = _solve_form(LA, A, b, bt, par, 0)
    for form in (1, 2, 4, 8, 16):  # clusters of 1 to 16 CTAs
        i1, x1 = _solve_form(LA, A, b, bt, par, form)
        for k in range(len(probs)):
            assert i1[k]["batch_form"] == 1 and i0[k]["batch_form"] == 0
            assert i1[k]["status"] == 0 and i0[k]["status"] == 0, (k, i1[k], i0[k])
            assert abs(i1[k]["iterations"] - i0[k]["iterations"]) <= 1, (k, i1[k], i0[k])
            r0, r1 = bt.offsets[k], bt.offsets[k + 1]
            assert np.linalg.norm(x1[r0:r1] - x0[r0:r1]) <= 1e-9 * np.linalg.norm(x0[r0:r1])
            assert i1[k]["true_residual"] <= 1.01e-12 * i1[k]["rhs_norm"] or \
                i1[k]["true_residual"] <= 2 * i0[k]["true_residual"], (k, i1[k], i0[k])


@pytest.mark.gpu
def test_cluster_form_uneven_sizes_against_oracle():
    # more systems than clusters fit at once, sizes 3x3 to 30x30 cells,
    # taken from the queue largest first; each against the oracle alone
    oracle.build()
    from getdp_gb300 import generate as G_
    from getdp_gb300 import linalg as LA
    probs = W.eddy_sweep(n_problems=48, seed=11, n_min=3, n_max=30)
    bt = W.concat_problems(probs)
    A = LA.gMatrix(bt.dofmap.n_dof)
    b = LA.gVector(bt.dofmap.n_dof)
    terms = G_.DeviceTerms(bt.problem, bt.dofmap)
    G_.generate(A, b, terms.batch, pattern=True)
    par = {"Algorithm": 9, "Preconditioner": 6, "Krylov_Size": 30,
           "Renumbering_Technique": 1, "Stopping_Test": "1e-14", "Nb_Iter_Max": 5000}
    infos, xs = _solve_form(LA, A, b, bt, par, 4)
    assert all(d["batch_form"] == 1 and d["status"] == 0 for d in infos), infos
    for k in (0, 7, 19, 33, 47):
        oip, oix, odv, ob = oracle.assemble(probs[k], bt.dofmaps[k])
        xo, st, its, _ = oracle.solve(oip, oix, odv, ob, algorithm=9, preconditioner=6,
                                      renumbering=1, krylov_size=30,
                                      stopping_test=float(np.float32(1e-14)),
                                      nb_iter_max=5000)
        assert st == 0
        xk = xs[bt.offsets[k]:bt.offsets[k + 1]]
        assert np.linalg.norm(xk - xo) <= 1e-10 * np.linalg.norm(xo), k


@pytest.mark.gpu
def test_cluster_form_without_preconditioner_and_at_the_iteration_cap():
    probs, bt, A, b, LA = _gpu_setup()
    # without a preconditioner some of these systems stagnate (GMRES(15)):
    # both forms end the same way, converged or at the cap
    par = {"Algorithm": 8, "Preconditioner": 0, "Krylov_Size": 15,
           "Renumbering_Technique": 1, "Stopping_Test": "1e-10", "Nb_Iter_Max": 800}
    i1, x1 = _solve_form(LA, A, b, bt, par, 4)
    i0, x0 = _solve_form(LA, A, b, bt, par, 0)
    for k in range(len(probs)):
        assert i1[k]["batch_form"] == 1
        assert i1[k]["status"] == i0[k]["status"], (k, i1[k], i0[k])
        assert abs(i1[k]["iterations"] - i0[k]["iterations"]) <= 0.05 * i0[k]["iterations"] + 2
        if i0[k]["status"] != 0:
            assert abs(i1[k]["residual_estimate"] - i0[k]["residual_estimate"]) <= \
                1e-6 * i0[k]["residual_estimate"], (k, i1[k], i0[k])
    # a cap every system reaches: status -1 and the cap's product count, as
    # the per-kernel form reports them (a warning, as LinAlg_Solve gives)
    capped = dict(par, Nb_Iter_Max=7)
    i1, x1 = _solve_form(LA, A, b, bt, capped, 4)
    i0, x0 = _solve_form(LA, A, b, bt, capped, 0)
    for k in range(len(probs)):
        assert i1[k]["status"] == i0[k]["status"] == -1
        assert "terminated" in i1[k]["warning"]
        assert i1[k]["iterations"] == i0[k]["iterations"]
        r0, r1 = bt.offsets[k], bt.offsets[k + 1]
        assert np.linalg.norm(x1[r0:r1] - x0[r0:r1]) <= 1e-10 * np.linalg.norm(x0[r0:r1])


@pytest.mark.gpu
def test_cluster_form_falls_back_beyond_its_krylov_size():
    probs, bt, A, b, LA = _gpu_setup()
    par = {"Algorithm": 9, "Preconditioner": 6, "Krylov_Size": 80,
           "Renumbering_Technique": 1, "Stopping_Test": "1e-10", "Nb_Iter_Max": 2000}
    infos, _ = _solve_form(LA, A, b, bt, par, 4)
    assert all(d["batch_form"] == 0 and d["status"] == 0 for d in infos)
