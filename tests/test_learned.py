"""The learned correction of the ILU(0) preconditioner: the network's
hand-written forward and backward kernels against the FP64 oracle
(oracle/mpnn_port.py), the oracle's gradient against finite differences,
training on the GPU, and the solve with its fallback.

Tolerances: oracle gradient vs central differences (FP64, no BF16
rounding): 1e-6 of the largest gradient entry; GPU vs oracle (same BF16
weights; the GPU accumulates in FP32 with atomics in varying order): loss
within 1e-5 relative, gradient within 2e-3 of the largest entry.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle
from getdp_gb300 import workloads as W
from oracle import mpnn_port as M


def small_system(n=6, seed=5):
    p = W.nonlinear_2d(n=n, seed=seed)
    dm = W.dofmap_for(p)
    ip, ix, dv, b = oracle.assemble(p, dm)
    return p, dm, ip, ix, dv, b


@pytest.mark.parametrize("with_solution", [True, False])
def test_oracle_gradient_matches_finite_differences(with_solution):
    oracle.build()
    _, _, ip, ix, dv, _ = small_system()
    A = sp.csr_matrix((dv, ix, ip))
    g = M.graph(ip, ix, dv)
    rng = np.random.default_rng(3)
    w = rng.standard_normal(M.NPARAM) * 0.3
    r1 = rng.standard_normal(g["n"])
    e1 = rng.standard_normal(g["n"]) if with_solution else None
    _, grad, _ = M.loss_grad(w, g, r1, e1, A, bf16_weights=False)
    idx = np.concatenate([rng.choice(M.NPARAM, 40, replace=False),
                          [M.OFF_CO, M.OFF_BD, M.OFF_WO + 1, M.OFF_WD + 2, M.OFF_WIN]])
    h = 1e-6
    for k in idx:
        wp, wm = w.copy(), w.copy()
        wp[k] += h
        wm[k] -= h
        fd = (M.loss_grad(wp, g, r1, e1, A, bf16_weights=False)[0] -
              M.loss_grad(wm, g, r1, e1, A, bf16_weights=False)[0]) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-6 * np.abs(grad).max() + 1e-12, (k, fd, grad[k])


def _coarse(p, dm, ip, ix, dv, cells=3):
    agg, nc = W.cell_aggregates(p, dm, cells)
    A = sp.csr_matrix((dv, ix, ip))
    P0 = sp.csr_matrix((np.ones(dm.n_dof), (np.arange(dm.n_dof), agg)),
                       shape=(dm.n_dof, nc))
    return agg, nc, P0, np.linalg.inv((P0.T @ A @ P0).toarray())


@pytest.mark.parametrize("with_solution", [True, False])
def test_oracle_two_level_gradient_matches_finite_differences(with_solution):
    # the loss after the coarse correction, (e1 - y)^T (A - A C A) (e1 - y) / S
    oracle.build()
    p, dm, ip, ix, dv, _ = small_system()
    A = sp.csr_matrix((dv, ix, ip))
    _, _, P0, Aci = _coarse(p, dm, ip, ix, dv)
    g = M.graph(ip, ix, dv)
    rng = np.random.default_rng(4)
    w = rng.standard_normal(M.NPARAM) * 0.3
    r1 = rng.standard_normal(g["n"])
    # the loss is written for e1 = A^-1 r1 (the error that r1 leaves)
    e1 = spla.spsolve(A.tocsc(), r1) if with_solution else None
    lo, grad, G = M.loss_grad(w, g, r1, e1, A, bf16_weights=False, coarse=(P0, Aci))
    # the loss itself, written out
    y = np.zeros(g["n"])
    np.add.at(y, g["rows"], G * r1[g["cols"]])
    if with_solution:
        C = P0 @ Aci @ P0.T
        d = e1 - y
        want = float(d @ (A @ d) - (A @ d) @ (C @ (A @ d))) / float(e1 @ (A @ e1))
        assert abs(lo - want) <= 1e-12 * max(1.0, abs(want))
    idx = np.concatenate([rng.choice(M.NPARAM, 40, replace=False),
                          [M.OFF_CO, M.OFF_BD, M.OFF_WO + 1, M.OFF_WD + 2, M.OFF_WIN]])
    h = 1e-6
    for k in idx:
        wp, wm = w.copy(), w.copy()
        wp[k] += h
        wm[k] -= h
        fd = (M.loss_grad(wp, g, r1, e1, A, bf16_weights=False, coarse=(P0, Aci))[0] -
              M.loss_grad(wm, g, r1, e1, A, bf16_weights=False, coarse=(P0, Aci))[0]) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-6 * np.abs(grad).max() + 1e-12, (k, fd, grad[k])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], np.float32)
    r = M.bf16(x)
    u = np.asarray(r, np.float32).view(np.uint32)
    assert np.all(u & 0xFFFF == 0)
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)
    assert r[1] == 1.0  # the tie 1 + 2^-8 rounds to even


# ----------------------------------------------------------------- GPU
def _gpu():
    from getdp_gb300 import build
    build.build()
    oracle.build()
    from getdp_gb300 import generate as G
    from getdp_gb300 import learned as LR
    from getdp_gb300 import linalg as LA
    return G, LR, LA


@pytest.mark.gpu
@pytest.mark.parametrize("with_solution", [True, False])
def test_gpu_forward_backward_match_oracle(with_solution):
    G, LR, LA = _gpu()
    p, dm, ip, ix, dv, b = small_system(n=12, seed=9)
    A = LA.gMatrix(dm.n_dof)
    A.set_csr(ip, ix, dv)
    net = LR.MPNN(seed=4)
    rng = np.random.default_rng(5)
    w = (rng.standard_normal(net.n_params) * 0.2).astype(np.float32)
    net.set_params(w)
    r1 = rng.standard_normal(dm.n_dof)
    e1 = rng.standard_normal(dm.n_dof)
    vr, ve = LA.gVector(dm.n_dof), LA.gVector(dm.n_dof)
    vr.set(r1)
    ve.set(e1)
    loss, grad = net.loss_grad(A, vr, ve if with_solution else None, want_grad=True)
    g = M.graph(ip, ix, dv)
    lo, go, _ = M.loss_grad(w.astype(np.float64), g, r1, e1 if with_solution else None,
                            sp.csr_matrix((dv, ix, ip)))
    assert abs(loss - lo) <= 1e-5 * abs(lo), (loss, lo)
    assert np.abs(grad - go).max() <= 2e-3 * np.abs(go).max(), np.abs(grad - go).max()


@pytest.mark.gpu
@pytest.mark.parametrize("with_solution", [True, False])
def test_gpu_two_level_loss_matches_oracle(with_solution):
    G, LR, LA = _gpu()
    p, dm, ip, ix, dv, b = small_system(n=12, seed=9)
    agg, nc, P0, Aci = _coarse(p, dm, ip, ix, dv, cells=4)
    A = LA.gMatrix(dm.n_dof)
    A.set_csr(ip, ix, dv)
    A.set_aggregates(agg, nc)
    net = LR.MPNN(seed=4)
    net.set_loss(1)
    rng = np.random.default_rng(6)
    w = (rng.standard_normal(net.n_params) * 0.2).astype(np.float32)
    net.set_params(w)
    r1 = rng.standard_normal(dm.n_dof)
    e1 = rng.standard_normal(dm.n_dof)
    vr, ve = LA.gVector(dm.n_dof), LA.gVector(dm.n_dof)
    vr.set(r1)
    ve.set(e1)
    loss, grad = net.loss_grad(A, vr, ve if with_solution else None, want_grad=True)
    g = M.graph(ip, ix, dv)
    lo, go, _ = M.loss_grad(w.astype(np.float64), g, r1, e1 if with_solution else None,
                            sp.csr_matrix((dv, ix, ip)), coarse=(P0, Aci))
    assert abs(loss - lo) <= 1e-5 * abs(lo), (loss, lo)
    assert np.abs(grad - go).max() <= 2e-3 * np.abs(go).max(), np.abs(grad - go).max()
    # the energy the coarse correction removes, u^T C u, against numpy
    u = LA.gVector(dm.n_dof)
    u.set(r1)
    t = P0.T @ r1
    assert abs(LR.coarse_energy(A, u) - t @ Aci @ t) <= 1e-9 * abs(t @ Aci @ t)


@pytest.mark.gpu
def test_gpu_training_lowers_held_out_loss_and_solve_falls_back_safely():
    G, LR, LA = _gpu()

    def system(n, seed):
        p = W.nonlinear_2d(n=n, seed=seed)
        dm = W.dofmap_for(p)
        A, b = G.generate_problem(p, dm)
        S = LA.LinAlg_CreateSolver(None)
        for k, v in dict(Algorithm=8, Preconditioner=6, Krylov_Size=50,
                         Nb_Iter_Max=20000, Renumbering_Technique=1).items():
            S.set(k, v)
        S["stopping_test"] = 1e-12
        x = LA.gVector(dm.n_dof)
        LA.LinAlg_Solve(A, b, S, x)
        return A, b, x

    samples = []
    for s in range(16):
        A, b, x = system(24, 200 + s)
        samples.append(LR.make_sample(A, b, x))
        samples.extend(LR.make_probes(A, 2, seed=300 + s))
    A, b, x = system(24, 999)
    held = LR.make_sample(A, b, x)
    net = LR.MPNN(seed=2)
    before, _ = net.loss_grad(held.A, held.r1, held.e1)
    assert abs(before - 1.0) < 1e-9  # the head starts at zero: no correction
    LR.train(net, samples, epochs=30, lr=3e-3, batch=8)
    after, _ = net.loss_grad(held.A, held.r1, held.e1)
    assert after < 0.97, after  # the energy error left by the ILU step shrinks
    # the solve converges (learned, or the plain fallback when capped) to the
    # plain solution
    xs = LA.gVector(A.n)
    info = LR.solve(A, b, xs, net, stopping_test=1e-12, cap=400)
    assert info["status"] == 0
    assert np.linalg.norm(xs.numpy() - x.numpy()) <= 1e-7 * np.linalg.norm(x.numpy())
    # a cap of one step forces the fallback
    info = LR.solve(A, b, xs, net, stopping_test=1e-12, cap=1)
    assert info["preconditioner"].startswith("ilu0") and info["status"] == 0


@pytest.mark.gpu
def test_gpu_step_length_and_newton_policy():
    """The energy-optimal step along a correction is 1 for G = A^-1 on the
    ILU residual's span (here: a scaled exact correction is rescaled back),
    and the Newton policy switches the correction off after a failed
    attempt while the loop still converges."""
    G, LR, LA = _gpu()
    import ctypes
    from getdp_gb300 import _lib
    from getdp_gb300 import nonlinear as NL
    p = W.nonlinear_2d(n=16, seed=3)
    dm = W.dofmap_for(p)
    A, b = G.generate_problem(p, dm)
    net = LR.MPNN(seed=2)
    # an untrained head predicts G = 0: no step can be taken along it
    net.infer(A)
    assert LR.step_length(A) == 0.0
    # scaling a correction scales the step inversely
    A.assemble()
    rng = np.random.default_rng(0)
    vals = rng.standard_normal(A.nnz()) * 1e-3
    L = _lib.load()
    _lib.check(L.gb300_matrix_set_correction(A.h, vals.ctypes.data_as(ctypes.c_void_p), 0))
    s1 = LR.step_length(A)
    _lib.check(L.gb300_matrix_scale_correction(A.h, ctypes.c_double(2.0)))
    s2 = LR.step_length(A)
    assert s1 != 0.0 and abs(s2 * 2.0 - s1) <= 1e-9 * abs(s1), (s1, s2)
    # policy: a cap of one step makes the first attempt fail, then it is off
    terms = G.DeviceTerms(p, dm)
    pol = LR.NewtonSolver(net, stopping_test=1e-10, precision=1, first_cap=1)
    r = NL.newton(terms, dm.n_dof, pol, tol_rel=1e-8, iter_max=50,
                  relaxation=(1.0, 0.5, 0.25, 0.125))
    assert r.converged
    kinds = [s["preconditioner"] for s in pol.log]
    assert kinds[0] != "learned"
    assert all(k == "ilu0 (learned off)" for k in kinds[1:]), kinds


@pytest.mark.parametrize("name", ["mpnn_nl2d_256.npy", "mpnn_nl2d_256_twolevel.npy",
                                  "mpnn_nl2d_256_sai.npy"])
def test_committed_weights_fit_the_network(name):
    # the weights that getdp_gb300/weights/train_nl2d.py produced: one
    # parameter vector of the network's layout, finite, with a non-zero head
    import os
    import importlib
    w = np.load(os.path.join(os.path.dirname(__file__), "..", "getdp_gb300", "weights",
                             name))
    assert w.dtype == np.float32 and w.shape == (M.NPARAM,)
    assert np.all(np.isfinite(w))
    assert np.any(w[M.OFF_WO:M.OFF_CO] != 0)  # trained: the output head moved off zero
    # the network's forward pass (the oracle's) runs on them
    rng = np.random.default_rng(0)
    n = 12
    A = sp.diags([-np.ones(n - 1), 2.5 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1]).tocsr()
    g = M.graph(A.indptr, A.indices, A.data)
    out = M.forward(w, g)
    assert np.all(np.isfinite(np.asarray(out[0] if isinstance(out, tuple) else out)))
    importlib.import_module("getdp_gb300.weights.train_nl2d")


@pytest.mark.gpu
def test_gpu_two_level_correction_reduces_steps_on_held_out_systems():
    """The committed correction for the two-level cycle
    (mpnn_nl2d_256_twolevel.npy, trained on Newton systems of seeds 200-364
    at 256^2) on held-out systems of the same distribution (seeds 5, 6):
    FGMRES with it (Preconditioner 22) takes fewer steps than the cycle
    without it (21) and reaches the same solution.  It does not take less
    time than 21: the correction costs two more sparse products per
    smoothing.  Against plain ILU(0)-FGMRES (Preconditioner 6) the learned
    arm takes far fewer steps and less wall time -- a gain of the coarse
    level of the cycle, which the correction is trained inside, more than
    of the network.  Each solver is timed on its second solve (the first
    makes the colouring, the factor's schedule and the CUDA graphs)."""
    import os
    import time
    G, LR, LA = _gpu()
    wfile = os.path.join(os.path.dirname(LR.__file__), "weights",
                         "mpnn_nl2d_256_twolevel.npy")
    net = LR.MPNN(seed=1)
    net.set_params(np.load(wfile))
    for seed in (5, 6):
        p = W.nonlinear_2d(n=256, seed=seed)
        dm = W.dofmap_for(p)
        terms = G.DeviceTerms(p, dm)
        A, b = LA.gMatrix(dm.n_dof), LA.gVector(dm.n_dof)
        G.generate(A, b, terms.batch, pattern=True)
        agg, nc = W.cell_aggregates(p, dm, 8)
        A.set_aggregates(agg, nc)
        net.infer(A)
        sols, steps, secs = [], [], []
        for prec in (21, 22, 6):
            S = LA.LinAlg_CreateSolver(None)
            for k, v in dict(Algorithm=9, Preconditioner=prec, Krylov_Size=50,
                             Nb_Iter_Max=20000, Renumbering_Technique=1,
                             Precision=1).items():
                S.set(k, v)
            S["stopping_test"] = 1e-10
            x = LA.gVector(dm.n_dof)
            for _ in range(2):
                t0 = time.perf_counter()
                info = LA.LinAlg_Solve(A, b, S, x)
                dt = time.perf_counter() - t0
            assert info["status"] == 0
            sols.append(x.numpy())
            steps.append(info["iterations"])
            secs.append(dt)
        print(f"seed {seed}: two-level {steps[0]} steps {secs[0]:.4f} s, with the "
              f"correction {steps[1]} steps {secs[1]:.4f} s, ILU(0) {steps[2]} steps "
              f"{secs[2]:.4f} s")
        assert steps[1] <= 0.95 * steps[0]
        assert np.linalg.norm(sols[1] - sols[0]) <= 1e-6 * np.linalg.norm(sols[0])
        assert steps[1] < steps[2] and secs[1] < secs[2]
        assert np.linalg.norm(sols[2] - sols[1]) <= 1e-6 * np.linalg.norm(sols[2])
