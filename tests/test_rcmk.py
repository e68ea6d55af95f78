"""The reference's RCMK renumbering (Renumbering_Technique 1 in Sparskit,
cmkreord.f with reordering.f's pseudo-peripheral search, Sparskit.cpp:
245-256) on this backend: gb300_rcmk_order is the host order the solver uses
for Renumbering_Technique 2, checked permutation for permutation against the
oracle's restated cmkreord; on the GPU, ILU(0)-GMRES in that order follows
the reference's default iteration trajectory (step counts within 5 % + 2,
solutions within 1e-10 at Stopping_Test 1e-14, as test_gpu_parity)."""
import ctypes

import numpy as np
import pytest

import oracle
from getdp_gb300 import workloads as W


def _order(ip, ix):
    from getdp_gb300 import _lib
    L = _lib.load(build_if_missing=True)
    n = len(ip) - 1
    rp = np.ascontiguousarray(ip, np.int32)
    ci = np.ascontiguousarray(ix, np.int32)
    out = np.zeros(max(n, 1), np.int32)
    P = ctypes.POINTER(ctypes.c_int)
    _lib.check(L.gb300_rcmk_order(n, rp.ctypes.data_as(P), ci.ctypes.data_as(P),
                                  out.ctypes.data_as(P)))
    return out[:n]


def _patterns():
    oracle.build()
    out = []
    for name, p in (("ms2d 16", W.magnetostatics_2d(n=16, seed=5)),
                    ("ms2d 24", W.magnetostatics_2d(n=24, seed=9)),
                    ("p2 elasticity 3", W.elasticity_p2(n=3, seed=2)),
                    ("edge curl-curl 4", W.curlcurl_edge(n=4, seed=1)),
                    ("eddy 8", W.eddy_2d(8, seed=501))):
        ip, ix, dv, b = oracle.assemble(p, W.dofmap_for(p))
        out.append((name, ip, ix))
    # a block-diagonal batch (several connected components)
    probs = [W.eddy_2d(n, seed=600 + k) for k, n in enumerate((5, 3, 7))]
    bt = W.concat_problems(probs)
    ips, ixs, shift, nnz = [0], [], 0, 0
    for k, (p, dm) in enumerate(zip(probs, bt.dofmaps)):
        ip, ix, dv, b = oracle.assemble(p, dm)
        ips.extend((ip[1:] + nnz).tolist())
        ixs.extend((ix + shift).tolist())
        shift += len(ip) - 1
        nnz += len(ix)
    out.append(("eddy batch", np.array(ips), np.array(ixs)))
    return out


def test_rcmk_order_equals_the_reference_permutation():
    for name, ip, ix in _patterns():
        got = _order(ip, ix)
        want = oracle.rcmk_new_of(ip, ix)
        assert np.array_equal(got, want), name
        assert np.array_equal(np.sort(got), np.arange(len(ip) - 1)), name


def test_rcmk_order_rejects_bad_patterns():
    from getdp_gb300._lib import GetDPError
    with pytest.raises(GetDPError, match="out of range"):
        _order(np.array([0, 1, 2]), np.array([0, 5]))
    with pytest.raises(GetDPError, match="decrease"):
        _order(np.array([0, 2, 1]), np.array([0, 1]))


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", [8, 9])
def test_rcmk_solve_follows_the_reference_default(algorithm):
    from getdp_gb300 import linalg as LA
    from getdp_gb300.generate import generate_problem
    oracle.build()
    p = W.magnetostatics_2d(n=24, seed=9)
    dm = W.dofmap_for(p)
    A, b = generate_problem(p, dm)
    ip, ix, dv, ob = oracle.assemble(p, dm)
    S = LA.LinAlg_CreateSolver(None)
    for k, v in (("Algorithm", algorithm), ("Preconditioner", 6), ("Krylov_Size", 40),
                 ("Renumbering_Technique", 2), ("Stopping_Test", "1e-14"),
                 ("Nb_Iter_Max", 5000)):
        S.set(k, v)
    x = LA.gVector(dm.n_dof)
    info = LA.LinAlg_Solve(A, b, S, x)
    xo, st, its, _ = oracle.solve(ip, ix, dv, ob, algorithm=algorithm, preconditioner=6,
                                  renumbering=1, krylov_size=40,
                                  stopping_test=float(np.float32(1e-14)), nb_iter_max=5000)
    assert info["status"] == 0 and st == 0
    assert abs(info["iterations"] - its) <= 0.05 * its + 2, (info["iterations"], its)
    assert np.linalg.norm(x.numpy() - xo) <= 1e-10 * np.linalg.norm(xo)
    # the multicolour order (Renumbering_Technique 1) takes another trajectory
    S.set("Renumbering_Technique", 1)
    info1 = LA.LinAlg_Solve(A, b, S, x)
    print(f"RCMK {info['iterations']} (oracle {its}), multicolour {info1['iterations']}")


@pytest.mark.parametrize("seed", range(8))
def test_rcmk_order_random_symmetric_patterns(seed):
    # random structurally symmetric patterns with a full diagonal, some in
    # several components and with isolated rows: the order equals the
    # restated cmkreord's permutation
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 400))
    m = int(rng.integers(0, 4 * n))
    i = rng.integers(0, n, m)
    j = rng.integers(0, n, m)
    if seed % 2:  # two diagonal blocks: no entry couples them
        cut = n // 2
        keep = (i < cut) == (j < cut)
        i, j = i[keep], j[keep]
    import scipy.sparse as sp
    S = sp.coo_matrix((np.ones(len(i)), (i, j)), shape=(n, n))
    S = (S + S.T + sp.eye(n)).tocsr()
    S.sort_indices()
    ip, ix = S.indptr.astype(np.int32), S.indices.astype(np.int32)
    got = _order(ip, ix)
    want = oracle.rcmk_new_of(ip, ix)
    assert np.array_equal(got, want)
