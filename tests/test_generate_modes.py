"""Generate's scatter modes and its pattern cache (GPU).

* Every mode (binary search + atomics, position table + atomics, colour by
  colour without atomics) matches the oracle within the per-entry bound of
  tests/tolerances.py, for every formulation.
* The coloured mode gives A and b identical to the last bit on every run.
* A Generate of the same element table into a new matrix (GetDP's
  ZeroMatrix destroys and recreates A before each Generate) reuses the
  context's cached pattern; a changed table is detected and rebuilt.
"""
import numpy as np
import pytest

import oracle
from getdp_gb300 import _lib
from getdp_gb300 import generate as G_
from getdp_gb300 import linalg as LA
from getdp_gb300 import workloads as W
from tests import tolerances as TOL

pytestmark = pytest.mark.gpu

MODES = [_lib.SCATTER_SEARCH, _lib.SCATTER_TABLE, _lib.SCATTER_COLOURED]
PROBLEMS = {
    "elasticity": lambda: W.elasticity_p2(6, seed=2),
    "elasticity_dir": lambda: W.elasticity_p2(4, seed=23, dirichlet=2),
    "magnetostatics": lambda: W.magnetostatics_2d(32, seed=1, dirichlet=1),
    "eddy": lambda: W.eddy_2d(16, seed=4, dirichlet=1),
    "curlcurl": lambda: W.curlcurl_edge(6, seed=3),
    "nonlinear": lambda: W.nonlinear_2d(32, seed=5),
}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from getdp_gb300 import build
    build.build()
    oracle.build()


def _gen(p, dm, mode, terms=None, A=None, solution=None):
    terms = terms or G_.DeviceTerms(p, dm)
    A = A or LA.gMatrix(dm.n_dof)
    b = LA.gVector(dm.n_dof)
    x = None
    if solution is not None:
        x = LA.gVector(dm.n_dof)
        x.set(solution)
    G_.generate(A, b, terms.batch, pattern=True, solution=x, scatter=mode)
    ip, ix, dv = A.csr()
    return terms, A, ip, ix, dv, b.numpy()


@pytest.mark.parametrize("name", sorted(PROBLEMS))
@pytest.mark.parametrize("mode", MODES)
def test_scatter_modes_match_oracle(name, mode):
    p = PROBLEMS[name]()
    dm = W.dofmap_for(p)
    sol = None
    if p.formulation == "nonlinear2d":
        sol = 0.3 * np.sin(np.arange(dm.n_dof) * 0.37)
    _, _, ip, ix, dv, bb = _gen(p, dm, mode, solution=sol)
    oip, oix, odv, ob, sabs, babs = oracle.assemble(p, dm, solution=sol, with_abs=True)
    assert np.array_equal(ip, oip) and np.array_equal(ix, oix)
    scale = TOL.matrix_scale(oip, oix, odv, sabs, p.formulation == "eddy2d")
    assert TOL.values_close(dv, odv, scale), TOL.report(dv, odv, scale)
    assert TOL.values_close(bb, ob, babs), TOL.report(bb, ob, babs)


@pytest.mark.parametrize("name", ["elasticity", "nonlinear", "curlcurl", "eddy"])
def test_coloured_scatter_is_reproducible(name):
    p = PROBLEMS[name]()
    dm = W.dofmap_for(p)
    sol = 0.3 * np.sin(np.arange(dm.n_dof) * 0.37) if p.formulation == "nonlinear2d" else None
    terms, A, ip, ix, dv1, b1 = _gen(p, dm, _lib.SCATTER_COLOURED, solution=sol)
    for _ in range(3):
        _, _, _, _, dv2, b2 = _gen(p, dm, _lib.SCATTER_COLOURED, terms=terms, A=A,
                                   solution=sol)
        assert np.array_equal(dv1, dv2) and np.array_equal(b1, b2)


def test_pattern_cache_reused_and_invalidated():
    p = W.elasticity_p2(5, seed=2)
    dm = W.dofmap_for(p)
    terms, A1, ip1, ix1, dv1, _ = _gen(p, dm, _lib.SCATTER_DEFAULT)
    # a new matrix, the same table: the cached pattern
    A2 = LA.gMatrix(dm.n_dof)
    _, _, ip2, ix2, dv2, _ = _gen(p, dm, _lib.SCATTER_DEFAULT, terms=terms, A=A2)
    assert np.array_equal(ip1, ip2) and np.array_equal(ix1, ix2)
    oip, oix, odv, ob, sabs, babs = oracle.assemble(p, dm, with_abs=True)
    scale = TOL.matrix_scale(oip, oix, odv, sabs)
    assert TOL.values_close(dv2, odv, scale)
    # another mesh of the same size class: a different table, a new pattern
    q = W.elasticity_p2(4, seed=2)
    dq = W.dofmap_for(q)
    _, _, ipq, ixq, dvq, bq = _gen(q, dq, _lib.SCATTER_DEFAULT)
    qip, qix, qdv, qb, qs, qbs = oracle.assemble(q, dq, with_abs=True)
    assert np.array_equal(ipq, qip) and np.array_equal(ixq, qix)
    assert TOL.values_close(dvq, qdv, TOL.matrix_scale(qip, qix, qdv, qs))
    # a same-size table with one element's unknowns permuted: detected
    dm2 = W.dofmap_for(p)
    dm2.elem_dofs = dm2.elem_dofs.copy()
    e = 7
    dm2.elem_dofs[e, [0, 1]] = dm2.elem_dofs[e, [1, 0]]
    dm2.elem_dofs[e, [10, 11]] = dm2.elem_dofs[e, [11, 10]]
    dm2.elem_dofs[e, [20, 21]] = dm2.elem_dofs[e, [21, 20]]
    _, _, ip3, ix3, dv3, b3 = _gen(p, dm2, _lib.SCATTER_DEFAULT)
    rip, rix, rdv, rb, rs, rbs = oracle.assemble(p, dm2, with_abs=True)
    assert np.array_equal(ip3, rip) and np.array_equal(ix3, rix)
    assert TOL.values_close(dv3, rdv, TOL.matrix_scale(rip, rix, rdv, rs))


def test_coloured_scatter_needs_a_generated_pattern():
    p = W.magnetostatics_2d(8, seed=1)
    dm = W.dofmap_for(p)
    ip, ix, dv, bb = oracle.assemble(p, dm)
    A = LA.gMatrix(dm.n_dof)
    A.set_csr(ip, ix, dv)
    b = LA.gVector(dm.n_dof)
    terms = G_.DeviceTerms(p, dm)
    with pytest.raises(_lib.GetDPError):
        G_.generate(A, b, terms.batch, pattern=False, scatter=_lib.SCATTER_COLOURED)


@pytest.mark.parametrize("name,gen", [
    ("elasticity", lambda: W.elasticity_p2(16, seed=2)),
    ("magnetostatics", lambda: W.magnetostatics_2d(96, seed=1)),
    ("curlcurl", lambda: W.curlcurl_edge(16, seed=3)),
    ("nonlinear", lambda: W.nonlinear_2d(96, seed=5)),
])
def test_tuned_launch_shape_matches_oracle(name, gen):
    # batches of >= 16,384 elements get their launch shape from the tuner
    # (lanes per element, threads per CTA), chosen once per pattern among the
    # shapes whose result agrees with the warp-per-element kernel's
    p = gen()
    dm = W.dofmap_for(p)
    assert p.mesh.n_elems >= 16384
    sol = 0.3 * np.sin(np.arange(dm.n_dof) * 0.37) if p.formulation == "nonlinear2d" else None
    terms = G_.DeviceTerms(p, dm)
    for _ in range(2):  # the first Generate builds the pattern, the second tunes
        _, _, ip, ix, dv, bb = _gen(p, dm, _lib.SCATTER_DEFAULT, terms=terms, solution=sol)
    oip, oix, odv, ob, sabs, babs = oracle.assemble(p, dm, solution=sol, with_abs=True)
    assert np.array_equal(ip, oip) and np.array_equal(ix, oix)
    scale = TOL.matrix_scale(oip, oix, odv, sabs)
    assert TOL.values_close(dv, odv, scale), TOL.report(dv, odv, scale)
    assert TOL.values_close(bb, ob, babs), TOL.report(bb, ob, babs)
