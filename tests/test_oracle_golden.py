"""The oracle (CPU restatement) against the reference's own outputs.

Fixtures come from the reference GetDP compiled from its sources; the
restatement must reproduce them bit for bit: DOF numbering (.pre records),
CSR pattern, every matrix and RHS value, the iteration count and the
solution of the Sparskit solve.
"""
import numpy as np
import pytest

import oracle
from getdp_gb300 import workloads as W
from tests import golden_cases as G


@pytest.mark.parametrize("name", G.names())
def test_dof_numbering_matches_pre(name):
    d, p, dm = G.load(name)
    pre = d["pre"]
    unk = pre[pre[:, 3] == 1]
    assert dm.n_dof == int(d["n"]) == len(unk)
    # every unknown DOF of the element tables is a NumDof of the .pre file
    got = np.unique(dm.elem_dofs[dm.elem_dofs >= 0])
    if dm.nharm == 2:
        got = np.unique(np.concatenate([got, got + 1]))
    assert np.array_equal(got, np.arange(dm.n_dof))
    assert np.array_equal(np.sort(unk[:, 4] - 1), np.arange(dm.n_dof))


@pytest.mark.parametrize("name", G.names())
def test_assembly_bit_exact(name):
    d, p, dm = G.load(name)
    ip, ix, dv, b = oracle.assemble(p, dm)
    assert np.array_equal(ip, d["indptr"])
    assert np.array_equal(ix, d["indices"])
    assert np.array_equal(dv, d["data"])
    assert np.array_equal(b, d["b"])


@pytest.mark.parametrize("name", G.names())
def test_solve_bit_exact(name):
    d, p, dm = G.load(name)
    ilu = "32" if name.endswith("ilu32") else "64"
    pr = oracle.params_from_golden(d["par_keys"], d["par_vals"])
    x, st, its, res = oracle.solve(d["indptr"], d["indices"], d["data"],
                                   d["b"], ilu=ilu, **pr)
    assert st == 0
    assert its == int(d["iterations"])
    assert np.array_equal(x, d["x"])


def test_edge_orientation_signs():
    p = W.curlcurl_edge(n=2, seed=1)
    dm = W.dofmap_for(p)
    e = p.mesh.elems[:, W.TET4_EDGES]
    assert np.array_equal(dm.elem_sign == 1, e[..., 0] < e[..., 1])


def test_zero_pivot_reported():
    # a matrix with a zero diagonal: ILU0 must stop with Sparskit's code
    ip = np.array([0, 2, 4], np.int32)
    ix = np.array([0, 1, 0, 1], np.int32)
    dv = np.array([0.0, 1.0, 1.0, 1.0])
    x, st, its, res = oracle.solve(ip, ix, dv, np.ones(2), renumbering=0)
    assert st == 101  # zero pivot at row 1
