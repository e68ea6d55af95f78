"""cell_aggregates: the aggregates of the two-level preconditioners (host)."""
import numpy as np
import pytest

from getdp_gb300 import workloads as W


def test_cell_aggregates_cover_every_unknown_once_and_follow_the_cells():
    p = W.nonlinear_2d(n=32, seed=5)
    dm = W.dofmap_for(p)
    agg, nc = W.cell_aggregates(p, dm, 4)
    assert agg.shape == (dm.n_dof,) and agg.dtype == np.int32
    assert nc == 16 and agg.min() == 0 and agg.max() == nc - 1
    counts = np.bincount(agg, minlength=nc)
    assert counts.min() > 0 and counts.sum() == dm.n_dof
    # an unknown's aggregate is the cell holding its node
    node_of = np.full(dm.n_dof, -1)
    m = dm.elem_dofs >= 0
    node_of[dm.elem_dofs[m]] = p.mesh.elems[m]
    xy = p.mesh.nodes[node_of, :2]
    cell = np.minimum((xy * 4).astype(int), 3)
    key = cell[:, 0] * 4 + cell[:, 1]
    for a in range(nc):
        assert len(np.unique(key[agg == a])) == 1


def test_cell_aggregates_drop_empty_cells_and_reject_vector_problems():
    p = W.nonlinear_2d(n=8, seed=5)
    dm = W.dofmap_for(p)
    agg, nc = W.cell_aggregates(p, dm, 64)   # more cells than nodes per side
    assert nc == len(np.unique(agg)) <= dm.n_dof
    assert np.array_equal(np.unique(agg), np.arange(nc))
    e = W.elasticity_p2(n=2, seed=2)
    with pytest.raises(ValueError):
        W.cell_aggregates(e, W.dofmap_for(e), 2)
