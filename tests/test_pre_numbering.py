"""DOF numbering (GetDP's pre-processing, DofData.cpp:1279-1319; edges
GeoEntity.cpp:436-485) entity by entity against the reference's .pre
records: for every (NumType, Entity, Harmonic), the unknown number (or
fixed) our element tables give equals the reference's, on the golden cases
and, where the reference binary is built, on large meshes (with the time
each side takes)."""
import os
import subprocess
import sys
import tempfile
import time

import numpy as np
import pytest

from getdp_gb300 import workloads as W
from tests import golden_cases as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref", "getdp_ilu64")


def our_records(p, dm):
    """(numtype, entity, harmonic, numdof or -1) for every DOF the element
    tables touch."""
    m = p.mesh
    f = p.formulation
    # a fixed DOF is -1 in the .pre comparison (with Dirichlet values the
    # tables number fixed DOFs -1-k)
    edofs = np.where(dm.elem_dofs >= 0, dm.elem_dofs, -1)
    if f in ("magnetostatics2d", "nonlinear2d", "eddy2d"):
        ent = m.elems + 1
        nt = np.ones_like(ent)
        d = edofs
        recs = [np.stack([nt.ravel(), ent.ravel(), np.zeros(ent.size, np.int64),
                          d.ravel()], 1)]
        if f == "eddy2d":
            d1 = np.where(d >= 0, d + 1, -1)
            recs.append(np.stack([nt.ravel(), ent.ravel(), np.ones(ent.size, np.int64),
                                  d1.ravel()], 1))
        r = np.concatenate(recs)
    elif f == "elasticity":
        nv = m.elems.shape[1]
        ent = np.tile(m.elems + 1, (1, 3))
        nt = np.repeat(np.arange(1, 4), nv)[None, :].repeat(m.n_elems, 0)
        r = np.stack([nt.ravel(), ent.ravel(), np.zeros(ent.size, np.int64),
                      edofs.ravel()], 1)
    elif f == "curlcurl":
        ve = m.elems[:, W.TET4_EDGES].reshape(-1, 2)
        nn = m.n_nodes
        key = np.minimum(ve[:, 0], ve[:, 1]).astype(np.int64) * nn + np.maximum(ve[:, 0], ve[:, 1])
        ekey = dm.edges[:, 0].astype(np.int64) * nn + dm.edges[:, 1]
        order = np.argsort(ekey)
        ent = order[np.searchsorted(ekey[order], key)] + 1
        r = np.stack([np.ones(len(ent), np.int64), ent, np.zeros(len(ent), np.int64),
                      edofs.ravel()], 1)
    else:
        raise ValueError(f)
    return np.unique(r.astype(np.int64), axis=0)


def check_against_pre(p, dm, pre):
    ours = our_records(p, dm)
    ref = pre[:, [0, 1, 2, 4]].copy()
    ref[:, 3] = np.where(pre[:, 3] == 1, pre[:, 4] - 1, -1)  # 0-based, fixed -1
    ref = np.unique(ref, axis=0)
    # every DOF touched by an element is in the .pre file with our number
    keys_o = ours[:, :3]
    keys_r = ref[:, :3]
    assert len(np.unique(keys_o, axis=0)) == len(keys_o), "one number per DOF"
    idx = {tuple(k): v for k, v in zip(map(tuple, keys_r), ref[:, 3])}
    mism = [(tuple(k), v, idx.get(tuple(k))) for k, v in zip(keys_o, ours[:, 3])
            if idx.get(tuple(k), "missing") != v]
    assert not mism, mism[:5]
    assert len(keys_o) == len(keys_r)


@pytest.mark.parametrize("name", G.names())
def test_numbering_entity_by_entity(name):
    d, p, dm = G.load(name)
    check_against_pre(p, dm, d["pre"])


@pytest.mark.skipif(not os.path.exists(REF), reason="reference binary not built")
@pytest.mark.parametrize("gen,kw", [(W.magnetostatics_2d, dict(n=256, seed=1)),
                                    (W.curlcurl_edge, dict(n=16, seed=3)),
                                    (W.eddy_2d, dict(n=96, seed=4))])
def test_numbering_large_against_reference_pre(gen, kw):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_golden import read_pre
    p = gen(**kw)
    t0 = time.perf_counter()
    dm = W.dofmap_for(p)
    t_ours = time.perf_counter() - t0
    with tempfile.TemporaryDirectory() as tmp:
        W.write_pro(p, os.path.join(tmp, "p.pro"))
        W.write_msh22(p.mesh, os.path.join(tmp, "p.msh"))
        t0 = time.perf_counter()
        r = subprocess.run([REF, "p.pro", "-pre", "R", "-msh", "p.msh", "-v", "2"], cwd=tmp,
                           stdin=subprocess.DEVNULL, capture_output=True, text=True,
                           timeout=900)
        t_ref = time.perf_counter() - t0
        assert os.path.exists(os.path.join(tmp, "p.pre")), r.stdout[-2000:] + r.stderr[-2000:]
        pre = read_pre(os.path.join(tmp, "p.pre"))
    check_against_pre(p, dm, pre)
    print(f"{p.name}: {dm.n_dof} unknowns, numbering {t_ours:.3f} s here, "
          f"reference pre-processing {t_ref:.2f} s (incl. reading the mesh)")
