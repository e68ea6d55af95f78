"""Shared loader for the golden fixtures made by tests/golden/make_golden.py."""
import glob
import os

import numpy as np

from getdp_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_GEN = {"ms2d": W.magnetostatics_2d, "el": W.elasticity_p2,
        "cc": W.curlcurl_edge, "eddy": W.eddy_2d}


def names():
    """The solve fixtures (post-processing and Newton fixtures are
    post_*.npz and newton_*.npz)."""
    return sorted(os.path.basename(f)[:-4]
                  for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(f).startswith(("post_", "newton_")))


def load(name):
    """(fixture dict, regenerated Problem, DofMap)."""
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    kw = {str(k): (float(v) if k == "freq" else int(v))
          for k, v in zip(d["gen_kw_keys"], d["gen_kw_vals"])}
    p = _GEN[name.split("_")[0]](**kw)
    assert abs(float(np.sum(p.mesh.nodes * np.arange(1, 4))) -
               float(d["node_checksum"])) < 1e-9, "mesh generator drifted"
    return d, p, W.dofmap_for(p)
