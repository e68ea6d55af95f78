"""Golden fixtures for the post-processing step, from the reference GetDP.

Runs the reference (oracle/_ref, see make_golden.py) on the same seeded
problems as the solve fixtures, with a PostOperation that prints the curl
of the solution on every element and the field and its curl at seeded
interior points (Print[..., Format Table], Pos_Format.cpp), and stores the
printed values with the solution they were computed from.
Usage: python tests/golden/make_post_golden.py
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from getdp_gb300 import workloads as W  # noqa: E402
from make_golden import REF_BIN, read_res  # noqa: E402

CASES = [
    ("post_ms2d_n8", W.magnetostatics_2d, dict(n=8, seed=11), 2),
    ("post_eddy_n8", W.eddy_2d, dict(n=8, seed=41, freq=500.0), 2),
    ("post_cc_edge_n4", W.curlcurl_edge, dict(n=4, seed=31), 3),
    # fixed DOFs with values (workloads.DIRICHLET_SETS)
    ("post_ms2d_n8_dir", W.magnetostatics_2d, dict(n=8, seed=14, dirichlet=1), 2),
    ("post_eddy_n8_dir", W.eddy_2d, dict(n=8, seed=43, freq=500.0, dirichlet=1), 2),
]
PAR = "Algorithm 8\nPreconditioner 6\nKrylov_Size 50\nStopping_Test 1e-12\n" \
      "Nb_Iter_Max 5000\n"


def parse_table(path, nv, nvals):
    """Format Table lines: gmsh type, element number, nv node coordinates,
    3 dummies, then nvals numbers per line."""
    nums, coords, vals = [], [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            nums.append(int(t[1]))
            c = np.array([float(v) for v in t[2:2 + 3 * nv]]).reshape(nv, 3)
            coords.append(c)
            vals.append(np.array([float(v) for v in t[2 + 3 * nv + 3:]]))
            assert len(vals[-1]) == nvals, (path, len(vals[-1]), nvals)
    return np.array(nums), np.array(coords), np.array(vals)


def run(name, gen, kw, dim):
    p = gen(**kw)
    dm = W.dofmap_for(p)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    npts = 24
    pts = rng.uniform(0.03, 0.97, size=(npts, 3))
    if dim == 2:
        pts[:, 2] = 0.0
    tmp = tempfile.mkdtemp(prefix="postgolden_")
    W.prepare_regions(p)
    try:
        with open(os.path.join(tmp, "p.pro"), "w") as f:
            f.write(W.pro_text(p) + W.post_text(p, [tuple(q) for q in pts]))
        W.write_msh22(p.mesh, os.path.join(tmp, "p.msh"))
        with open(os.path.join(tmp, "solver.par"), "w") as f:
            f.write(PAR)
        cmd = [os.path.join(REF_BIN, "getdp_ilu64"), "p.pro", "-solve", "R", "-pos", "Map",
               "-msh", "p.msh", "-bin", "-v", "2"]
        out = subprocess.run(cmd, cwd=tmp, stdin=subprocess.DEVNULL, capture_output=True,
                             text=True, timeout=600)
        log = out.stdout + out.stderr
        if out.returncode != 0 and "E n d   P r o c e s s i n g" not in log:
            raise RuntimeError(f"{name}: reference failed\n{log[-3000:]}")
        nh = 2 if p.formulation == "eddy2d" else 1
        nv = p.mesh.elems.shape[1]
        x = read_res(os.path.join(tmp, "p.res"), dm.n_dof)
        en, ec, ev = parse_table(os.path.join(tmp, "post_elem.txt"), nv, nh * nv * 3)
        pn, pc, pa = parse_table(os.path.join(tmp, "post_pts.txt"), 1, nh * 3)
        _, _, pb = parse_table(os.path.join(tmp, "post_pts_b.txt"), 1, nh * 3)
        # element number k+1 is mesh element k (write_msh22 writes the
        # volume elements first): check it through the printed coordinates
        k = en - 1
        assert np.allclose(ec, p.mesh.nodes[p.mesh.elems[k]], atol=1e-14)
        assert np.allclose(pc[:, 0, :], pts)
        return dict(x=x, elem_index=k, elem_vals=ev.reshape(len(k), nh, nv, 3),
                    pts=pts, pts_elem=pn - 1, pts_a=pa.reshape(npts, nh, 3),
                    pts_b=pb.reshape(npts, nh, 3), n_dof=dm.n_dof)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main():
    only = set(sys.argv[1:])
    for name, gen, kw, dim in CASES:
        if only and name not in only:
            continue
        d = run(name, gen, kw, dim)
        d["gen_kw_keys"] = np.array(list(kw.keys()))
        d["gen_kw_vals"] = np.array([float(v) for v in kw.values()])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
        print(name, len(d["elem_index"]), "elements", len(d["pts"]), "points")


if __name__ == "__main__":
    main()
