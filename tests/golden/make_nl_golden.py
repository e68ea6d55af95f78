"""Golden fixtures for the nonlinear (Newton) path, from the reference GetDP.

Runs the reference (oracle/_ref, see make_golden.py) on seeded small
instances of the nonlinear 2D magnetostatic problem with the Newton loop of
templates/Lib_Magnetostatics_a_phi.pro, and stores the first Generate's
matrix and RHS (at the zero initial solution), the residual history
printed by GetResidual, the linear iteration counts, and the final
solution.  Usage: python tests/golden/make_nl_golden.py
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from getdp_gb300 import workloads as W  # noqa: E402
from make_golden import REF_BIN, read_list_matrix, read_pre, read_res  # noqa: E402

CASES = [("nl2d_n12", dict(n=12, seed=5)), ("nl2d_n16", dict(n=16, seed=7))]
PAR = dict(Algorithm=8, Preconditioner=6, Krylov_Size=50, Stopping_Test=1e-13,
           Nb_Iter_Max=5000, Renumbering_Technique=1)


def run(name, kw):
    p = W.nonlinear_2d(**kw)
    tmp = tempfile.mkdtemp(prefix="nlgolden_")
    try:
        W.write_pro(p, os.path.join(tmp, "p.pro"))
        W.write_msh22(p.mesh, os.path.join(tmp, "p.msh"))
        with open(os.path.join(tmp, "solver.par"), "w") as f:
            for k, v in PAR.items():
                f.write(f"{k} {v!r}\n" if isinstance(v, float) else f"{k} {v}\n")
        cmd = [os.path.join(REF_BIN, "getdp_ilu64"), "p.pro", "-solve", "R", "-msh",
               "p.msh", "-bin", "-v", "4"]
        out = subprocess.run(cmd, cwd=tmp, stdin=subprocess.DEVNULL, capture_output=True,
                             text=True, timeout=600)
        log = out.stdout + out.stderr
        if out.returncode != 0 and "E n d   P r o c e s s i n g" not in log:
            raise RuntimeError(f"{name}: reference failed\n{log[-3000:]}")
        n, indptr, indices, data = read_list_matrix(os.path.join(tmp, "A.mat"))
        b = np.fromfile(os.path.join(tmp, "b.bin"), np.float64, count=n)
        x = read_res(os.path.join(tmp, "p.res"), n)
        hist = np.array([float(v) for v in
                         re.findall(r"Residual \d+: abs (\S+) rel", log)])
        its = np.array([int(v) for v in re.findall(r"(\d+) Iterations / Residual", log)])
        return dict(n=n, indptr=indptr, indices=indices, data=data, b=b, x=x,
                    pre=read_pre(os.path.join(tmp, "p.pre")), history=hist,
                    linear_iterations=its,
                    par_keys=np.array(list(PAR.keys())),
                    par_vals=np.array([float(v) for v in PAR.values()]),
                    gen_kw_keys=np.array(list(kw.keys())),
                    gen_kw_vals=np.array([float(v) for v in kw.values()]),
                    node_checksum=float(np.sum(p.mesh.nodes * np.arange(1, 4))))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main():
    for name, kw in CASES:
        d = run(name, kw)
        np.savez_compressed(os.path.join(HERE, f"newton_{name}.npz"), **d)
        print(name, "n", d["n"], "newton steps", len(d["history"]) - 1,
              "final rel", d["history"][-1] / d["history"][0])


if __name__ == "__main__":
    main()
