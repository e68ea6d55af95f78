"""Generate the golden fixtures in this directory from the reference GetDP.

Runs the reference GetDP 3.5.0, compiled from its own sources by
``oracle/build_ref.sh`` (into ``oracle/_ref``; unchanged kernel, parser, DOF
numbering, element loop, LinAlg_SPARSKIT.cpp and Sparskit.cpp, with the
Sparskit Fortran routines restated in ``oracle/sparskit_port.c``), on small
seeded instances of every workload, and stores for each:

* the DOF records of the ``.pre`` file (NumType, Entity, Harmonic, Type,
  NumDof) -- GetDP's own numbering;
* the assembled matrix, exact: ``Write[A]`` makes Sparskit
  dump its per-column linked lists in binary (Sparskit.cpp binary_write_matrix),
  which are turned into CSR here; plus the RHS as raw doubles;
* the solution (binary ``.res``) and the iteration count / residual that the
  solver reports, with the solver parameters used.

This script needs the reference sources and only runs in the development
container; the fixtures it writes are committed and travel with the tests.
Usage: python tests/golden/make_golden.py [case names...]   (default: all)
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

from getdp_gb300 import workloads as W  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref")

# (name, generator, kwargs, solver.par entries)
CASES = [
    ("ms2d_n8", W.magnetostatics_2d, dict(n=8, seed=11),
     dict(Algorithm=8, Preconditioner=6, Krylov_Size=50, Stopping_Test=1e-12,
          Nb_Iter_Max=2000, Renumbering_Technique=1)),
    ("ms2d_n24", W.magnetostatics_2d, dict(n=24, seed=12),
     dict(Algorithm=8, Preconditioner=6, Krylov_Size=50, Stopping_Test=1e-10,
          Nb_Iter_Max=2000, Renumbering_Technique=1)),
    ("ms2d_n24_norcm", W.magnetostatics_2d, dict(n=24, seed=12),
     dict(Algorithm=8, Preconditioner=6, Krylov_Size=20, Stopping_Test=1e-10,
          Nb_Iter_Max=2000, Renumbering_Technique=0)),
    ("el_p2_n2", W.elasticity_p2, dict(n=2, seed=21),
     dict(Algorithm=1, Preconditioner=0, Scaling=1, Stopping_Test=1e-10,
          Nb_Iter_Max=5000, Renumbering_Technique=1)),
    ("el_p2_n3", W.elasticity_p2, dict(n=3, seed=22),
     dict(Algorithm=1, Preconditioner=0, Scaling=1, Stopping_Test=1e-10,
          Nb_Iter_Max=5000, Renumbering_Technique=0)),
    ("cc_edge_n4", W.curlcurl_edge, dict(n=4, seed=31),
     dict(Algorithm=9, Preconditioner=6, Krylov_Size=40, Stopping_Test=1e-10,
          Nb_Iter_Max=5000, Renumbering_Technique=1)),
    ("eddy_n8", W.eddy_2d, dict(n=8, seed=41, freq=500.0),
     dict(Algorithm=8, Preconditioner=6, Krylov_Size=50, Stopping_Test=1e-10,
          Nb_Iter_Max=2000, Renumbering_Technique=1)),
    # non-homogeneous Dirichlet values (workloads.DIRICHLET_SETS)
    ("ms2d_n12_dir", W.magnetostatics_2d, dict(n=12, seed=13, dirichlet=1),
     dict(Algorithm=8, Preconditioner=6, Krylov_Size=50, Stopping_Test=1e-12,
          Nb_Iter_Max=2000, Renumbering_Technique=1)),
    ("el_p2_n2_dir", W.elasticity_p2, dict(n=2, seed=23, dirichlet=2),
     dict(Algorithm=1, Preconditioner=0, Scaling=1, Stopping_Test=1e-10,
          Nb_Iter_Max=5000, Renumbering_Technique=1)),
    ("eddy_n8_dir", W.eddy_2d, dict(n=8, seed=42, freq=500.0, dirichlet=1),
     dict(Algorithm=8, Preconditioner=6, Krylov_Size=50, Stopping_Test=1e-10,
          Nb_Iter_Max=2000, Renumbering_Technique=1)),
]


def read_list_matrix(path):
    """Sparskit binary_write_matrix: linked lists per column -> CSR.

    jptr[col] heads a list through ptr[]; ai[] holds the 1-based row of each
    entry (add_matrix_double(M, row, col) keys its lists on col,
    Sparskit.cpp:809-862)."""
    with open(path, "rb") as f:
        T = int(f.readline())
        assert T == 1, "sparse matrix expected"
        n, nb = map(int, f.readline().split())
        for _ in range(4):
            f.readline()
        ptr = np.frombuffer(f.read(4 * nb), np.int32)
        ai = np.frombuffer(f.read(4 * nb), np.int32)
        jptr = np.frombuffer(f.read(4 * n), np.int32)
        a = np.frombuffer(f.read(8 * nb), np.float64)
    rows, cols, vals = [], [], []
    for col in range(n):
        it = jptr[col]
        while it > 0:
            rows.append(ai[it - 1] - 1)
            cols.append(col)
            vals.append(a[it - 1])
            it = ptr[it - 1]
    rows = np.array(rows, np.int64)
    cols = np.array(cols, np.int64)
    vals = np.array(vals, np.float64)
    o = np.lexsort((cols, rows))
    rows, cols, vals = rows[o], cols[o], vals[o]
    indptr = np.zeros(n + 1, np.int64)
    np.add.at(indptr, rows + 1, 1)
    return n, np.cumsum(indptr).astype(np.int32), cols.astype(np.int32), vals


def read_pre(path):
    recs = []
    with open(path) as f:
        lines = f.read().splitlines()
    i = lines.index([l for l in lines if l.startswith("$DofData")][0])
    nrec = int(lines[i + 5].split()[0])
    for l in lines[i + 6:i + 6 + nrec]:
        t = l.split()
        numtype, ent, harm, typ = map(int, t[:4])
        numdof = int(t[4]) if typ == 1 else -1  # DOF_UNKNOWN = 1
        recs.append((numtype, ent, harm, typ, numdof))
    return np.array(recs, np.int64)


def read_res(path, n):
    with open(path, "rb") as f:
        data = f.read()
    k = data.index(b"$Solution")
    k = data.index(b"\n", k) + 1
    k = data.index(b"\n", k) + 1
    return np.frombuffer(data[k:k + 8 * n], np.float64).copy()


def run_case(name, gen, kw, par, exe="getdp_ilu64"):
    p = gen(**kw)
    tmp = tempfile.mkdtemp(prefix="golden_")
    try:
        W.write_pro(p, os.path.join(tmp, "p.pro"))
        W.write_msh22(p.mesh, os.path.join(tmp, "p.msh"))
        with open(os.path.join(tmp, "solver.par"), "w") as f:
            for k, v in par.items():
                f.write(f"{k} {v!r}\n" if isinstance(v, float) else f"{k} {v}\n")
        cmd = [os.path.join(REF_BIN, exe), "p.pro", "-solve", "R", "-msh",
               "p.msh", "-bin", "-v", "4"]
        out = subprocess.run(cmd, cwd=tmp, stdin=subprocess.DEVNULL,
                             capture_output=True, text=True, timeout=600)
        log = out.stdout + out.stderr
        # the reference can abort in its exit-time cleanup after every output
        # file is written ("double free" in some runs); accept a run that
        # reached the end of processing
        if out.returncode != 0 and "E n d   P r o c e s s i n g" not in log:
            raise RuntimeError(f"{name}: reference failed\n{log[-3000:]}")
        n, indptr, indices, data = read_list_matrix(os.path.join(tmp, "A.mat"))
        b = np.fromfile(os.path.join(tmp, "b.bin"), np.float64, count=n)
        x = read_res(os.path.join(tmp, "p.res"), n)
        pre = read_pre(os.path.join(tmp, "p.pre"))
        m = re.findall(r"(\d+) Iterations / Residual: (\S+)", log)
        its = int(m[-1][0]) if m else -1
        res = float(m[-1][1]) if m else -1.0
        return dict(n=n, indptr=indptr, indices=indices, data=data, b=b, x=x,
                    pre=pre, iterations=its, residual=res,
                    node_checksum=float(np.sum(p.mesh.nodes * np.arange(1, 4))),
                    par_keys=np.array(list(par.keys())),
                    par_vals=np.array([float(v) for v in par.values()]),
                    gen_kw_keys=np.array(list(kw.keys())),
                    gen_kw_vals=np.array([float(v) for v in kw.values()]),
                    exe=exe)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def main():
    if not os.path.exists(os.path.join(REF_BIN, "getdp_ilu64")):
        raise SystemExit("build the reference first: oracle/build_ref.sh")
    only = set(sys.argv[1:])
    for name, gen, kw, par in CASES:
        if only and name not in only:
            continue
        d = run_case(name, gen, kw, par)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
        print(f"{name}: n={d['n']} nnz={len(d['data'])} its={d['iterations']} "
              f"res={d['residual']:.3e}")
    # the FP32-ILU flavour (the official build's HAVE_ILU_FLOAT) on one case
    name, gen, kw, par = CASES[1]
    if only and name + "_ilu32" not in only:
        return
    d = run_case(name + "_ilu32", gen, kw, par, exe="getdp_ilu32")
    np.savez_compressed(os.path.join(HERE, f"{name}_ilu32.npz"), **d)
    print(f"{name}_ilu32: its={d['iterations']} res={d['residual']:.3e}")


if __name__ == "__main__":
    main()
