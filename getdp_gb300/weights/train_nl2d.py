"""Trains the learned correction's network on Newton Jacobians of the
nonlinear 2D magnetostatic problem (saturating B-H law, lognormal
reluctivity field, 8 current blobs) and saves its weights.

    python -m getdp_gb300.weights.train_nl2d --n 256 --seeds 20 \
        --out getdp_gb300/weights/mpnn_nl2d_256.npy

For every seed, the Newton loop runs with the plain FP64 ILU(0)-GMRES(50)
to 1e-10; each step's Jacobian, right-hand side and solution become one
training system (r1 = b - A ILU^-1 b, e1 = x* - ILU^-1 b) plus two random
probes.  Training is Adam on the GPU with the network's own forward and
backward kernels.

With --two-level CELLS the correction is trained for the two-level cycle
(Preconditioner 22): the Newton solves use the two-level cycle with plain
ILU(0) (Preconditioner 21) on cells of CELLS per side, every training
system carries those aggregates, the probes are random errors e0 with
b = A e0 (so that r1 = A e1 exactly), and the loss is the energy of the
error left after the coarse correction (gb300_mpnn_set_loss mode 1):

    python -m getdp_gb300.weights.train_nl2d --n 256 --seeds 165 \
        --two-level 8 --out getdp_gb300/weights/mpnn_nl2d_256_twolevel.npy

With --smoother g, G is trained to stand alone as the smoother of the
cycle (Preconditioner 24: z = G v, no ILU(0)): the samples skip the ILU(0)
step (r1 = b, e1 = x*).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from .. import generate as G
from .. import learned as LR
from .. import linalg as LA
from .. import nonlinear as NL
from .. import workloads as W

RELAX = (1.0, 0.5, 0.25, 0.125, 0.0625, 0.03125)


def plain_fp64(precond: int = 6):
    S = LA.LinAlg_CreateSolver(None)
    for k, v in dict(Algorithm=8, Preconditioner=precond, Krylov_Size=50,
                     Nb_Iter_Max=20000, Renumbering_Technique=1, Precision=0).items():
        S.set(k, v)
    S["stopping_test"] = 1e-10
    return S


def dataset(n: int, seeds: int, probes: int = 2, first_seed: int = 200,
            cells: int = 0, ilu: bool = True):
    """(samples, number of Newton systems among them); cells > 0: the
    systems carry aggregates of cells per side (two-level training)"""
    samples = []
    systems = [0]
    for s in range(seeds):
        p = W.nonlinear_2d(n=n, seed=first_seed + s)
        dm = W.dofmap_for(p)
        terms = G.DeviceTerms(p, dm)
        agg = nc = None
        if cells:
            agg, nc = W.cell_aggregates(p, dm, cells)

        def keep(A, b, x):
            if cells:
                A.set_aggregates(agg, nc)
            info = LA.LinAlg_Solve(A, b, plain_fp64(21 if cells else 6), x)
            Ac, bc, xc = LR.copy_matrix(A), LR.copy_vector(b), LR.copy_vector(x)
            if cells:
                Ac.set_aggregates(agg, nc)
            samples.append(LR.make_sample(Ac, bc, xc, ilu=ilu))
            systems[0] += 1
            if cells:  # the two-level loss needs r1 = A e1 exactly
                samples.extend(LR.make_error_probes(Ac, probes, seed=5000 + len(samples),
                                                    ilu=ilu))
            else:
                samples.extend(LR.make_probes(Ac, probes, seed=5000 + len(samples)))
            return info

        NL.newton(terms, dm.n_dof, keep, tol_rel=1e-8, iter_max=50, relaxation=RELAX)
    return samples, systems[0]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--seeds", type=int, default=20)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--probes", type=int, default=2,
                    help="random probes per Newton system")
    ap.add_argument("--two-level", type=int, default=0, metavar="CELLS",
                    help="train for the two-level cycle on CELLS x CELLS aggregates")
    ap.add_argument("--smoother", choices=["ilu", "g"], default="ilu",
                    help="two-level: train G after the ILU(0) step (Preconditioner 22) "
                         "or standing alone (24)")
    ap.add_argument("--out", required=True)
    a = ap.parse_args()
    t0 = time.time()
    samples, systems = dataset(a.n, a.seeds, probes=a.probes, cells=a.two_level,
                               ilu=a.smoother == "ilu")
    t1 = time.time()
    net = LR.MPNN(seed=1)
    if a.two_level:
        net.set_loss(1)
    hist = LR.train(net, samples, epochs=a.epochs, lr=3e-3, batch=8)
    np.save(a.out, net.params())
    print(json.dumps({"n": a.n, "seeds": a.seeds, "two_level_cells": a.two_level,
                      "probes": a.probes, "smoother": a.smoother,
                      "skipped_per_run": getattr(net, "skipped", 0),
                      "systems": systems,
                      "samples": len(samples), "data_s": round(t1 - t0, 1),
                      "train_s": round(time.time() - t1, 1),
                      "loss": [round(h, 4) for h in hist]}))


if __name__ == "__main__":
    main()
