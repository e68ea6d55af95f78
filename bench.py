#!/usr/bin/env python
"""Headline benchmark: Generate + Solve of GetDP's 3D P2 elasticity case.

Workload: unit cube of n^3 hexes x 6 Kuhn tets
with 10-node (P2) elements, n = 48: 663,552 tets, 2,709,792 unknowns,
~229 M nonzeros; per-element lognormal Young's modulus, Poisson 0.3,
gravity load, face x = 0 clamped; 4-point Gauss.  Solve: Jacobi-scaled CG
(Sparskit Algorithm 1, Scaling 1, Preconditioner 0) to a relative FP64
residual of 1e-8 on the scaled system.

One step = Generate[A] (CSR pattern + all element matrices, from element
tables resident in HBM) + Solve[A] with FP32-SpMV CG inside FP64 reliable
updates.  `value` = seconds per step (lower is better).  `e2e` = the same
step through the public API with the element tables copied from pinned host
memory and the solution copied back.  The plain FP64 GPU solve is timed once
beside it.  Inputs (2.8 GB of CSR) exceed L2 (129 MB), so no L2 flush is
used between steps.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("time to 1e-8 FP64 residual (Generate + Solve), 3D P2 elasticity, "
          "mixed FP32/FP64 GPU solve")
UNIT = "s"

# The reference arm's full FP64 solution of the headline system is kept here
# (keyed by size and seed) so that the GPU arm, run next on the same host,
# can state its solutions' error against it.
ORACLE_SOLUTION = os.path.join(tempfile.gettempdir(),
                               "getdp_gb300_oracle_elasticity_n{n}_seed2.npz")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", "--size", dest="n", type=int, default=None,
                    help="cells per side (default: the workload's own size); "
                         "--size is the spelling torchrun passes through")
    ap.add_argument("--workload", default="elasticity",
                    choices=["elasticity", "magnetostatics2d", "curlcurl", "eddysweep",
                             "nonlinear", "io"],
                    help="elasticity: 3D P2 elasticity, Jacobi-CG (the headline); "
                         "magnetostatics2d: 2D P1 a_z, ILU(0)-GMRES(50) to 1e-10; "
                         "curlcurl: 3D Whitney-edge curl-curl, ILU(0)-FGMRES(40) "
                         "to 1e-8, FP64 and FP32-ILU; eddysweep: 512 complex 2D "
                         "eddy-current problems of 32^2..160^2 cells in one batched "
                         "Generate + batched ILU(0)-GMRES; io: the host steps either "
                         "side of the path (MSH 2.2 read, numbering, .pre/.res write)")
    ap.add_argument("--cpu-n", type=int, default=128,
                    help="nonlinear: mesh size of the CPU (oracle) comparison run")
    ap.add_argument("--problems", type=int, default=512,
                    help="eddysweep: number of problems")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 comparison solve (profiling runs)")
    ap.add_argument("--batch-kernel", type=int, default=4,
                    help="--profile sweep: Batch_Kernel of the batched solve")
    ap.add_argument("--profile", choices=["spmv32", "spmv64", "generate", "step", "twolevel",
                                          "sweep",
                                          "mpnn"],
                    help="minimal run for ncu: one Generate, then 3 warm-up "
                         "and 3 timed launches of the chosen kernel; 'step': "
                         "one warm-up step, then one Generate + mixed solve "
                         "capped at --profile-iterations CG iterations; "
                         "'twolevel': nonlinear 2D magnetostatics, two solves "
                         "with the two-level cycle; 'mpnn': three inferences of "
                         "the learned correction on that system")
    ap.add_argument("--profile-iterations", type=int, default=64)
    ap.add_argument("--coarse-cells", type=int, default=32,
                    help="nonlinear: cells per side of the aggregates of the two-level "
                         "preconditioner (Preconditioner 21); 0: aggregates from the "
                         "matrix graph")
    ap.add_argument("--two-level-only", action="store_true",
                    help="nonlinear workload: only the two-level (and learned) arms")
    ap.add_argument("--learned-two-level-weights", default=None,
                    help="nonlinear workload: also time the Newton loop with the correction "
                         "trained for the two-level cycle (Preconditioner 22, .npy)")
    ap.add_argument("--learned-weights", default=None,
                    help="nonlinear workload: also time the Newton loop with the learned "
                         "correction (network weights, .npy)")
    return ap.parse_args()


def profile_run(args):
    """The smallest program that runs the kernel under study (for ncu)."""
    from getdp_gb300 import _lib
    from getdp_gb300 import generate as G
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import workloads as W
    L = _lib.load(build_if_missing=True)
    if args.profile == "mpnn":
        # the learned correction's inference (3 message-passing layers and
        # the output head) on the nonlinear 2D system at a = 0, three times
        from getdp_gb300 import learned as LR
        n = args.n or 1024
        p = W.nonlinear_2d(n=n, seed=5)
        dm = W.dofmap_for(p)
        terms = G.DeviceTerms(p, dm)
        A, b = LA.gMatrix(dm.n_dof), LA.gVector(dm.n_dof)
        G.generate(A, b, terms.batch, pattern=True)
        net = LR.MPNN(seed=1)
        net.set_params(np.load(os.path.join(ROOT, "getdp_gb300", "weights",
                                            "mpnn_nl2d_256_twolevel.npy")))
        for _ in range(3):
            net.infer(A)
        print(json.dumps({"profile": "mpnn", "n": n, "nnz": A.nnz()}))
        return
    if args.profile == "sweep":
        # a small batched sweep (64 complex eddy-current problems of 16^2 to
        # 48^2 cells), solved twice in the one-launch cluster form (FP64
        # factor, GMRES(40)); the second solve is the one to capture
        probs = W.eddy_sweep(n_problems=64, seed=7, n_min=16, n_max=48)
        bt = W.concat_problems(probs)
        N = bt.dofmap.n_dof
        terms = G.DeviceTerms(bt.problem, bt.dofmap)
        A, b, x = LA.gMatrix(N), LA.gVector(N), LA.gVector(N)
        G.generate(A, b, terms.batch, pattern=True)
        S = LA.LinAlg_CreateSolver(None)
        for k, v in dict(Algorithm=8, Preconditioner=6, Krylov_Size=40, Nb_Iter_Max=5000,
                         Renumbering_Technique=1, Batch_Kernel=args.batch_kernel).items():
            S.set(k, v)
        S["stopping_test"] = 1e-10
        for _ in range(2):
            infos = LA.LinAlg_SolveBatch(A, b, S, x, bt.offsets)
        its = [d["iterations"] for d in infos]
        print(json.dumps({"profile": "sweep", "problems": len(probs), "unknowns": N,
                          "iterations_min_median_max": [min(its), int(np.median(its)),
                                                        max(its)],
                          "one_launch_form": all(d["batch_form"] == 1 for d in infos)}))
        return
    if args.profile == "twolevel":
        # nonlinear 2D magnetostatics at a = 0: one Generate, then two
        # solves with the two-level cycle (the first makes the colouring,
        # the aggregates and the graphs)
        n = args.n or 1024
        p = W.nonlinear_2d(n=n, seed=5)
        dm = W.dofmap_for(p)
        terms = G.DeviceTerms(p, dm)
        A, b, x = LA.gMatrix(dm.n_dof), LA.gVector(dm.n_dof), LA.gVector(dm.n_dof)
        G.generate(A, b, terms.batch, pattern=True)
        agg, nc = W.cell_aggregates(p, dm, args.coarse_cells)
        A.set_aggregates(agg, nc)
        S = LA.LinAlg_CreateSolver(None)
        for k, v in dict(Algorithm=8, Preconditioner=21, Krylov_Size=50, Nb_Iter_Max=20000,
                         Renumbering_Technique=1).items():
            S.set(k, v)
        S["stopping_test"] = 1e-10
        for _ in range(2):
            info = LA.LinAlg_Solve(A, b, S, x)
        print(json.dumps({"profile": "twolevel", "n": n, "aggregates": nc,
                          "iterations": info["iterations"]}))
        return
    p = W.elasticity_p2(n=args.n, seed=2)
    dm = W.dofmap_for(p)
    terms = G.DeviceTerms(p, dm)
    A = LA.gMatrix(dm.n_dof)
    b = LA.gVector(dm.n_dof)
    G.generate(A, b, terms.batch, pattern=True)
    if args.profile == "generate":
        G.generate(A, b, terms.batch, pattern=True)
        print(json.dumps({"profile": "generate", "n": args.n, "nnz": A.nnz()}))
        return
    if args.profile == "step":
        x = LA.gVector(dm.n_dof)
        S = solver_params(True, args.profile_iterations)
        for _ in range(2):  # the first step also tunes the SpMV
            G.generate(A, b, terms.batch, pattern=True)
            info = LA.LinAlg_Solve(A, b, S, x)
        print(json.dumps({"profile": "step", "n": args.n, "nnz": A.nnz(),
                          "iterations": info["iterations"]}))
        return
    ms = ctypes.c_double()
    prec = 1 if args.profile == "spmv32" else 0
    _lib.check(L.gb300_bench_spmv(A.h, prec, 3, ctypes.byref(ms)))
    print(json.dumps({"profile": args.profile, "n": args.n, "nnz": A.nnz(),
                      "launch_ms": ms.value}))


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "gb300":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:  # the reference arm runs on the host cores only
            dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def solver_params(mixed: bool, n_iter_max: int = 200000):
    from getdp_gb300 import linalg as LA
    S = LA.LinAlg_CreateSolver(None)
    S.set("Algorithm", 1)
    S.set("Preconditioner", 0)
    S.set("Scaling", 1)
    S.set("Stopping_Test", "1e-8")
    S.set("Nb_Iter_Max", n_iter_max)
    S.set("Precision", 1 if mixed else 0)
    # the value is read through a float like the reference; store 1e-8 exactly
    S["stopping_test"] = 1e-8
    return S


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            t = [x.strip() for x in line.split(",")]
            if len(t) >= 9:
                rows.append(t)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        out.update(sm_mhz=statistics.median(sm) if sm else None,
                   sm_max_mhz=max(mx) if mx else None, reasons=sorted(reasons),
                   samples=len(rows))
        return out


# FP64 operations per element of the P2 elasticity element kernel, counted by
# ncu on the GPU (2 DFMA + DADD + DMUL thread instructions, active lanes only;
# profiles/tet10_elasticity_values_n32.md); bytes per element as the
# algorithmic minimum (connectivity 40 B, coordinates 33 B, coefficient 4 B,
# the CSR values written once 8 nnz / E, the RHS 8 N / E)
TET10_FP64_FLOPS_PER_ELEMENT = 10970


def assembly_roofline(ne, n, nnz, t, fp64_tflops, hbm_gbs):
    """Generate (cached pattern: table comparison, zeroing, element kernel)
    against the FP64 pipe (measured FMA peak) and HBM (measured copy)."""
    flops = TET10_FP64_FLOPS_PER_ELEMENT * ne
    bytes_ = ne * (40 + 4) + (n // 3) * 24 + 8 * nnz + 8 * n
    ach = flops / t / 1e12
    gbs = bytes_ / t / 1e9
    return {"bound": "fp64", "unit": "TFLOP/s", "achieved": ach, "peak": fp64_tflops,
            "frac": ach / fp64_tflops, "peak_kind": "measured (gb300_bench_fp64_peak)",
            "flops_per_element": TET10_FP64_FLOPS_PER_ELEMENT,
            "algorithmic_bytes": bytes_, "achieved_gbs": gbs, "hbm_frac": gbs / hbm_gbs,
            "generate_s": t, "elements": ne}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU (oracle port) baseline on bounded samples
# ---------------------------------------------------------------------------
def cpu_baseline(n: int, A_csr=None, b=None, iterations=None):
    """Time the restated reference path on the host: the element loop on a
    sample mesh (per element), and Sparskit's CG on the full system for a
    few iterations (per iteration); extrapolate to the full workload."""
    import oracle
    from getdp_gb300 import workloads as W
    oracle.build()
    ns = 12
    ps = W.elasticity_p2(n=ns, seed=2)
    dms = W.dofmap_for(ps)
    t0 = time.perf_counter()
    ip, ix, dv, bb = oracle.assemble(ps, dms)
    t_asm = time.perf_counter() - t0
    per_elem = t_asm / ps.mesh.n_elems
    n_elems = 6 * n ** 3
    sample = {"assembly_sample_elements": ps.mesh.n_elems,
              "assembly_seconds": round(t_asm, 3)}
    per_iter = None
    if A_csr is not None:
        ip, ix, dv = A_csr
        t0 = time.perf_counter()
        oracle.solve(ip, ix, dv, b, algorithm=1, preconditioner=0, scaling=1,
                     renumbering=0, nb_iter_max=2, stopping_test=1e-8)
        t2 = time.perf_counter() - t0
        t0 = time.perf_counter()
        oracle.solve(ip, ix, dv, b, algorithm=1, preconditioner=0, scaling=1,
                     renumbering=0, nb_iter_max=6, stopping_test=1e-8)
        t6 = time.perf_counter() - t0
        per_iter = max((t6 - t2) / 4.0, 1e-9)
        setup = max(t2 - 2 * per_iter, 0.0)
        sample.update(cg_iterations_timed=6, cg_seconds_2=round(t2, 3),
                      cg_seconds_6=round(t6, 3))
    else:
        setup = 0.0
    total = per_elem * n_elems
    if per_iter is not None and iterations:
        total += setup + per_iter * iterations
    return total, per_elem, per_iter, sample


def host_cpu():
    """The host CPU's model name and core count (lscpu, else /proc/cpuinfo)."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.lower().startswith(("model name", "cpu model")):
                        model = line.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"model": model or "unknown", "host_cores": os.cpu_count() or 1,
            "machine": platform.machine()}


def pin_one_core():
    """Run the single-threaded reference path on one core (as taskset would),
    so that the measurement does not move between cores; returns the core."""
    try:
        core = min(os.sched_getaffinity(0))
        os.sched_setaffinity(0, {core})
        return core
    except (AttributeError, OSError):
        return None


def _rhs_checksum(b):
    b = np.asarray(b, np.float64)
    return float(np.dot(b, np.arange(1, len(b) + 1, dtype=np.float64) % 97.0))


def run_reference(args, ws, rank):
    """--impl reference: the reference's CPU path for the headline workload,
    measured in full once -- the restated element loop over every element
    (Generate) and Sparskit's Jacobi-CG with the reference's defaults
    (Scaling 1, RCMK renumbering) to 1e-8 on the full system, on one host
    core (the reference path is single-threaded).  That measured time is
    `value`.  The warm-up and timed steps then time bounded samples of the
    same work (the element loop on a 12^3 sub-mesh, 6 CG iterations on the
    full system), extrapolated with the full solve's own iteration count, as
    a cross-check.  The FP64 solution is kept for the GPU arm."""
    if rank != 0:
        return
    import oracle
    from getdp_gb300 import workloads as W
    oracle.build()
    cpu = host_cpu()
    cpu["pinned_core"] = pin_one_core()
    n = args.n
    p = W.elasticity_p2(n=n, seed=2)
    dm = W.dofmap_for(p)
    t0 = time.perf_counter()
    ip, ix, dv, b = oracle.assemble(p, dm)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    xo, st, its, _ = oracle.solve(ip, ix, dv, b, algorithm=1, preconditioner=0, scaling=1,
                                  renumbering=1, nb_iter_max=200000, stopping_test=1e-8)
    t_sol = time.perf_counter() - t0
    import scipy.sparse as sp
    A = sp.csr_matrix((dv, ix, ip), shape=(dm.n_dof, dm.n_dof))
    true_rel = float(np.linalg.norm(b - A @ xo) / np.linalg.norm(b))
    del A
    try:
        np.savez(ORACLE_SOLUTION.format(n=n), x=xo, iterations=its, status=st,
                 true_rel_residual=true_rel, rhs_checksum=_rhs_checksum(b))
    except OSError:
        pass
    v = t_gen + t_sol
    vals = []
    samples = None
    for s in range(args.warmup + args.steps):
        total, pe, pi, samples = cpu_baseline(n, (ip, ix, dv), b, its)
        if s >= args.warmup:
            vals.append(total)
    full = {"generate_s": round(t_gen, 3), "solve_s": round(t_sol, 3),
            "cg_iterations": its, "status": st, "true_rel_residual": true_rel,
            "renumbering": "RCMK", "scaling": "diagonal"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"3D P2 elasticity {n}^3x6 tets, Jacobi-CG to 1e-8",
                       "elements": 6 * n ** 3, "unknowns": dm.n_dof},
            "full_run": full,
            "sampled_extrapolation_s": float(np.mean(vals)),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                             "cpu": cpu,
                             "sample": json.dumps({"full_run": full,
                                                   "steps_sampled": samples})},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def run_other(args, ws, rank, local):
    """The other single-GPU workloads: Generate + Solve through the same
    LinAlg entry points, timed with CUDA events, next to the oracle's CPU
    time on the same system (one core)."""
    from getdp_gb300 import _lib
    from getdp_gb300 import generate as G
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import workloads as W
    L = _lib.load(build_if_missing=True)
    if args.workload == "magnetostatics2d":
        n = args.n or 256
        p = W.magnetostatics_2d(n=n, seed=1)
        par = dict(Algorithm=8, Preconditioner=6, Krylov_Size=50,
                   Stopping_Test=1e-10, Nb_Iter_Max=5000)
        desc = (f"2D P1 magnetostatics {n}^2x2 triangles, ILU(0)-GMRES(50) to 1e-10")
        precisions = [0]
        metric = "time to 1e-10 residual (Generate + Solve), 2D P1 magnetostatics"
    else:
        n = args.n or 40
        p = W.curlcurl_edge(n=n, seed=3)
        par = dict(Algorithm=9, Preconditioner=6, Krylov_Size=40,
                   Stopping_Test=1e-8, Nb_Iter_Max=5000)
        desc = (f"3D curl-curl Whitney edges {n}^3x6 tets, ILU(0)-FGMRES(40) to 1e-8")
        precisions = [0, 1]
        metric = ("time to 1e-8 residual (Generate + Solve), 3D edge curl-curl, "
                  "FP32-ILU FGMRES")
    dm = W.dofmap_for(p)
    N = dm.n_dof
    ctx = LA.context()
    terms = G.DeviceTerms(p, dm)
    A = LA.gMatrix(N)
    b = LA.gVector(N)
    x = LA.gVector(N)

    def params(prec):
        S = LA.LinAlg_CreateSolver(None)
        for k, v in par.items():
            S.set(k, v)
        S.set("Precision", prec)
        S["stopping_test"] = par["Stopping_Test"]
        return S

    def ev(slot):
        _lib.check(L.gb300_event_record(ctx, slot))

    def elapsed(a, c):
        ms = ctypes.c_float()
        _lib.check(L.gb300_event_elapsed(ctx, a, c, ctypes.byref(ms)))
        return ms.value / 1e3

    res = {}
    for prec in precisions:
        S = params(prec)
        for _ in range(args.warmup):
            G.generate(A, b, terms.batch, pattern=True)
            LA.LinAlg_Solve(A, b, S, x)
        tg = ts = 0.0
        infos = []
        for _ in range(args.steps):
            ev(0)
            G.generate(A, b, terms.batch, pattern=True)
            ev(1)
            infos.append(LA.LinAlg_Solve(A, b, S, x))
            ev(2)
            tg += elapsed(0, 1)
            ts += elapsed(1, 2)
        inf = infos[-1]
        res[prec] = {"s": (tg + ts) / args.steps, "generate_s": tg / args.steps,
                     "solve_s": ts / args.steps, "iterations": inf["iterations"],
                     "status": inf["status"],
                     "true_rel_residual": inf["true_residual"] / max(inf["rhs_norm"], 1e-300)}
    two = None
    if args.workload == "magnetostatics2d":
        # the two-level cycle (Preconditioner 21) on aggregates of 8 x 8 nodes
        agg, nc = W.cell_aggregates(p, dm, max(1, min(n // 8, 45)))
        S = params(0)
        S.set("Preconditioner", 21)
        for _ in range(args.warmup):
            G.generate(A, b, terms.batch, pattern=True)
            A.set_aggregates(agg, nc)
            LA.LinAlg_Solve(A, b, S, x)
        tg = ts = 0.0
        for _ in range(args.steps):
            ev(0)
            G.generate(A, b, terms.batch, pattern=True)
            ev(1)
            A.set_aggregates(agg, nc)
            inf = LA.LinAlg_Solve(A, b, S, x)
            ev(2)
            tg += elapsed(0, 1)
            ts += elapsed(1, 2)
        two = {"s": (tg + ts) / args.steps, "solve_s": ts / args.steps,
               "iterations": inf["iterations"], "status": inf["status"], "aggregates": nc,
               "true_rel_residual": inf["true_residual"] / max(inf["rhs_norm"], 1e-300)}
    best = res[precisions[-1]]
    line = {"metric": metric, "value": best["s"], "unit": "s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": best["s"] * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if precisions[-1] == 0 else "f64+f32",
            "data": "synthetic (seeded)",
            "config": {"workload": desc, "elements": p.mesh.n_elems, "unknowns": N,
                       "nnz": A.nnz(), "parallelism": f"replicas x{ws}"},
            "fp64": res[0], "mixed": res.get(1)}
    if two is not None:
        line["two_level_fp64"] = two
    if not args.skip_cpu and rank == 0:
        import oracle
        oracle.build()
        t0 = time.perf_counter()
        ip, ix, dv, bb = oracle.assemble(p, dm)
        t_asm = time.perf_counter() - t0
        # the reference solves with RCMK renumbering (its default); one solve
        # capped at a bounded number of iterations, extrapolated
        cap = 600 if args.workload == "curlcurl" else 5000
        t0 = time.perf_counter()
        xs, st_, its, r_ = oracle.solve(ip, ix, dv, bb, algorithm=par["Algorithm"],
                                        preconditioner=6, renumbering=1,
                                        krylov_size=par["Krylov_Size"],
                                        nb_iter_max=cap,
                                        stopping_test=par["Stopping_Test"])
        t_sol = time.perf_counter() - t0
        total = t_asm + t_sol
        # the GPU's last solution against the oracle's (both to the same
        # relative residual; different orderings, so not bit-equal)
        rel_oracle = rel_curl = None
        if st_ == 0:
            rel_oracle = float(np.linalg.norm(x.numpy() - xs) / max(np.linalg.norm(xs), 1e-300))
            if args.workload == "curlcurl":
                # the field b = curl a: a curl-curl solution is fixed up to
                # the near-null gradients the 1e-6 mass term barely weighs,
                # so two solutions to 1e-8 agree in b, not in a
                from getdp_gb300 import post as PO
                from oracle import post_port
                bg = PO.curl_on_elements(terms.batch, x)
                bo = post_port.curl_on_elements(p, dm, xs)
                rel_curl = float(np.linalg.norm(bg - bo) / max(np.linalg.norm(bo), 1e-300))
        if st_ != 0 and its > 0:
            # capped: scale the solve to the GPU FP64 iteration count
            total = t_asm + t_sol * max(res[0]["iterations"], its) / its
        line["cpu_baseline"] = {
            "value": total, "unit": "s", "cores": 1, "kind": "port",
            "sample": json.dumps({"assembly_seconds": round(t_asm, 3),
                                  "solve_seconds": round(t_sol, 3),
                                  "iterations": its, "status": st_,
                                  "iteration_cap": cap,
                                  "extrapolated": bool(st_ != 0),
                                  "rel_diff_solution_vs_oracle": rel_oracle,
                                  "rel_diff_curl_vs_oracle": rel_curl})}
    if rank == 0:
        print(json.dumps(line))


def run_sweep(args, ws, rank, local):
    """Batched sweep: every problem's elements in one Generate, every system
    in one batched solve (FP64 GMRES, and FGMRES with an FP32 ILU(0)), each
    system with its own convergence test; solves/s, and the per-problem
    error against the oracle on a sample of problems."""
    from getdp_gb300 import _lib
    from getdp_gb300 import generate as G
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import workloads as W
    L = _lib.load(build_if_missing=True)
    probs = W.eddy_sweep(n_problems=args.problems, seed=7)
    bt = W.concat_problems(probs)
    N = bt.dofmap.n_dof
    ctx = LA.context()
    terms = G.DeviceTerms(bt.problem, bt.dofmap)
    A = LA.gMatrix(N)
    b = LA.gVector(N)
    x = LA.gVector(N)

    def params(prec, form=1):
        S = LA.LinAlg_CreateSolver(None)
        par = dict(Algorithm=8 if prec == 0 else 9, Preconditioner=6, Krylov_Size=40,
                   Stopping_Test=1e-10, Nb_Iter_Max=5000, Renumbering_Technique=1,
                   Precision=prec, Batch_Kernel=form)
        for k, v in par.items():
            S.set(k, v)
        S["stopping_test"] = 1e-10
        return S

    def ev(slot):
        _lib.check(L.gb300_event_record(ctx, slot))

    def elapsed(a, c):
        ms = ctypes.c_float()
        _lib.check(L.gb300_event_elapsed(ctx, a, c, ctypes.byref(ms)))
        return ms.value / 1e3

    res = {}
    sols = {}
    # Batch_Kernel c > 0: one launch, a thread-block cluster of c CTAs per
    # system; 0: one launch per Krylov kernel for all systems in step
    for prec, form in ((0, 4), (1, 4), (0, 1), (1, 1), (0, 2), (1, 2), (0, 8), (1, 8),
                       (0, 0), (1, 0)):
        S = params(prec, form)
        for _ in range(args.warmup):
            G.generate(A, b, terms.batch, pattern=True)
            LA.LinAlg_SolveBatch(A, b, S, x, bt.offsets)
        tg = ts = 0.0
        for _ in range(args.steps):
            ev(0)
            G.generate(A, b, terms.batch, pattern=True)
            ev(1)
            infos = LA.LinAlg_SolveBatch(A, b, S, x, bt.offsets)
            ev(2)
            tg += elapsed(0, 1)
            ts += elapsed(1, 2)
        its = [d["iterations"] for d in infos]
        rel = [d["true_residual"] / max(d["rhs_norm"], 1e-300) for d in infos]
        res[prec, form] = {"s": (tg + ts) / args.steps, "generate_s": tg / args.steps,
                     "solve_s": ts / args.steps,
                     "solves_per_s": len(probs) / ((tg + ts) / args.steps),
                     "converged": int(sum(d["status"] == 0 for d in infos)),
                     "iterations_min_median_max": [int(min(its)), int(np.median(its)),
                                                   int(max(its))],
                     "max_true_rel_residual": float(max(rel)),
                     "one_launch_form": all(d["batch_form"] == 1 for d in infos)}
        sols[prec, form] = x.numpy().copy()
    best = res[1, 4]
    line = {"metric": "batched sweep: 512 complex eddy-current problems, solves/s "
                      "(Generate + Solve to 1e-10)",
            "value": best["solves_per_s"], "unit": "solves/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": best["s"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32", "data": "synthetic (seeded)",
            "config": {"workload": f"{len(probs)} complex 2D eddy-current problems, "
                                   "32^2..160^2 cells, one batched Generate + "
                                   "batched ILU(0)-(F)GMRES(40)",
                       "elements": bt.problem.mesh.n_elems, "unknowns": N,
                       "nnz": A.nnz(), "parallelism": f"replicas x{ws}"},
            "fp64": res[0, 4], "mixed": res[1, 4],
            "cluster_ctas": {c: {"fp64": res[0, c], "mixed": res[1, c]} for c in (1, 2, 8)},
            "per_kernel_form": {"fp64": res[0, 0], "mixed": res[1, 0]},
            "forms_max_rel_diff": max(
                float(np.linalg.norm(sols[q, 4] - sols[q, 0]) /
                      max(np.linalg.norm(sols[q, 0]), 1e-300)) for q in (0, 1))}
    if not args.skip_cpu and rank == 0:
        import oracle
        oracle.build()
        rng = np.random.default_rng(0)
        sample = sorted(rng.choice(len(probs), size=6, replace=False).tolist())
        t_cpu = 0.0
        n_sample = 0
        errs = {0: [], 1: []}
        for k in sample:
            p, dm = probs[k], bt.dofmaps[k]
            t0 = time.perf_counter()
            ip, ix, dv, bb = oracle.assemble(p, dm)
            xo, st_, its_, _ = oracle.solve(ip, ix, dv, bb, algorithm=8, preconditioner=6,
                                            renumbering=1, krylov_size=40,
                                            stopping_test=float(np.float32(1e-10)),
                                            nb_iter_max=5000)
            t_cpu += time.perf_counter() - t0
            n_sample += dm.n_dof
            r0, r1 = bt.offsets[k], bt.offsets[k + 1]
            for prec in (0, 1):
                xg = sols[prec, 4][r0:r1]
                errs[prec].append(float(np.linalg.norm(xg - xo) / max(np.linalg.norm(xo), 1e-300)))
        total = t_cpu * N / max(n_sample, 1)
        line["per_problem_rel_error_vs_oracle"] = {"fp64_max": max(errs[0]),
                                                   "mixed_max": max(errs[1]),
                                                   "sample": sample}
        line["cpu_baseline"] = {
            "value": len(probs) / total, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": json.dumps({"problems": sample, "seconds": round(t_cpu, 3),
                                  "unknowns": n_sample,
                                  "extrapolated_seconds_all": round(total, 1)})}
        # the same path on every host core: one oracle process per core,
        # independent problems (the reference runs one system per process)
        import multiprocessing as mp
        cores = os.cpu_count() or 1
        many = sorted(rng.choice(len(probs), size=min(len(probs), 4 * cores),
                                 replace=False).tolist())
        jobs = [(probs[k], bt.dofmaps[k]) for k in many]
        with mp.get_context("spawn").Pool(cores) as pool:
            pool.map(_oracle_sweep_job, jobs[:cores])  # start-up, not timed
            t0 = time.perf_counter()
            pool.map(_oracle_sweep_job, jobs, chunksize=1)
            wall = time.perf_counter() - t0
        n_many = sum(bt.dofmaps[k].n_dof for k in many)
        total_all = wall * N / max(n_many, 1)
        line["cpu_baseline_all_cores"] = {
            "value": len(probs) / total_all, "unit": "solves/s", "cores": cores,
            "kind": "port",
            "sample": json.dumps({"problems": len(many), "seconds": round(wall, 3),
                                  "unknowns": n_many,
                                  "extrapolated_seconds_all": round(total_all, 1)})}
    if rank == 0:
        print(json.dumps(line))


def _oracle_sweep_job(job):
    """One problem of the sweep on the CPU oracle (a worker process)."""
    import oracle
    p, dm = job
    ip, ix, dv, bb = oracle.assemble(p, dm)
    oracle.solve(ip, ix, dv, bb, algorithm=8, preconditioner=6, renumbering=1,
                 krylov_size=40, stopping_test=float(np.float32(1e-10)), nb_iter_max=5000)
    return dm.n_dof


# adaptive relaxation factors of the Newton step (SolveJac_AdaptRelax list)
RELAX = (1.0, 0.5, 0.25, 0.125, 0.0625, 0.03125)


def run_nonlinear(args, ws, rank, local):
    """Nonlinear 2D magnetostatics (saturating B-H law, lognormal field):
    the reference's Newton loop (Generate; Solve; Generate; GetResidual;
    While[...] { Solve; Generate; GetResidual }) with adaptive relaxation of
    each step, to a 1e-8 relative nonlinear residual, each Solve
    ILU(0)-GMRES(50) to 1e-10 (FP64), or FGMRES with an FP32 ILU(0); wall
    time of the whole loop."""
    from getdp_gb300 import _lib
    from getdp_gb300 import generate as G
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import nonlinear as NL
    from getdp_gb300 import workloads as W
    _lib.load(build_if_missing=True)
    LA.context()
    n = args.n or 1024

    def params(prec):
        S = LA.LinAlg_CreateSolver(None)
        for k, v in dict(Algorithm=8 if prec == 0 else 9, Preconditioner=6, Krylov_Size=50,
                         Stopping_Test=1e-10, Nb_Iter_Max=20000, Renumbering_Technique=1,
                         Precision=prec).items():
            S.set(k, v)
        S["stopping_test"] = 1e-10
        return S

    def two_level(p, dm, prec):
        """Preconditioner 21: the two-level cycle on cells of the mesh; the
        aggregates are handed to the matrix at its first solve (the host's
        counting sort is inside the timed loop)."""
        S = params(prec)
        S.set("Preconditioner", 21)
        if args.coarse_cells <= 0:
            # no mesh given: the solver aggregates A's graph at its first solve
            return S, "from the matrix graph"
        agg, nc = W.cell_aggregates(p, dm, args.coarse_cells)
        seen = []

        def solve(A, b, x):
            if not seen or seen[0] is not A:
                A.set_aggregates(agg, nc)
                seen[:] = [A]
            return LA.LinAlg_Solve(A, b, S, x)
        return solve, nc

    def run_gpu(size, prec, reps, scatter=_lib.SCATTER_DEFAULT, coarse=False):
        p = W.nonlinear_2d(n=size, seed=5)
        dm = W.dofmap_for(p)
        terms = G.DeviceTerms(p, dm)
        terms.batch.scatter = scatter
        out = None
        ts = []
        nc = None
        for _ in range(reps):
            solver = params(prec)
            if coarse:
                solver, nc = two_level(p, dm, prec)
            t0 = time.perf_counter()
            r = NL.newton(terms, dm.n_dof, solver, tol_rel=1e-8, iter_max=50,
                          relaxation=RELAX)
            ts.append(time.perf_counter() - t0)
            out = r
        d = {"s": float(np.median(ts)), "newton_steps": len(out.history) - 1,
             "linear_iterations": int(sum(s["iterations"] for s in out.solves)),
             "final_rel_residual": out.history[-1] / out.history[0],
             "converged": out.converged, "unknowns": dm.n_dof}
        if coarse:
            d["aggregates"] = nc
        return d, out

    res = {}
    for prec in (() if args.two_level_only else (0, 1)):
        run_gpu(n, prec, 1)  # warm-up (pattern, colouring, tuning)
        res[prec], _ = run_gpu(n, prec, max(args.steps, 1))
    two = {}
    for prec in (0, 1):
        run_gpu(n, prec, 1, coarse=True)
        two[prec], _ = run_gpu(n, prec, max(args.steps, 1), coarse=True)
    best = min(list(res.values()) + list(two.values()), key=lambda r: r["s"])
    # the same with the coloured (atomic-free) scatter: Generate, and so the
    # whole Newton loop, gives the same numbers on every run
    deterministic = None
    if not args.two_level_only:
        det = []
        for _ in range(2):
            r, o = run_gpu(n, 1, 1, scatter=_lib.SCATTER_COLOURED)
            det.append((r, float(o.history[-1])))
        deterministic = dict(det[1][0])
        deterministic["repeat_identical"] = bool(
            det[0][0]["linear_iterations"] == det[1][0]["linear_iterations"] and
            det[0][1] == det[1][1])
    learned = None
    if args.learned_weights:
        from getdp_gb300 import learned as LR
        net = LR.MPNN(seed=1)
        net.set_params(np.load(args.learned_weights))
        p = W.nonlinear_2d(n=n, seed=5)
        dm = W.dofmap_for(p)
        terms = G.DeviceTerms(p, dm)
        pol = LR.NewtonSolver(net, stopping_test=1e-10, precision=1)
        t0 = time.perf_counter()
        r = NL.newton(terms, dm.n_dof, pol, tol_rel=1e-8, iter_max=50, relaxation=RELAX)
        learned = {"s": time.perf_counter() - t0, "newton_steps": len(r.history) - 1,
                   "linear_iterations": int(sum(s["iterations"] for s in r.solves)),
                   "learned_attempt_iterations": int(sum(
                       s.get("learned_attempt_iterations") or 0 for s in pol.log)),
                   "solves": pol.log, "converged": r.converged,
                   "weights": os.path.basename(args.learned_weights)}
    learned2 = None
    if args.learned_two_level_weights:
        # the correction trained for the two-level cycle (Preconditioner 22),
        # against the same cycle without it (two_level_mixed) and plain FP64
        from getdp_gb300 import learned as LR
        net = LR.MPNN(seed=1)
        net.set_params(np.load(args.learned_two_level_weights))
        p = W.nonlinear_2d(n=n, seed=5)
        dm = W.dofmap_for(p)
        agg, nc = W.cell_aggregates(p, dm, args.coarse_cells)
        terms = G.DeviceTerms(p, dm)
        runs = []
        for _ in range(2):  # the first run also makes the network's graph buffers
            pol = LR.TwoLevelNewtonSolver(net, agg, nc, stopping_test=1e-10, precision=1)
            t0 = time.perf_counter()
            r = NL.newton(terms, dm.n_dof, pol, tol_rel=1e-8, iter_max=50,
                          relaxation=RELAX)
            runs.append((time.perf_counter() - t0, r, pol))
        t_l, r, pol = runs[-1]
        learned2 = {"s": t_l, "newton_steps": len(r.history) - 1,
                    "linear_iterations": int(sum(s["iterations"] for s in r.solves)),
                    "learned_attempt_iterations": int(sum(
                        s.get("learned_attempt_iterations") or 0 for s in pol.log)),
                    "solves": pol.log, "converged": r.converged, "aggregates": nc,
                    "speedup_vs_plain_fp64": res[0]["s"] / t_l if 0 in res else None,
                    "speedup_vs_two_level_mixed": two[1]["s"] / t_l,
                    "weights": os.path.basename(args.learned_two_level_weights)}
    line = {"metric": "nonlinear 2D magnetostatics: time to 1e-8 Newton residual "
                      "(Generate + Solve per step)",
            "value": best["s"], "unit": "s", "n_gpus": ws, "steps": args.steps,
            "warmup": 1, "ms_per_step": best["s"] * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
            "data": "synthetic (seeded)",
            "config": {"workload": f"nonlinear a_z P1 {n}^2x2 triangles, lognormal GRF "
                                   "reluctivity x saturating B-H law, 8 current blobs; "
                                   "Newton, ILU(0)-(F)GMRES(50) per step; two-level "
                                   "arms: ILU(0) around a coarse correction on "
                                   f"{args.coarse_cells}^2 cells (Preconditioner 21)",
                       "elements": 2 * n * n, "unknowns": two[0]["unknowns"],
                       "parallelism": f"replicas x{ws}"},
            "fp64": res.get(0), "mixed": res.get(1), "two_level_fp64": two[0],
            "two_level_mixed": two[1],
            "speedup_two_level_mixed_vs_plain_fp64":
                res[0]["s"] / two[1]["s"] if 0 in res else None,
            "mixed_coloured_scatter": deterministic}
    if learned is not None:
        line["learned_mixed"] = learned
    if learned2 is not None:
        line["learned_two_level_mixed"] = learned2
    if not args.skip_cpu and rank == 0:
        import oracle
        oracle.build()
        m = args.cpu_n
        p = W.nonlinear_2d(n=m, seed=5)
        dm = W.dofmap_for(p)
        t0 = time.perf_counter()
        xo, hist, its = oracle.newton(p, dm, tol=1e-8, iter_max=50, relaxation=RELAX,
                                      algorithm=8,
                                      preconditioner=6, renumbering=1, krylov_size=50,
                                      stopping_test=float(np.float32(1e-10)),
                                      nb_iter_max=20000)
        t_cpu = time.perf_counter() - t0
        gsame, gout = run_gpu(m, 0, 1)
        err = float(np.linalg.norm(gout.x.numpy() - xo) / np.linalg.norm(xo))
        line["cpu_baseline"] = {
            "value": t_cpu, "unit": "s", "cores": 1, "kind": "port",
            "sample": json.dumps({"size": f"{m}^2", "newton_steps": len(hist) - 1,
                                  "linear_iterations": int(sum(its)),
                                  "gpu_fp64_same_size_s": round(gsame["s"], 4),
                                  "gpu_newton_steps_same_size": gsame["newton_steps"],
                                  "rel_diff_solution_vs_oracle": err})}
    if rank == 0:
        print(json.dumps(line))


def run_io(args, ws, rank):
    """The steps either side of the path, on the host: the MSH 2.2 reader
    (native and numpy), DOF numbering and edge creation, and the .pre and
    .res writers, as MB/s or unknowns/s on the largest configurations'
    meshes.  Best of `steps` runs after `warmup`."""
    from getdp_gb300 import fileio as FI
    from getdp_gb300 import workloads as W

    def best(f):
        for _ in range(args.warmup):
            f()
        ts = []
        for _ in range(max(args.steps, 1)):
            t0 = time.perf_counter()
            f()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    out = {}
    tmp = tempfile.mkdtemp()
    n = args.n or 1024
    p = W.nonlinear_2d(n=n, seed=5)
    msh = os.path.join(tmp, "m.msh")
    W.write_msh22(p.mesh, msh)
    mb = os.path.getsize(msh) / 1e6
    t_nat = best(lambda: FI.read_msh22(msh))
    t_np = best(lambda: FI.read_msh22_numpy(msh))
    out["msh22_read"] = {"file_mb": round(mb, 1), "nodes": p.mesh.n_nodes,
                         "elements": p.mesh.n_elems, "native_s": t_nat,
                         "native_mb_s": mb / t_nat, "numpy_s": t_np, "numpy_mb_s": mb / t_np}
    t_num = best(lambda: W.dofmap_for(p))
    dm = W.dofmap_for(p)
    out["dof_numbering_2d"] = {"unknowns": dm.n_dof, "s": t_num,
                               "unknowns_per_s": dm.n_dof / t_num}
    pre = os.path.join(tmp, "m.pre")
    t_pre = best(lambda: FI.write_pre(pre, p.mesh, dm))
    out["pre_write"] = {"mb": round(os.path.getsize(pre) / 1e6, 1), "s": t_pre,
                        "mb_s": os.path.getsize(pre) / 1e6 / t_pre}
    res = os.path.join(tmp, "m.res")
    x = np.random.default_rng(0).standard_normal(dm.n_dof)
    t_res = best(lambda: FI.write_res(res, x, binary=True))
    out["res_write_binary"] = {"mb": round(os.path.getsize(res) / 1e6, 1), "s": t_res,
                               "mb_s": os.path.getsize(res) / 1e6 / t_res}
    e = W.elasticity_p2(n=48, seed=2)
    t_e = best(lambda: W.dofmap_for(e))
    ne = W.dofmap_for(e).n_dof
    out["dof_numbering_p2_48"] = {"unknowns": ne, "s": t_e, "unknowns_per_s": ne / t_e}
    c = W.curlcurl_edge(n=40, seed=3)
    t_c = best(lambda: W.dofmap_for(c))
    nc = W.dofmap_for(c).n_dof
    out["edge_creation_numbering_40"] = {"unknowns": nc, "s": t_c, "unknowns_per_s": nc / t_c}
    for f in (msh, pre, res):
        os.remove(f)
    os.rmdir(tmp)
    line = {"metric": "host pre-processing and file formats: MSH 2.2 read, DOF numbering, "
                      ".pre/.res write", "value": out["msh22_read"]["native_mb_s"],
            "unit": "MB/s (MSH 2.2 read)", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "host", "data": "synthetic (seeded)",
            "config": {"workload": f"nonlinear 2D mesh {n}^2x2 triangles (MSH 2.2 ASCII), "
                                   "P2 elasticity 48^3, edge curl-curl 40^3"},
            "gpu_launches": 0}
    line.update(out)
    if rank == 0:
        print(json.dumps(line))


def main():
    args = parse()
    ws, rank, local, pg = dist_setup(args)
    if args.workload == "io":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference arm times the headline workload only"}))
            return
        run_io(args, ws, rank)
        return
    if args.workload == "nonlinear":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference arm times the headline workload only"}))
            return
        run_nonlinear(args, ws, rank, local)
        return
    if args.workload == "eddysweep":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference arm times the headline workload only"}))
            return
        run_sweep(args, ws, rank, local)
        return
    if args.workload != "elasticity":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference arm times the headline workload only"}))
            return
        run_other(args, ws, rank, local)
        return
    if args.n is None:
        args.n = 48
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.profile:
        profile_run(args)
        return
    from getdp_gb300 import _lib
    from getdp_gb300 import generate as G
    from getdp_gb300 import linalg as LA
    from getdp_gb300 import workloads as W
    _lib.load(build_if_missing=True)
    L = _lib.load()
    n = args.n
    p = W.elasticity_p2(n=n, seed=2)
    dm = W.dofmap_for(p)
    N = dm.n_dof
    ctx = LA.context()
    terms = G.DeviceTerms(p, dm)  # resident element tables
    A = LA.gMatrix(N)
    b = LA.gVector(N)
    x = LA.gVector(N)
    S_mixed = solver_params(True)
    S_plain = solver_params(False)

    def step(S):
        G.generate(A, b, terms.batch, pattern=True)
        return LA.LinAlg_Solve(A, b, S, x)

    def barrier():
        if pg:
            pg.barrier()

    def ev(slot):
        _lib.check(L.gb300_event_record(ctx, slot))

    def elapsed(a, c):
        ms = ctypes.c_float()
        _lib.check(L.gb300_event_elapsed(ctx, a, c, ctypes.byref(ms)))
        return ms.value / 1e3

    # components, once (outside the timed region): the first Generate builds
    # the pattern and caches it on the context; a Generate of the same
    # element table reuses it (the steady state of every step)
    ev(0)
    G.generate(A, b, terms.batch, pattern=True)
    ev(1)
    G.generate(A, b, terms.batch, pattern=True)
    ev(2)
    t_gen_cold, t_gen_full = elapsed(0, 1), elapsed(1, 2)
    t_gen_values = t_gen_full
    nnz = A.nnz()
    # the scatter modes of the element kernel, each timed warm (its first
    # call builds the position table or the colouring, once per pattern)
    scatter_modes = {}
    for name, m in (("search_atomic", _lib.SCATTER_SEARCH), ("table_atomic", _lib.SCATTER_TABLE),
                    ("coloured_no_atomics", _lib.SCATTER_COLOURED)):
        ev(0)
        G.generate(A, b, terms.batch, pattern=True, scatter=m)
        ev(1)
        G.generate(A, b, terms.batch, pattern=True, scatter=m)
        ev(2)
        scatter_modes[name] = {"first_s": elapsed(0, 1), "s": elapsed(1, 2)}
    terms.batch.scatter = _lib.SCATTER_DEFAULT
    fp64_peak = ctypes.c_double()
    _lib.check(L.gb300_bench_fp64_peak(ctx, ctypes.byref(fp64_peak)))
    fp64_peak = fp64_peak.value
    if args.no_plain:
        info_plain, t_plain = {"iterations": None}, None
    else:
        ev(3)
        info_plain = LA.LinAlg_Solve(A, b, S_plain, x)
        ev(4)
        t_plain = elapsed(3, 4)
        if info_plain["status"] != 0:
            raise SystemExit(f"plain FP64 solve failed: {info_plain}")
        x_plain = x.numpy()  # the FP64 solution, for the mixed solve's error

    for _ in range(args.warmup):
        step(S_mixed)
    clocks = Clocks(local)
    barrier()
    clocks.start()
    ev(5)
    infos = []
    for _ in range(args.steps):
        infos.append(step(S_mixed))
    ev(6)
    barrier()
    clk = clocks.stop()
    t_total = elapsed(5, 6)
    if pg:
        import torch
        t = torch.tensor([t_total], device=f"cuda:{local}")
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        t_total = float(t.item())
    per_step = t_total / args.steps
    for inf in infos:
        if inf["status"] != 0:
            raise SystemExit(f"mixed solve failed: {inf}")
    # the mixed solution against the plain FP64 one (both to 1e-8 relative
    # residual of the scaled system), outside the timed region
    rel_vs_fp64 = None
    xm = x.numpy()
    if not args.no_plain:
        rel_vs_fp64 = float(np.linalg.norm(xm - x_plain) / np.linalg.norm(x_plain))
    # both solutions against the oracle's FP64 Sparskit CG solution of the
    # same system, when the reference arm ran before on this host
    vs_oracle = {"available": False,
                 "note": "the reference arm (bench.py --impl reference) keeps the "
                         "oracle's full FP64 solution for this comparison"}
    path = ORACLE_SOLUTION.format(n=n)
    if os.path.exists(path):
        try:
            d = np.load(path)
            if len(d["x"]) == N and abs(float(d["rhs_checksum"]) - _rhs_checksum(b.numpy())) <= \
                    1e-12 * abs(float(d["rhs_checksum"])):
                xo = d["x"]
                no = np.linalg.norm(xo)
                vs_oracle = {"available": True,
                             "mixed_rel_diff": float(np.linalg.norm(xm - xo) / no),
                             "plain_fp64_rel_diff": (float(np.linalg.norm(x_plain - xo) / no)
                                                     if not args.no_plain else None),
                             "oracle_cg_iterations": int(d["iterations"]),
                             "oracle_true_rel_residual": float(d["true_rel_residual"])}
        except Exception as e:  # a stale or partial file: no comparison
            vs_oracle = {"available": False, "note": f"unreadable: {e}"}

    # e2e: element tables from pinned host memory, solution back to host
    arrays = G.term_arrays(p, dm)
    pinned = {}
    h2d = 0
    for k, v in arrays.items():
        if k.startswith("_"):
            continue
        hp = ctypes.c_void_p()
        _lib.check(L.gb300_host_alloc(v.nbytes, ctypes.byref(hp)))
        ctypes.memmove(hp, v.ctypes.data, v.nbytes)
        pinned[k] = (hp, v.nbytes)
        h2d += v.nbytes
    xh_p = ctypes.c_void_p()
    _lib.check(L.gb300_host_alloc(8 * N, ctypes.byref(xh_p)))

    def e2e_step():
        for k, (hp, nb) in pinned.items():
            _lib.check(L.gb300_copy_to_device(ctx, ctypes.c_void_p(terms.ptrs[k]), hp, nb))
        info = step(S_mixed)
        _lib.check(L.gb300_vector_get(x.h, xh_p))
        return info

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    t_e2e = (time.perf_counter() - t0) / args.steps

    # roofline of the dominant kernel: the FP32 CSR SpMV of the CG
    ms = ctypes.c_double()
    _lib.check(L.gb300_bench_spmv(A.h, 1, 20, ctypes.byref(ms)))
    t_spmv32 = ms.value / 1e3
    _lib.check(L.gb300_bench_spmv(A.h, 0, 20, ctypes.byref(ms)))
    t_spmv64 = ms.value / 1e3
    # the CG iterates on the node-blocked (3x3 BSR) copy of this system:
    # per block 9 values + 1 column index; vectors padded to 4 per node,
    # read once (p) and written once (q)
    nblk, nn = nnz // 9, N // 3
    bytes32 = nblk * (9 * 4 + 4) + (nn + 1) * 4 + 2 * 4 * nn * 4
    bytes64 = nblk * (9 * 8 + 4) + (nn + 1) * 4 + 2 * 4 * nn * 8
    peak, peak_kind = peaks()
    ach = bytes32 / t_spmv32 / 1e9
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "spmv_traffic.json")
    if os.path.exists(tr_path):
        try:
            tr = json.load(open(tr_path))
            traffic = tr.get("bytes_per_launch_full_size")
        except Exception:
            traffic = None
    inf = infos[-1]
    # per step: Generate (pattern ~12 kernels + values) and solve set-up
    # (~15), then graph replays of 16 CG iterations x 3 kernels (SpMV, step,
    # direction; a replay ends early at each reliable update) and 5 kernels
    # per reliable update
    upd = inf.get("refinement_steps", 0) or 0
    main_replays = -(-inf["iterations"] // 16) + upd
    gpu_launches = args.steps * (27 + main_replays * 16 * 3 + upd * 5)

    line = {
        "metric": METRIC, "value": per_step, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32", "data": "synthetic (seeded)",
        "config": {"workload": f"3D P2 elasticity {n}^3x6 tets, "
                               "Generate + Jacobi-CG to 1e-8, FP32 SpMV in FP64 reliable updates",
                   "elements": p.mesh.n_elems, "unknowns": N, "nnz": nnz,
                   "parallelism": f"replicas x{ws}", "l2": "inputs larger than L2, no flush"},
        "assembly_gdof_s": N / t_gen_full / 1e9,
        "assembly_cold_gdof_s": N / t_gen_cold / 1e9,
        "generate_s": t_gen_full, "generate_cold_s": t_gen_cold,
        "generate_scatter_modes": scatter_modes,
        "roofline_assembly": assembly_roofline(p.mesh.n_elems, N, nnz, t_gen_full,
                                               fp64_peak, peak),
        "solve_iterations": inf["iterations"], "reliable_updates": inf["refinement_steps"],
        "true_rel_residual": inf["true_residual"] / inf["rhs_norm"],
        "plain_fp64_solve_s": t_plain, "plain_fp64_iterations": info_plain["iterations"],
        "mixed_vs_plain_fp64_rel_diff": rel_vs_fp64,
        "error_vs_oracle_fp64": vs_oracle,
        "plain_fp64_time_to_solution_s": (t_gen_full + t_plain) if t_plain else None,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "traffic": traffic,
                     "kernel": "k_bsr_spmv<2,float> (3x3-block SpMV + fused <p,Ap>)",
                     "algorithmic_bytes_per_launch": bytes32,
                     "launch_ms": t_spmv32 * 1e3, "peak_kind": peak_kind,
                     "fp64_spmv_gbs": bytes64 / t_spmv64 / 1e9},
        "e2e": {"value": t_e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 8 * N},
        "gpu_launches": gpu_launches,
        "clocks": clk,
    }
    if rank == 0 and ws == 1 and not args.skip_cpu:
        ip, ix, dv = A.csr()
        total, pe, pi, sample = cpu_baseline(n, (ip, ix, dv), b.numpy(),
                                             info_plain["iterations"])
        line["cpu_baseline"] = {"value": total, "unit": UNIT, "cores": 1,
                                "kind": "port", "cpu": host_cpu(),
                                "sample": json.dumps(sample),
                                "per_element_s": pe, "per_cg_iteration_s": pi}
    if rank == 0:
        print(json.dumps(line))
    for hp, _ in pinned.values():
        L.gb300_host_free(hp)
    L.gb300_host_free(xh_p)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
