"""ORACLE — test infrastructure only.

CPU restatement of the reference's Generate/Solve path (GetDP 3.5.0 element
loop + Sparskit backend) used to check the GPU product.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may load
it, and only as the checker; the product never routes through it.

The C sources next to this file are compiled into ``oracle/_build`` by
:func:`build` (two flavours: double-precision ILU, and single-precision ILU
as in the official reference build, ``HAVE_ILU_FLOAT``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SOURCES = ["sparskit_port.c", "solve_port.c", "assemble_port.c"]
_LIBS: dict = {}

# Sparskit.h codes
CG, GMRES, FGMRES = 1, 8, 9
NONE, ILU0, DIAGONAL = 0, 6, 8


def _lib_path(ilu: str) -> str:
    return os.path.join(BUILD, f"liboracle_ilu{ilu}.so")


def build(force: bool = False) -> None:
    """Compile both oracle flavours (a few seconds with gcc)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    newest = max(os.path.getmtime(s) for s in srcs)
    for ilu, flag in (("64", []), ("32", ["-DHAVE_ILU_FLOAT"])):
        out = _lib_path(ilu)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
            continue
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w",
               *flag, *srcs, "-o", out, "-lm"]
        subprocess.check_call(cmd)


class _Params(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int), ("preconditioner", ctypes.c_int),
                ("precond_position", ctypes.c_int), ("scaling", ctypes.c_int),
                ("renumbering", ctypes.c_int), ("krylov_size", ctypes.c_int),
                ("nb_iter_max", ctypes.c_int), ("stopping_test", ctypes.c_double)]


def lib(ilu: str = "64") -> ctypes.CDLL:
    if ilu not in _LIBS:
        path = _lib_path(ilu)
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        i64, i32p, dp = ctypes.c_int64, ctypes.POINTER(ctypes.c_int32), \
            ctypes.POINTER(ctypes.c_double)
        L.oracle_assemble_tri_p1.restype = i64
        L.oracle_assemble_tet10_elasticity.restype = i64
        L.oracle_assemble_tet4_curlcurl.restype = i64
        L.oracle_assemble_tri3_nl.restype = i64
        L.oracle_coo_to_csr.restype = i64
        L.oracle_solve_csr.restype = ctypes.c_int
        _LIBS[ilu] = L
    return _LIBS[ilu]


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def assemble(problem, dofmap, ilu: str = "64", solution=None, with_abs=False):
    """Run the restated element loop (at the current solution, for the
    nonlinear formulation); returns (indptr, indices, data, b), plus with
    with_abs the per-entry sums of |contribution| and the per-row sums of
    |RHS contribution| (the rounding scales of sums in another order)."""
    L = lib(ilu)
    babs = None
    if with_abs:
        babs = np.zeros(dofmap.n_dof, np.float64)
        L.oracle_set_rhs_abs(_p(babs, ctypes.c_double))
    try:
        rr, cc, vv, b = assemble_coo(problem, dofmap, ilu, solution)
    finally:
        if with_abs:
            L.oracle_set_rhs_abs(None)
    I32, D = ctypes.c_int32, ctypes.c_double
    n = dofmap.n_dof
    nz = len(vv)
    indptr = np.empty(n + 1, np.int32)
    indices = np.empty(max(nz, 1), np.int32)
    data = np.empty(max(nz, 1), np.float64)
    absd = np.empty(max(nz, 1), np.float64) if with_abs else None
    nnz = L.oracle_coo_to_csr(n, ctypes.c_int64(nz), _p(rr, I32), _p(cc, I32),
                              _p(vv, D), _p(indptr, I32), _p(indices, I32),
                              _p(data, D), _p(absd, D) if with_abs else None)
    del rr, cc, vv
    out = (indptr, indices[:nnz].copy(), data[:nnz].copy(), b)
    if with_abs:
        return out + (absd[:nnz].copy(), babs)
    return out


def assemble_coo(problem, dofmap, ilu: str = "64", solution=None):
    """The matrix contributions in the reference's call order (the
    LinAlg_AddDoubleInMatrix sequence) and the RHS: (rows, cols, vals, b)."""
    L = lib(ilu)
    fixed = getattr(dofmap, "fixed_values", None)
    if fixed is not None:
        fixed = np.ascontiguousarray(fixed, np.float64)
        L.oracle_set_fixed(_p(fixed, ctypes.c_double))
    try:
        return _assemble_coo(L, problem, dofmap, solution)
    finally:
        if fixed is not None:
            L.oracle_set_fixed(None)


def _assemble_coo(L, problem, dofmap, solution):
    m = problem.mesh
    n = dofmap.n_dof
    ne = m.n_elems
    nodes = np.ascontiguousarray(m.nodes, np.float64)
    elems = np.ascontiguousarray(m.elems, np.int32)
    edofs = np.ascontiguousarray(dofmap.elem_dofs, np.int32)
    nloc = edofs.shape[1]
    f = problem.formulation
    # per element: eddy 4 entries per pair (2 real + 2 imaginary), curl-curl
    # two terms (curl and mass), the others one
    cap = ne * nloc * nloc * {"eddy2d": 4, "curlcurl": 2}.get(f, 1)
    rr = np.empty(cap, np.int32)
    cc = np.empty(cap, np.int32)
    vv = np.empty(cap, np.float64)
    b = np.zeros(n, np.float64)
    I32, D = ctypes.c_int32, ctypes.c_double
    if f in ("magnetostatics2d", "eddy2d"):
        cplx = f == "eddy2d"
        sigma = np.ascontiguousarray(problem.params.get("sigma", np.zeros(ne)), np.float64)
        omega = problem.params.get("freq", 0.0) * 6.2831853071795865
        nz = L.oracle_assemble_tri_p1(
            ne, _p(nodes, D), _p(elems, ctypes.c_int), _p(edofs, ctypes.c_int),
            _p(np.ascontiguousarray(problem.coef, np.float64), D),
            _p(np.ascontiguousarray(problem.source, np.float64), D),
            _p(sigma, D), ctypes.c_double(omega), int(cplx), ctypes.c_int64(cap),
            _p(rr, I32), _p(cc, I32), _p(vv, D), _p(b, D))
    elif f == "elasticity":
        fz = -problem.params["rho"] * problem.params["g"]
        nz = L.oracle_assemble_tet10_elasticity(
            ne, _p(nodes, D), _p(elems, ctypes.c_int), _p(edofs, ctypes.c_int),
            _p(np.ascontiguousarray(problem.coef, np.float64), D),
            ctypes.c_double(problem.params["poisson"]), ctypes.c_double(fz),
            ctypes.c_int64(cap), _p(rr, I32), _p(cc, I32), _p(vv, D), _p(b, D))
    elif f == "curlcurl":
        sg = np.ascontiguousarray(dofmap.elem_sign, np.int8)
        nz = L.oracle_assemble_tet4_curlcurl(
            ne, _p(nodes, D), _p(elems, ctypes.c_int), _p(edofs, ctypes.c_int),
            _p(sg, ctypes.c_byte),
            _p(np.ascontiguousarray(problem.coef, np.float64), D),
            _p(np.ascontiguousarray(problem.source, np.float64).reshape(ne, 3), D),
            ctypes.c_double(problem.params["reg"]),
            ctypes.c_int64(cap), _p(rr, I32), _p(cc, I32), _p(vv, D), _p(b, D))
    elif f == "nonlinear2d":
        x = np.zeros(n) if solution is None else np.ascontiguousarray(solution, np.float64)
        nz = L.oracle_assemble_tri3_nl(
            ne, _p(nodes, D), _p(elems, ctypes.c_int), _p(edofs, ctypes.c_int),
            _p(np.ascontiguousarray(problem.coef, np.float64), D),
            _p(np.ascontiguousarray(problem.source, np.float64), D), _p(x, D),
            ctypes.c_double(problem.params["k_sat"]), ctypes.c_double(problem.params["b_sat2"]),
            ctypes.c_int64(cap), _p(rr, I32), _p(cc, I32), _p(vv, D), _p(b, D))
    else:
        raise ValueError(f)
    if nz > cap:
        raise RuntimeError("oracle COO capacity exceeded")
    return rr[:nz].copy(), cc[:nz].copy(), vv[:nz].copy(), b


def solve(indptr, indices, data, b, algorithm=GMRES, preconditioner=ILU0,
          scaling=0, renumbering=1, krylov_size=40, nb_iter_max=1000,
          stopping_test=1e-10, precond_position=2, ilu: str = "64"):
    """Restated Sparskit solve_matrix; returns (x, status, iterations, res)."""
    L = lib(ilu)
    n = len(indptr) - 1
    p = _Params(algorithm, preconditioner, precond_position, scaling,
                renumbering, krylov_size, nb_iter_max, stopping_test)
    x = np.zeros(n, np.float64)
    its = ctypes.c_int(0)
    res = ctypes.c_double(0.0)
    ip = np.ascontiguousarray(indptr, np.int32)
    ix = np.ascontiguousarray(indices, np.int32)
    dv = np.ascontiguousarray(data, np.float64)
    bv = np.ascontiguousarray(b, np.float64)
    st = L.oracle_solve_csr(n, _p(ip, ctypes.c_int), _p(ix, ctypes.c_int),
                            _p(dv, ctypes.c_double), _p(bv, ctypes.c_double),
                            _p(x, ctypes.c_double), ctypes.byref(p),
                            ctypes.byref(its), ctypes.byref(res))
    return x, st, its.value, res.value


def params_from_golden(keys, vals) -> dict:
    """solver.par keys (as stored in the golden fixtures) -> solve() kwargs."""
    m = {"Algorithm": "algorithm", "Preconditioner": "preconditioner",
         "Scaling": "scaling", "Renumbering_Technique": "renumbering",
         "Krylov_Size": "krylov_size", "Nb_Iter_Max": "nb_iter_max",
         "Stopping_Test": "stopping_test"}
    out = {}
    for k, v in zip(keys, vals):
        k = str(k)
        out[m[k]] = float(v) if k == "Stopping_Test" else int(v)
    # reference defaults (Sparskit.cpp:1847-1868) for keys not given
    out.setdefault("krylov_size", 40)
    out.setdefault("scaling", 0)
    out.setdefault("renumbering", 1)
    return out


def newton(problem, dofmap, tol=1e-8, iter_max=50, relaxation=(1.0,), **solve_kw):
    """The Newton loop of the reference's nonlinear resolution
    (Lib_Magnetostatics_a_phi.pro:220-240): Generate; Solve; Generate;
    GetResidual; While[res > 0 && res/res0 > tol && res/res0 <= 1 &&
    iter < iter_max] { Solve; Generate; GetResidual }.  GetResidual is
    ||b - A x||_2 (SolvingOperations.cpp:1318-1341).  With several
    relaxation factors, each Solve's step dx = x_new - x is relaxed as
    SolveJac_AdaptRelax does with CheckAll 0 (SolvingOperations.cpp:
    1593-1700): factors tried in order, the residual ||b - A x|| / N at
    x + f dx (regenerated there) kept while it decreases, the best factor
    taken.  Returns (x, residual history, linear iterations per solve)."""
    import scipy.sparse as sp
    n = dofmap.n_dof
    x = np.zeros(n)
    its = []

    def gen(xc):
        ip, ix, dv, bb = assemble(problem, dofmap, solution=xc)
        return ip, ix, dv, bb

    def sol(sysm):
        ip, ix, dv, bb = sysm
        xs, st, k, _ = solve(ip, ix, dv, bb, **solve_kw)
        if st != 0:
            raise RuntimeError(f"oracle linear solve failed ({st})")
        its.append(k)
        return xs

    def resid(sysm, xc):
        ip, ix, dv, bb = sysm
        A = sp.csr_matrix((dv, ix, ip), shape=(n, n))
        return float(np.linalg.norm(bb - A @ xc))

    def step(sysm, x):
        xn = sol(sysm)
        if len(relaxation) == 1:
            return xn, gen(xn)
        dx = xn - x
        err_prev, f_opt, best = 1e99, relaxation[0], None
        for k, f in enumerate(relaxation):
            xt = x + f * dx
            st = gen(xt)
            e = resid(st, xt) / n
            if e < err_prev:
                err_prev, f_opt, best = e, f, (xt, st)
            elif k > 0:
                break
        return best

    sysm = gen(x)
    x, sysm = step(sysm, x)
    res0 = resid(sysm, x)
    hist = [res0]
    res, it = res0, 0
    while res > 1e-300 and res / res0 > tol and res / res0 <= 1 and it < iter_max:
        x, sysm = step(sysm, x)
        res = resid(sysm, x)
        it += 1
        hist.append(res)
    return x, np.array(hist), its


def rcmk_new_of(indptr, indices):
    """The reference's RCMK permutation (the restated cmkreord, as
    Sparskit.cpp:247-250 calls it) of a 0-based CSR pattern: new_of[i] is the
    new 0-based index of row i."""
    L = lib()
    n = len(indptr) - 1
    nnz = int(indptr[-1])
    ia = np.ascontiguousarray(np.asarray(indptr) + 1, np.int32)
    ja = np.ascontiguousarray(np.asarray(indices) + 1, np.int32)
    a = np.zeros(max(nnz, 1), np.float64)
    a0 = np.zeros(max(nnz, 1), np.float64)
    ja0 = np.zeros(max(nnz, 1), np.int32)
    ia0 = np.zeros(n + 1, np.int32)
    iperm = np.zeros(n, np.int32)
    mask = np.zeros(max(nnz, n), np.int32)
    riord = np.zeros(n, np.int32)
    levels = np.zeros(n + 1, np.int32)
    init, maskval, nlev = ctypes.c_int(1), ctypes.c_int(1), ctypes.c_int(1)
    P = ctypes.POINTER
    f = L.cmkreord_
    f.restype = None
    f(ctypes.byref(ctypes.c_int(n)), a.ctypes.data_as(P(ctypes.c_double)),
      ja.ctypes.data_as(P(ctypes.c_int)), ia.ctypes.data_as(P(ctypes.c_int)),
      a0.ctypes.data_as(P(ctypes.c_double)), ja0.ctypes.data_as(P(ctypes.c_int)),
      ia0.ctypes.data_as(P(ctypes.c_int)), ctypes.byref(init),
      iperm.ctypes.data_as(P(ctypes.c_int)), mask.ctypes.data_as(P(ctypes.c_int)),
      ctypes.byref(maskval), ctypes.byref(nlev), riord.ctypes.data_as(P(ctypes.c_int)),
      levels.ctypes.data_as(P(ctypes.c_int)))
    return iperm - 1

