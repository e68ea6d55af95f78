"""gb300_residual_noalloc: the residual entry point for callers that cannot
allocate device memory while they run.

It is called through the C ABI twice in a row (its scratch array keeps the
previous call's contents) and each result is checked against the library's
existing entry points -- gb300_matrix_mult for A x and gb300_vector_norm2
for the norm -- within the tolerance the other SpMV tests use (1e-13
relative), and against b - A x formed on the host in FP64 by scipy (within
1e-13 of sum_j |a_ij x_j| + |b_i|, the rounding bound of a row's dot
product).  Further calls must leave the device's free memory unchanged,
and an r that aliases x or b is rejected.  This file is collected last so
that a run stopping at the first failure has already run every other test;
it also passes on its own in a fresh process (the first call does the
per-device set-up).
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from getdp_gb300 import _lib
from getdp_gb300 import linalg as LA
from tests import golden_cases as G

pytestmark = pytest.mark.gpu

RTOL = 1e-13


@pytest.fixture(scope="module")
def lib():
    from getdp_gb300 import build
    build.build()
    return _lib.load()


def _reference(L, A, xv, bv):
    """r = b - A x through the existing entry points."""
    n = A.n
    x = LA.gVector(n)
    x.set(xv)
    y = LA.gVector(n)
    _lib.check(L.gb300_matrix_mult(A.h, x.h, y.h))
    r = bv - y.numpy()
    rv = LA.gVector(n)
    rv.set(r)
    nrm = ctypes.c_double()
    _lib.check(L.gb300_vector_norm2(rv.h, ctypes.byref(nrm)))
    return r, nrm.value


@pytest.mark.parametrize("name", ["el_p2_n3", "ms2d_n24", "eddy_n8"])
def test_residual_noalloc_matches_existing_entry_points(lib, name):
    d, p, dm = G.load(name)
    n = dm.n_dof
    A = LA.gMatrix(n)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    rng = np.random.default_rng(7)
    x = LA.gVector(n)
    b = LA.gVector(n)
    r = LA.gVector(n)
    for call in range(2):  # two calls in a row share the scratch array
        xv = rng.standard_normal(n)
        bv = d["b"] + rng.standard_normal(n) * (call + 1)
        x.set(xv)
        b.set(bv)
        nrm = ctypes.c_double(-1.0)
        _lib.check(lib.gb300_residual_noalloc(A.h, x.h, b.h, r.h, ctypes.byref(nrm)))
        r_ref, n_ref = _reference(lib, A, xv, bv)
        got = r.numpy()
        scale = np.max(np.abs(r_ref))
        assert np.all(np.abs(got - r_ref) <= RTOL * (np.abs(r_ref) + scale)), call
        assert abs(nrm.value - n_ref) <= RTOL * n_ref, (call, nrm.value, n_ref)
        # independent host product (FP64, scipy CSR)
        M = sp.csr_matrix((d["data"], d["indices"], d["indptr"]), shape=(n, n))
        r_host = bv - M @ xv
        bound = abs(M) @ np.abs(xv) + np.abs(bv)
        assert np.all(np.abs(got - r_host) <= RTOL * bound), call
        assert abs(nrm.value - np.linalg.norm(r_host)) <= RTOL * np.linalg.norm(bound), call


def _free_device_bytes():
    """cudaMemGetInfo from the CUDA runtime the library is linked with."""
    rt = ctypes.CDLL("libcudart.so.13")
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_residual_noalloc_allocates_nothing_and_rejects_aliases(lib):
    d, p, dm = G.load("ms2d_n24")
    n = dm.n_dof
    A = LA.gMatrix(n)
    A.set_csr(d["indptr"], d["indices"], d["data"])
    x, b, r = LA.gVector(n), LA.gVector(n), LA.gVector(n)
    x.set(np.linspace(-1.0, 1.0, n))
    b.set(d["b"])
    nrm = ctypes.c_double()
    # the first call sets up the device (kernel loading, symbol lookup)
    _lib.check(lib.gb300_residual_noalloc(A.h, x.h, b.h, r.h, ctypes.byref(nrm)))
    free0 = _free_device_bytes()
    for _ in range(5):
        _lib.check(lib.gb300_residual_noalloc(A.h, x.h, b.h, r.h, ctypes.byref(nrm)))
    assert _free_device_bytes() == free0
    # r must be a vector of its own
    assert lib.gb300_residual_noalloc(A.h, x.h, b.h, x.h, ctypes.byref(nrm)) == 1
    assert b"alias" in lib.gb300_last_error()
    assert lib.gb300_residual_noalloc(A.h, x.h, b.h, b.h, ctypes.byref(nrm)) == 1


def test_residual_noalloc_rejects_oversized_and_unassembled(lib):
    # one row beyond the maximum: rejected before anything runs
    big = LA.gMatrix(33554432 + 1)
    v = LA.gVector(4)
    nrm = ctypes.c_double()
    rc = lib.gb300_residual_noalloc(big.h, v.h, v.h, v.h, ctypes.byref(nrm))
    assert rc == 6 and b"exceed the maximum" in lib.gb300_last_error()
    # an unassembled matrix would need an allocation: rejected
    A = LA.gMatrix(4)
    LA.LinAlg_AddDoubleInMatrix(1.0, A, 0, 0)
    x, b, r = LA.gVector(4), LA.gVector(4), LA.gVector(4)
    rc = lib.gb300_residual_noalloc(A.h, x.h, b.h, r.h, ctypes.byref(nrm))
    assert rc == 1 and b"assembled" in lib.gb300_last_error()
