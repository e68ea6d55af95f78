"""Post-processing on the GPU (PostOperation Print[ {d a}, OnElementsOf ];
Print[ {a} / {d a}, OnPoint ]): the calls the reference's Pos_Print.cpp /
Pos_FemInterpolation.cpp make per element and per point, here one batched
call each."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check

KINDS = {_lib.TERM_TRI3_MAGNETOSTATIC: (2, 1), _lib.TERM_TRI3_EDDY_COMPLEX: (2, 2),
         _lib.TERM_TET4_EDGE_CURLCURL: (3, 1)}


def _shape(batch):
    if batch.kind not in KINDS:
        raise ValueError(f"post-processing: unsupported term kind {batch.kind}")
    return KINDS[batch.kind]


def curl_on_elements(batch, x) -> np.ndarray:
    """{d a} per element: (n_elems, nh, 2) in 2D (real and imaginary
    harmonics), (n_elems, 3) in 3D."""
    dim, nh = _shape(batch)
    ne = batch.n_elems
    out = np.zeros(ne * (2 * nh if dim == 2 else 3), np.float64)
    check(_lib.load().gb300_post_elements(ctypes.byref(batch), x.h,
                                          out.ctypes.data_as(ctypes.c_void_p)))
    return out.reshape(ne, nh, 2) if dim == 2 else out.reshape(ne, 3)


def at_points(batch, x, xyz):
    """({a}, {d a}, element) at each point (rows of xyz): 2D a_z per
    harmonic (np, nh) and curl (np, nh, 2); 3D a (np, 3) and curl (np, 3);
    element -1 outside the mesh."""
    dim, nh = _shape(batch)
    pts = np.ascontiguousarray(np.asarray(xyz, np.float64).reshape(-1, 3))
    n = pts.shape[0]
    fa = np.zeros(n * (nh if dim == 2 else 3))
    fb = np.zeros(n * (2 * nh if dim == 2 else 3))
    fe = np.zeros(n, np.int32)
    check(_lib.load().gb300_post_points(
        ctypes.byref(batch), x.h, n, pts.ctypes.data_as(ctypes.c_void_p),
        fa.ctypes.data_as(ctypes.c_void_p), fb.ctypes.data_as(ctypes.c_void_p),
        fe.ctypes.data_as(ctypes.c_void_p)))
    if dim == 2:
        return fa.reshape(n, nh), fb.reshape(n, nh, 2), fe
    return fa.reshape(n, 3), fb.reshape(n, 3), fe
