"""ORACLE — test infrastructure only.

CPU restatement of the reference's post-processing of a local quantity
(PostOperation Print[ {a} / {d a}, OnElementsOf | OnPoint ]): the value of
the field or of its curl from the element's basis functions at a point,
Pos_FemInterpolation.cpp (Pos_FemInterpolation, summing coefficient x basis
function over the element's DOFs), with the basis functions and maps of the
Generate path: BF_PerpendicularEdge (BF_Perpendicular.cpp:36-64) with Form2P
for the 2D curl, BF_Edge / BF_CurlEdge (BF_Edge.cpp:95-130, :452-485) with
Form1 / Form2 (Get_Geometry.cpp ChangeOfCoord_Form1 / Form2) in 3D.  The
point is located by testing every element (the reference's bucket search,
Pos_Search.cpp, finds the same element for a point strictly inside one).
Fixed unknowns are homogeneous (zero).
"""
from __future__ import annotations

import numpy as np

CURL_EDGE = np.array([[0., -2., 2.], [2., 0., -2.], [-2., 2., 0.],
                      [0., 0., 2.], [0., -2., 0.], [2., 0., 0.]])


def _dof_values(dm, x, nh):
    """Per element and local DOF the field coefficient of each harmonic:
    the unknown's value, or a fixed DOF's value (dm.fixed_values; 0 when the
    fixed DOFs are homogeneous)."""
    ed = dm.elem_dofs
    fv = getattr(dm, "fixed_values", None)
    vals = np.zeros(ed.shape + (nh,))
    for h in range(nh):
        fixed = 0.0
        if fv is not None:
            f = np.asarray(fv, np.float64).reshape(len(fv), -1)
            fixed = f[np.maximum(-ed - 1, 0), h]
        vals[..., h] = np.where(ed >= 0, x[np.maximum(ed, 0) + h], fixed)
    return vals


def _tri_geo(nodes, tri):
    P = nodes[tri]
    c11 = P[:, 1, 0] - P[:, 0, 0]
    c21 = P[:, 2, 0] - P[:, 0, 0]
    c12 = P[:, 1, 1] - P[:, 0, 1]
    c22 = P[:, 2, 1] - P[:, 0, 1]
    D = c11 * c22 - c12 * c21
    return P, c11, c21, c12, c22, D


def _tri_curls(c11, c21, c12, c22, D):
    gu = np.array([-1., 1., 0.])
    gv = np.array([-1., 0., 1.])
    s0, s1 = gv, -gu
    cx = (s0[None, :] * c11[:, None] + s1[None, :] * c21[:, None]) / D[:, None]
    cy = (s0[None, :] * c12[:, None] + s1[None, :] * c22[:, None]) / D[:, None]
    return cx, cy


def _tet_geo(nodes, tet):
    P = nodes[tet]
    J = np.stack([P[:, 1] - P[:, 0], P[:, 2] - P[:, 0], P[:, 3] - P[:, 0]], axis=1)
    # J[e, r, c]: row r = reference direction (u, v, w), column c = (x, y, z)
    D = np.linalg.det(J)
    Jinv = np.linalg.inv(J)
    return P, J, D, Jinv


def curl_on_elements(p, dm, x):
    """{d a} per element: 2D (ne, nh, 2), 3D (ne, 3)."""
    nodes, el = p.mesh.nodes, p.mesh.elems
    if p.formulation in ("magnetostatics2d", "eddy2d"):
        nh = 2 if p.formulation == "eddy2d" else 1
        _, c11, c21, c12, c22, D = _tri_geo(nodes, el)
        cx, cy = _tri_curls(c11, c21, c12, c22, D)
        a = _dof_values(dm, x, nh)
        return np.stack([np.einsum("ei,eih->eh", cx, a),
                         np.einsum("ei,eih->eh", cy, a)], axis=-1)
    if p.formulation == "curlcurl":
        _, J, D, _ = _tet_geo(nodes, el)
        a = _dof_values(dm, x, 1)[..., 0] * dm.elem_sign
        # Form2: J^T s / det, s the reference curl
        cu = np.einsum("ic,erc->eir", CURL_EDGE, J.transpose(0, 2, 1)) / D[:, None, None]
        return np.einsum("ei,eir->er", a, cu)
    raise ValueError(p.formulation)


def _edge_ref(u, v, w):
    return np.array([[1 - v - w, u, u], [v, 1 - u - w, v], [w, w, 1 - u - v],
                     [-v, u, 0.], [-w, 0., u], [0., -w, v]])


def at_points(p, dm, x, pts, tol=1e-10):
    """({a}, {d a}, element) at each point, as the GPU's at_points."""
    nodes, el = p.mesh.nodes, p.mesh.elems
    curls = curl_on_elements(p, dm, x)
    n = len(pts)
    if p.formulation in ("magnetostatics2d", "eddy2d"):
        nh = 2 if p.formulation == "eddy2d" else 1
        P, c11, c21, c12, c22, D = _tri_geo(nodes, el)
        a = _dof_values(dm, x, nh)
        fa = np.zeros((n, nh))
        fb = np.zeros((n, nh, 2))
        fe = -np.ones(n, np.int64)
        for q, (px, py, _) in enumerate(pts):
            dx, dy = px - P[:, 0, 0], py - P[:, 0, 1]
            u = (c22 * dx - c21 * dy) / D
            v = (-c12 * dx + c11 * dy) / D
            ok = np.nonzero((u >= -tol) & (v >= -tol) & (1 - u - v >= -tol))[0]
            if len(ok) == 0:
                continue
            e = ok[0]
            N = np.array([1 - u[e] - v[e], u[e], v[e]])
            fe[q] = e
            fa[q] = N @ a[e]
            fb[q] = curls[e]
        return fa, fb, fe
    if p.formulation == "curlcurl":
        P, J, D, Jinv = _tet_geo(nodes, el)
        a = _dof_values(dm, x, 1)[..., 0] * dm.elem_sign
        fa = np.zeros((n, 3))
        fb = np.zeros((n, 3))
        fe = -np.ones(n, np.int64)
        for q, pt in enumerate(pts):
            uvw = np.einsum("ec,ecr->er", pt[None, :] - P[:, 0], Jinv)
            l0 = 1 - uvw.sum(1)
            ok = np.nonzero((uvw >= -tol).all(1) & (l0 >= -tol))[0]
            if len(ok) == 0:
                continue
            e = ok[0]
            s = _edge_ref(*uvw[e])
            fe[q] = e
            # Form1: inverse Jacobian applied to the reference vector
            fa[q] = a[e] @ (s @ Jinv[e].T)
            fb[q] = curls[e]
        return fa, fb, fe
    raise ValueError(p.formulation)
