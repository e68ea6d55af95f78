"""ORACLE — test infrastructure only.

FP64 restatement of the learned-preconditioner network of
getdp_gb300/csrc/learned.cu (forward pass, energy-norm loss
(G r1 - e1)^T A (G r1 - e1) / e1^T A e1, or its two-level form after a
coarse correction, and its gradient with respect to every weight, A
symmetric), used to check the GPU's
hand-written forward and backward kernels.  Weights are used BF16-rounded
as on the GPU unless bf16=False (for finite-difference checks of the
gradient formulas themselves).
"""
from __future__ import annotations

import numpy as np

H, FIN, L = 32, 4, 3
OFF_WIN = 0
OFF_BIN = OFF_WIN + H * FIN
OFF_LAYER = OFF_BIN + H
LAYER = 2 * H * H + H
OFF_WO = OFF_LAYER + L * LAYER
OFF_CO = OFF_WO + H
OFF_WD = OFF_CO + 1
OFF_BD = OFF_WD + H
NPARAM = OFF_BD + 1


def bf16(x):
    """Round float32 values to BF16 (nearest, ties to even), as float64."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _unpack(w):
    P = {"Win": w[OFF_WIN:OFF_BIN].reshape(H, FIN), "bin": w[OFF_BIN:OFF_LAYER]}
    for l in range(L):
        o = OFF_LAYER + l * LAYER
        P[f"Ws{l}"] = w[o:o + H * H].reshape(H, H)
        P[f"Wn{l}"] = w[o + H * H:o + 2 * H * H].reshape(H, H)
        P[f"b{l}"] = w[o + 2 * H * H:o + LAYER]
    P["wo"], P["co"] = w[OFF_WO:OFF_CO], w[OFF_CO]
    P["wd"], P["bd"] = w[OFF_WD:OFF_BD], w[OFF_BD]
    return P


def graph(ip, ix, dv):
    n = len(ip) - 1
    rows = np.repeat(np.arange(n), np.diff(ip))
    diag = np.array([ip[i] + np.searchsorted(ix[ip[i]:ip[i + 1]], i) for i in range(n)])
    d = dv[diag]
    ds = 1.0 / np.sqrt(d)
    e = dv * ds[rows] * ds[ix]
    off = rows != ix
    feat = np.zeros((n, FIN))
    feat[:, 0] = 1.0
    np.add.at(feat[:, 1], rows[off], np.abs(e[off]))
    mx = np.zeros(n)
    np.maximum.at(mx, rows[off], np.abs(e[off]))
    feat[:, 2] = mx
    feat[:, 3] = np.diff(ip) / 8.0
    return {"n": n, "rows": rows, "cols": ix, "e": e, "off": off, "ds": ds, "feat": feat}


def forward(w, g, bf16_weights=True):
    w = bf16(w) if bf16_weights else np.asarray(w, np.float64)
    P = _unpack(w)
    rows, cols, e, off = g["rows"], g["cols"], g["e"], g["off"]
    z0 = g["feat"] @ P["Win"].T + P["bin"]
    h = [np.maximum(z0, 0.0)]
    m = []
    for l in range(L):
        mi = np.zeros_like(h[-1])
        np.add.at(mi, rows[off], e[off, None] * h[-1][cols[off]])
        z = h[-1] @ P[f"Ws{l}"].T + mi @ P[f"Wn{l}"].T + P[f"b{l}"]
        m.append(mi)
        h.append(np.maximum(z, 0.0))
    hL = h[-1]
    gval = np.where(off, np.sum(P["wo"] * hL[rows] * hL[cols], axis=1) + P["co"] * e,
                    hL[rows] @ P["wd"] + P["bd"])
    G = gval * g["ds"][rows] * g["ds"][cols]
    return G, {"P": P, "h": h, "m": m}


def loss_grad(w, g, r1, e1, A, bf16_weights=True, coarse=None):
    """(loss, gradient with respect to the weights, G); A is the (symmetric)
    system matrix as scipy.sparse; e1 may be None (a probe: S = r1^T D^-1
    r1 in place of e1^T A e1).  coarse = (P0, Ac^-1): the two-level loss
    (e1 - y)^T (A - A C A) (e1 - y) / S, C = P0 Ac^-1 P0^T."""
    G, c = forward(w, g, bf16_weights)
    P, h, m = c["P"], c["h"], c["m"]
    rows, cols, e, off = g["rows"], g["cols"], g["e"], g["off"]
    n = g["n"]
    y = np.zeros(n)
    np.add.at(y, rows, G * r1[cols])
    if e1 is not None:
        S = float(e1 @ (A @ e1))
    else:
        S = float(np.sum((r1 * g["ds"]) ** 2))
    Ay = A @ y
    loss = 1.0 + (float(y @ Ay) - 2.0 * float(r1 @ y)) / S
    wv = Ay - r1
    if coarse is not None:
        P0, Aci = coarse
        t = P0.T @ wv
        ec = Aci @ t
        loss -= float(t @ ec) / S
        wv = wv - A @ (P0 @ ec)
    dG = 2.0 * wv[rows] * r1[cols] / S
    dg = dG * g["ds"][rows] * g["ds"][cols]
    grad = np.zeros(NPARAM)
    hL = h[-1]
    grad[OFF_WO:OFF_CO] = np.sum((dg[off])[:, None] * hL[rows[off]] * hL[cols[off]], axis=0)
    grad[OFF_CO] = np.sum(dg[off] * e[off])
    grad[OFF_WD:OFF_BD] = np.sum((dg[~off])[:, None] * hL[rows[~off]], axis=0)
    grad[OFF_BD] = np.sum(dg[~off])
    # position of the transposed entry of each (i, j)
    key = rows.astype(np.int64) * n + cols
    tkey = cols.astype(np.int64) * n + rows
    order = np.argsort(key)
    tpos = order[np.searchsorted(key[order], tkey)]
    dh = np.zeros_like(hL)
    dsum = dg + dg[tpos]
    np.add.at(dh, rows[off], (dsum[off])[:, None] * P["wo"] * hL[cols[off]])
    np.add.at(dh, rows[~off], (dg[~off])[:, None] * P["wd"])
    for l in reversed(range(L)):
        dz = dh * (h[l + 1] > 0)
        o = OFF_LAYER + l * LAYER
        grad[o:o + H * H] = (dz.T @ h[l]).ravel()
        grad[o + H * H:o + 2 * H * H] = (dz.T @ m[l]).ravel()
        grad[o + 2 * H * H:o + LAYER] = dz.sum(0)
        dm = dz @ P[f"Wn{l}"]
        dh = dz @ P[f"Ws{l}"]
        np.add.at(dh, rows[off], e[tpos[off], None] * dm[cols[off]])
    dz0 = dh * (h[0] > 0)
    grad[OFF_WIN:OFF_BIN] = (dz0.T @ g["feat"]).ravel()
    grad[OFF_BIN:OFF_LAYER] = dz0.sum(0)
    return loss, grad, G
