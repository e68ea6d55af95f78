"""Seeded synthetic meshes and problem descriptions for the GetDP hot path.

The reference measures on no public dataset; these generators produce the
meshes, materials and sources that its benchmark configurations describe
(2D P1 magnetostatics, 3D P2 elasticity, 3D Whitney-edge curl-curl, complex
2D eddy currents), at any size, from a seed.

Besides the in-memory arrays they write the two files GetDP itself reads:
a Gmsh MSH 2.2 mesh (the only mesh format GetDP reads without the Gmsh
library, src/kernel/GeoData.cpp:573-603) and a ``.pro`` problem file, so the
same problem can be run through the unchanged reference.

The host-side "PRE" step is mirrored here too: element -> DOF tables in
GetDP's own DOF numbering.  GetDP numbers unknowns by an in-order walk of its
DOF tree keyed by (NumType, Entity, Harmonic) (src/kernel/DofData.cpp:36-45,
:1299-1319), so unknowns follow (basis function, entity number, harmonic)
order; edges are numbered on first touch, constraint groups first
(src/kernel/ExtendedGroup.cpp:206-255, src/kernel/GeoEntity.cpp:436-485).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

MU0 = 4.0e-7 * math.pi

# element kinds understood by the assembly kernels
TRI3, TET4, TET10 = "tri3", "tet4", "tet10"
_MSH_TYPE = {"line2": 1, "tri3": 2, "tet4": 4, "tri6": 9, "tet10": 11}


@dataclasses.dataclass
class Mesh:
    """Nodes (0-based rows, GetDP node number = row + 1) and elements."""

    nodes: np.ndarray  # (nn, 3) float64
    kind: str  # volume element kind
    elems: np.ndarray  # (ne, nv) int32, 0-based node indices
    region: np.ndarray  # (ne,) int32 physical tag of each volume element
    bnd_kind: str  # boundary element kind ('line2', 'tri3', 'tri6')
    bnd: np.ndarray  # (nb, nbv) int32
    bnd_region: np.ndarray  # (nb,) int32

    @property
    def n_nodes(self) -> int:
        return self.nodes.shape[0]

    @property
    def n_elems(self) -> int:
        return self.elems.shape[0]


# --------------------------------------------------------------------------
# mesh generators
# --------------------------------------------------------------------------

def square_tri_mesh(n: int, seed: int, jitter: float = 0.2) -> Mesh:
    """Unit square, n x n cells, each cut on the (i,j)-(i+1,j+1) diagonal.

    Interior nodes are jittered by a seeded uniform +-jitter*h; the boundary
    stays straight.  Node (i, j) has 0-based index j*(n+1)+i.
    """
    h = 1.0 / n
    i, j = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="xy")
    xy = np.stack([i.ravel() * h, j.ravel() * h], axis=1)
    rng = np.random.default_rng(seed)
    interior = ((i > 0) & (i < n) & (j > 0) & (j < n)).ravel()
    xy[interior] += rng.uniform(-jitter * h, jitter * h, size=(interior.sum(), 2))
    nodes = np.zeros((xy.shape[0], 3))
    nodes[:, :2] = xy
    ci, cj = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    a = (cj * (n + 1) + ci).ravel()
    b, c, d = a + 1, a + n + 2, a + n + 1
    tris = np.empty((2 * n * n, 3), dtype=np.int32)
    tris[0::2] = np.stack([a, b, c], 1)
    tris[1::2] = np.stack([a, c, d], 1)
    # boundary lines, counter-clockwise from the origin
    s = np.arange(n)
    bottom = np.stack([s, s + 1], 1)
    right = np.stack([n + s * (n + 1), n + (s + 1) * (n + 1)], 1)
    top = np.stack([n * (n + 1) + n - s, n * (n + 1) + n - s - 1], 1)
    left = np.stack([(n - s) * (n + 1), (n - s - 1) * (n + 1)], 1)
    lines = np.concatenate([bottom, right, top, left]).astype(np.int32)
    return Mesh(nodes, TRI3, tris, np.zeros(len(tris), np.int32), "line2",
                lines, np.full(len(lines), 10, np.int32))


def _kuhn_tets(n: int):
    """Unit cube of n^3 hexes, each split into the 6 Kuhn tetrahedra that
    share its main diagonal (a conforming mesh), positively oriented."""
    h = 1.0 / n
    g = np.arange(n + 1)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1).astype(np.float64) * h
    # keep GetDP-friendly ordering: node index = (k*(n+1)+j)*(n+1)+i
    idx = lambda i, j, k: (k * (n + 1) + j) * (n + 1) + i  # noqa: E731
    order = np.empty((n + 1) ** 3, dtype=np.int64)
    order[idx(X.ravel(), Y.ravel(), Z.ravel())] = np.arange((n + 1) ** 3)
    nodes = nodes[order]
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    # sort cells k-major so that neighbouring elements are close in memory
    o = np.lexsort((ci, cj, ck))
    ci, cj, ck = ci[o], cj[o], ck[o]
    unit = np.eye(3, dtype=np.int64)
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    tets = []
    for p in perms:
        v0 = np.stack([ci, cj, ck], 1)
        v1 = v0 + unit[p[0]]
        v2 = v1 + unit[p[1]]
        v3 = v2 + unit[p[2]]
        t = np.stack([idx(*v.T) for v in (v0, v1, v2, v3)], 1)
        # orientation sign = parity of the permutation
        odd = p in [(0, 2, 1), (1, 0, 2), (2, 1, 0)]
        if odd:
            t = t[:, [0, 2, 1, 3]]
        tets.append(t)
    tets = np.stack(tets, 1).reshape(-1, 4).astype(np.int32)
    return nodes, tets


def _cube_boundary_tris(n: int, faces=("x0", "x1", "y0", "y1", "z0", "z1")):
    idx = lambda i, j, k: (k * (n + 1) + j) * (n + 1) + i  # noqa: E731
    s = np.arange(n)
    u, v = np.meshgrid(s, s, indexing="ij")
    u, v = u.ravel(), v.ravel()
    out = []
    for f in faces:
        c = 0 if f[1] == "0" else n
        if f[0] == "x":
            q = lambda a, b: idx(np.full_like(a, c), a, b)  # noqa: E731
        elif f[0] == "y":
            q = lambda a, b: idx(a, np.full_like(a, c), b)  # noqa: E731
        else:
            q = lambda a, b: idx(a, b, np.full_like(a, c))  # noqa: E731
        p00, p10, p11, p01 = q(u, v), q(u + 1, v), q(u + 1, v + 1), q(u, v + 1)
        # the Kuhn split cuts every face square on its (0,0)-(1,1) diagonal
        out.append(np.stack([p00, p10, p11], 1))
        out.append(np.stack([p00, p11, p01], 1))
    return np.concatenate(out).astype(np.int32)


# GetDP / Gmsh 10-node tetrahedron: nodes 5..10 on edges (1,2),(2,3),(1,3),
# (1,4),(3,4),(2,4)  (src/functions/BF_Node.cpp:174-186)
TET10_EDGES = np.array([[0, 1], [1, 2], [0, 2], [0, 3], [2, 3], [1, 3]])
TRI6_EDGES = np.array([[0, 1], [1, 2], [0, 2]])


def _add_midnodes(nodes, tets, tris):
    e = tets[:, TET10_EDGES].reshape(-1, 2)
    e = np.sort(e, axis=1)
    key = e[:, 0].astype(np.int64) * nodes.shape[0] + e[:, 1]
    uk, inv = np.unique(key, return_inverse=True)
    a, b = uk // nodes.shape[0], uk % nodes.shape[0]
    mid = 0.5 * (nodes[a] + nodes[b])
    nn = nodes.shape[0]
    tet10 = np.concatenate([tets, (nn + inv.reshape(-1, 6)).astype(np.int32)], 1)
    te = np.sort(tris[:, TRI6_EDGES].reshape(-1, 2), axis=1)
    tkey = te[:, 0].astype(np.int64) * nn + te[:, 1]
    pos = np.searchsorted(uk, tkey)
    assert np.all(uk[pos] == tkey)
    tri6 = np.concatenate([tris, (nn + pos.reshape(-1, 3)).astype(np.int32)], 1)
    return np.concatenate([nodes, mid]), tet10, tri6


# --------------------------------------------------------------------------
# problems
# --------------------------------------------------------------------------

@dataclasses.dataclass
class Problem:
    """A mesh plus everything a Galerkin term needs per element."""

    name: str
    mesh: Mesh
    formulation: str  # 'magnetostatics2d', 'elasticity', 'curlcurl', 'eddy2d'
    coef: np.ndarray  # per-element scalar coefficient (nu, or E)
    source: np.ndarray  # per-element source (J_z, or flags) ; shape depends
    params: dict


def magnetostatics_2d(n: int, seed: int = 1, jitter: float = 0.2,
                      dirichlet=None) -> Problem:
    """a_z nodal P1 magnetostatics on the unit square (BF_PerpendicularEdge).

    nu = 1/(mu0*mu_r), mu_r = 1000 inside the disk r < 0.25 about (0.5, 0.5);
    J_z = +1e6 A/m^2 in [0.1,0.3]x[0.4,0.6], -1e6 in [0.7,0.9]x[0.4,0.6];
    a = 0 on the outer boundary.  Regions are chosen by element centroid:
    1 iron, 2 air, 3 positive source, 4 negative source.
    """
    m = square_tri_mesh(n, seed, jitter)
    c = m.nodes[m.elems].mean(axis=1)
    reg = np.full(m.n_elems, 2, np.int32)
    reg[(c[:, 0] - 0.5) ** 2 + (c[:, 1] - 0.5) ** 2 < 0.25 ** 2] = 1
    in_y = (c[:, 1] > 0.4) & (c[:, 1] < 0.6)
    reg[in_y & (c[:, 0] > 0.1) & (c[:, 0] < 0.3)] = 3
    reg[in_y & (c[:, 0] > 0.7) & (c[:, 0] < 0.9)] = 4
    m.region = reg
    nu = np.where(reg == 1, 1.0 / (1000.0 * MU0), 1.0 / MU0)
    js = np.zeros(m.n_elems)
    js[reg == 3] = 1.0e6
    js[reg == 4] = -1.0e6
    return Problem(f"magnetostatics2d_n{n}", m, "magnetostatics2d", nu, js,
                   {"n": n, "seed": seed, "jitter": jitter, "dirichlet": dirichlet})


def gaussian_field(points: np.ndarray, seed: int, corr: float,
                   grid: int = 256) -> np.ndarray:
    """Unit-variance Gaussian random field with covariance exp(-d^2 / (2
    corr^2)) on the unit square, sampled at points (nearest node of a
    periodic FFT grid of grid^2 nodes)."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(grid, d=1.0 / grid) * 2.0 * np.pi
    kx, ky = np.meshgrid(k, k, indexing="ij")
    spec = np.exp(-0.25 * corr * corr * (kx * kx + ky * ky))  # sqrt of the PSD
    noise = rng.standard_normal((grid, grid))
    f = np.real(np.fft.ifft2(np.fft.fft2(noise) * spec))
    f = (f - f.mean()) / f.std()
    i = np.clip(np.rint(points[:, 0] * (grid - 1)).astype(int), 0, grid - 1)
    j = np.clip(np.rint(points[:, 1] * (grid - 1)).astype(int), 0, grid - 1)
    return f[i, j]


def nonlinear_2d(n: int, seed: int = 5, jitter: float = 0.2, corr: float = 0.05,
                 sigma_log: float = 1.0, n_blobs: int = 8,
                 blob_radius: float = 0.02, dirichlet=None) -> Problem:
    """Nonlinear a_z P1 magnetostatics on the unit square.

    nu(x, |B|) = nu0(x) (1 + 999 exp(-|B|^2 / 1.5^2))^-1 with nu0 =
    exp(sigma_log g(x)) / mu0, g a seeded Gaussian random field of
    correlation length corr (per element, at the centroid); J_z = sum of
    n_blobs seeded Gaussian blobs of amplitude +-1e6 A/m^2 and radius
    blob_radius (per element at the centroid); a = 0 on the boundary.
    Newton on the reference's Newton-Raphson formulation
    (Lib_Magnetostatics_a_phi.pro: nu[{d a}] {d a} + dhdb[{d a}] (Dof{d a}
    - {d a})).
    """
    m = square_tri_mesh(n, seed, jitter)
    c = m.nodes[m.elems].mean(axis=1)
    nu0 = np.exp(sigma_log * gaussian_field(c, seed + 1, corr)) / MU0
    rng = np.random.default_rng(seed + 2)
    js = np.zeros(m.n_elems)
    for _ in range(n_blobs):
        cx, cy = rng.uniform(0.15, 0.85, 2)
        s = rng.choice([-1.0, 1.0])
        js += s * 1.0e6 * np.exp(-((c[:, 0] - cx) ** 2 + (c[:, 1] - cy) ** 2) /
                                 (2 * blob_radius ** 2))
    m.region = np.full(m.n_elems, 1, np.int32)
    return Problem(f"nonlinear2d_n{n}", m, "nonlinear2d", nu0, js,
                   {"n": n, "seed": seed, "jitter": jitter, "b_sat2": 1.5 ** 2,
                    "k_sat": 999.0, "dirichlet": dirichlet})


def elasticity_p2(n: int, seed: int = 2, sigma_log: float = 0.5,
                  dirichlet=None) -> Problem:
    """3D linear elasticity, 10-node tetrahedra, per-element lognormal E.

    Unit cube of n^3 hexes x 6 Kuhn tets; E median 200 GPa, sigma_log 0.5;
    Poisson 0.3; gravity rho*g = 7800*9.81 along -z; face x = 0 clamped.
    """
    nodes, tets = _kuhn_tets(n)
    x0 = _cube_boundary_tris(n, faces=("x0",))
    nodes, tet10, tri6 = _add_midnodes(nodes, tets, x0)
    rng = np.random.default_rng(seed)
    E = 200.0e9 * np.exp(sigma_log * rng.standard_normal(len(tet10)))
    m = Mesh(nodes, TET10, tet10, np.ones(len(tet10), np.int32), "tri6", tri6,
             np.full(len(tri6), 20, np.int32))
    return Problem(f"elasticity_p2_n{n}", m, "elasticity", E,
                   np.zeros(len(tet10)),
                   {"n": n, "seed": seed, "poisson": 0.3, "rho": 7800.0,
                    "g": 9.81, "dirichlet": dirichlet})


# Analytic potential of the toroidal source current: T = h(z) Psi(r) e_z about
# the vertical axis through (0.5, 0.5), whose curl is the azimuthal current
# J = -dPsi/dr h(z) e_phi = J0 beta((r - RC)/WR) beta((z - ZC)/WZ) e_phi with
# the C2 bump beta(s) = (1 - s^2)^3 on |s| < 1: a coil of 1e6 A/m^2 peak in
# 0.32 < r < 0.45, 0.3 < z < 0.7, around the iron cube.
COIL_RC, COIL_WR, COIL_ZC, COIL_WZ = 0.385, 0.065, 0.5, 0.2


def _bump_integral(s):
    """int_{-1}^{s} (1 - t^2)^3 dt, clamped to [0, 32/35]."""
    s = np.clip(s, -1.0, 1.0)
    return s - s ** 3 + 0.6 * s ** 5 - s ** 7 / 7.0 + 16.0 / 35.0


def toroidal_potential_z(P: np.ndarray, J0: float) -> np.ndarray:
    """z component of T at points P (..., 3); T has no x, y components."""
    r = np.hypot(P[..., 0] - 0.5, P[..., 1] - 0.5)
    sz = np.clip((P[..., 2] - COIL_ZC) / COIL_WZ, -1.0, 1.0)
    h = (1.0 - sz * sz) ** 3
    return h * (-J0 * COIL_WR * _bump_integral((r - COIL_RC) / COIL_WR))


def edge_circulation(a: np.ndarray, b: np.ndarray, J0: float, ng: int = 6) -> np.ndarray:
    """int_a^b T . dl along straight edges (Gauss-Legendre, ng points)."""
    t, w = np.polynomial.legendre.leggauss(ng)
    t, w = 0.5 * (t + 1.0), 0.5 * w
    d = b - a
    acc = np.zeros(len(a))
    for tk, wk in zip(t, w):
        acc += wk * toroidal_potential_z(a + tk * d, J0)
    return acc * d[:, 2]


# the constant curls of the six Whitney functions of the reference tet
# (BF_CurlEdge, src/functions/BF_Edge.cpp:452-485), local edge order of
# GeoEntity.h:214-215
_CURL_EDGE_REF = np.array([[0., -2., 2.], [2., 0., -2.], [-2., 2., 0.],
                           [0., 0., 2.], [0., -2., 0.], [2., 0., 0.]])


def curl_of_edge_interpolant(m: Mesh, J0: float) -> np.ndarray:
    """Per element, the curl of the Whitney-edge interpolant of T: J_K =
    sum_i t_i curl(w_i), t_i the circulation of T along edge i oriented from
    the lower to the higher global node number.  The field is constant per
    element and its normal component is continuous across faces, so it is
    exactly divergence-free in the discrete sense: the right-hand side it
    gives is orthogonal to every discrete gradient (to rounding), which the
    nearly singular curl-curl operator (1e-6 mass regularisation) needs."""
    x = m.nodes[m.elems]
    c = np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], 1)
    D = np.linalg.det(c)
    J = np.zeros((m.n_elems, 3))
    for i, (la, lb) in enumerate(TET4_EDGES):
        na, nb = m.elems[:, la], m.elems[:, lb]
        lo, hi = np.minimum(na, nb), np.maximum(na, nb)
        t = edge_circulation(m.nodes[lo], m.nodes[hi], J0)
        sg = np.where(na < nb, 1.0, -1.0)
        cu = np.einsum("erc,er->ec", c, _CURL_EDGE_REF[i][None, :] * sg[:, None]) / D[:, None]
        J += t[:, None] * cu
    return J


def curlcurl_edge(n: int, seed: int = 3) -> Problem:
    """3D magnetostatics with first-order Whitney edge elements (BF_Edge).

    Iron cube [0.3,0.7]^3 with mu_r = 500 (by element centroid); a toroidal
    source current of 1e6 A/m^2 peak circulating about the vertical axis
    through (0.5, 0.5) around the iron, given analytically as the curl of the
    potential T (toroidal_potential_z) and taken per element as the curl of
    T's edge interpolant (curl_of_edge_interpolant: divergence-free in the
    discrete sense); regularisation 1e-6*nu*mass; n x a = 0 on the whole
    boundary.  ``source`` is (n_elems, 3).  Regions: 1 air, 2 iron, 3
    elements carrying current.
    """
    nodes, tets = _kuhn_tets(n)
    bt = _cube_boundary_tris(n)
    c = nodes[tets].mean(axis=1)
    reg = np.ones(len(tets), np.int32)
    iron = np.all((c > 0.3) & (c < 0.7), axis=1)
    reg[iron] = 2
    m = Mesh(nodes, TET4, tets, reg, "tri3", bt, np.full(len(bt), 30, np.int32))
    J0 = 1.0e6
    js = curl_of_edge_interpolant(m, J0)
    reg[~iron & np.any(js != 0.0, axis=1)] = 3
    nu = np.where(reg == 2, 1.0 / (500.0 * MU0), 1.0 / MU0)
    return Problem(f"curlcurl_edge_n{n}", m, "curlcurl", nu, js,
                   {"n": n, "seed": seed, "J0": J0, "reg": 1.0e-6})


def eddy_2d(n: int, seed: int = 4, freq: Optional[float] = None,
            jitter: float = 0.2, dirichlet=None) -> Problem:
    """Complex (time-harmonic) a_z P1 eddy-current problem on the unit square.

    sigma = 5.8e7 S/m in 1-4 seeded disks (radius 0.05-0.15), frequency
    log-uniform in [10 Hz, 10 kHz] unless given, the two source rectangles
    of the magnetostatic case (which take precedence over conductors),
    a = 0 on the boundary.  Regions: 2 air, 3/4 sources, 5 conductor.
    """
    m = square_tri_mesh(n, seed, jitter)
    rng = np.random.default_rng(seed + 1000)
    nd = int(rng.integers(1, 5))
    disks = [(rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8),
              rng.uniform(0.05, 0.15)) for _ in range(nd)]
    if freq is None:
        freq = float(10.0 ** rng.uniform(1.0, 4.0))
    c = m.nodes[m.elems].mean(axis=1)
    reg = np.full(m.n_elems, 2, np.int32)
    for (cx, cy, r) in disks:
        reg[(c[:, 0] - cx) ** 2 + (c[:, 1] - cy) ** 2 < r * r] = 5
    in_y = (c[:, 1] > 0.4) & (c[:, 1] < 0.6)
    reg[in_y & (c[:, 0] > 0.1) & (c[:, 0] < 0.3)] = 3
    reg[in_y & (c[:, 0] > 0.7) & (c[:, 0] < 0.9)] = 4
    m.region = reg
    nu = np.full(m.n_elems, 1.0 / MU0)
    sigma = np.where(reg == 5, 5.8e7, 0.0)
    js = np.zeros(m.n_elems)
    js[reg == 3] = 1.0e6
    js[reg == 4] = -1.0e6
    return Problem(f"eddy2d_n{n}", m, "eddy2d", nu, js,
                   {"n": n, "seed": seed, "freq": freq, "sigma": sigma,
                    "disks": disks, "dirichlet": dirichlet})


# --------------------------------------------------------------------------
# GetDP PRE mirror: DOF numbering and element -> DOF tables
# --------------------------------------------------------------------------

@dataclasses.dataclass
class DofMap:
    """Element -> equation/unknown table in GetDP's numbering (0-based).

    elem_dofs[e, k] is the 0-based unknown number of local DOF k of element
    e, or -1 when that DOF is fixed (Dirichlet, eliminated into the RHS).
    elem_sign[e, k] is the orientation sign of edge DOFs (+-1), 1 otherwise.
    """

    n_dof: int
    elem_dofs: np.ndarray  # (ne, nloc) int32
    elem_sign: np.ndarray  # (ne, nloc) int8
    ncomp: int = 1
    nharm: int = 1
    edges: Optional[np.ndarray] = None  # (n_edges, 2) global edge nodes
    # non-homogeneous Dirichlet: fixed DOF k has value fixed_values[k]
    # ((n_fixed, 2) re/im for two harmonics) and elem_dofs holds -1-k for it;
    # None when every fixed DOF is 0 (elem_dofs then holds -1)
    fixed_values: Optional[np.ndarray] = None


# Named sets of non-homogeneous Dirichlet data, one (c0, cx, cy, cz) per
# field component: a generator's ``dirichlet`` may be a set number.
DIRICHLET_SETS = {
    1: [(1.0e-3, 2.0e-3, -1.5e-3, 0.0)],                    # a_z (2D)
    2: [(0.0, 0.0, 0.0, 0.0), (0.0, 0.0, 0.0, 0.0),
        (0.0, 0.0, -2.0e-5, 1.0e-5)],                        # (ux, uy, uz)
}


def dirichlet_coefs(g):
    """None, a DIRICHLET_SETS number, or per-component coefficient tuples."""
    if g is None:
        return None
    return DIRICHLET_SETS[int(g)] if isinstance(g, (int, np.integer)) else g


def dirichlet_values(nodes: np.ndarray, coefs) -> np.ndarray:
    """g = c0 + cx X + cy Y + cz Z at the nodes, evaluated left to right as
    GetDP evaluates the constraint expression written by constraint_expr."""
    c0, cx, cy, cz = coefs
    return c0 + cx * nodes[:, 0] + cy * nodes[:, 1] + cz * nodes[:, 2]


def constraint_expr(coefs) -> str:
    c0, cx, cy, cz = coefs
    return f"{c0!r} + {cx!r}*X[] + {cy!r}*Y[] + {cz!r}*Z[]"


def nodal_dofmap(m: Mesh, ncomp: int = 1, nharm: int = 1, dirichlet=None) -> DofMap:
    """BF_Node / BF_PerpendicularEdge on NodesOf[All] with the boundary group
    fixed: a = 0, or with ``dirichlet`` (one (c0, cx, cy, cz) per component)
    a = c0 + cx X + cy Y + cz Z at each fixed node (real for two harmonics).
    Unknowns: (component, node, harmonic) sorted, i.e. component-major across
    function spaces (their basis functions carry increasing NumType) and
    harmonic-minor (DofData.cpp:1287-1295).  Fixed DOFs with values are
    numbered component by component in node order."""
    used = np.zeros(m.n_nodes, bool)
    used[m.elems.ravel()] = True
    fixed = np.zeros(m.n_nodes, bool)
    fixed[m.bnd.ravel()] = True
    unknown = used & ~fixed
    num = np.full(m.n_nodes, -1, np.int64)
    num[unknown] = np.arange(unknown.sum())
    nu = int(unknown.sum())
    nloc = m.elems.shape[1]
    # local DOF order: component-major over the element's nodes (GetDP keeps
    # one QuantityStorage per quantity; each Galerkin term uses one of them)
    fnum = np.full(m.n_nodes, -1, np.int64)
    fixed_nodes = np.flatnonzero(used & fixed)
    fnum[fixed_nodes] = np.arange(len(fixed_nodes))
    nf = len(fixed_nodes)
    blocks = []
    for c in range(ncomp):
        for h in range(nharm):
            base = num[m.elems]
            fx = -1 if dirichlet is None else -1 - (c * nf + fnum[m.elems])
            blocks.append(np.where(base >= 0, (c * nu + base) * nharm + h, fx))
    if nharm == 1:
        dofs = np.concatenate(blocks, axis=1)
    else:
        # complex: harmonic pairs are consecutive numbers; keep harmonic 0 in
        # the table (the assembly adds harmonic 1 as +1)
        dofs = np.concatenate(blocks[0::nharm], axis=1)
    fv = None
    if dirichlet is not None:
        fv = np.concatenate([dirichlet_values(m.nodes[fixed_nodes], dirichlet[c])
                             for c in range(ncomp)])
        if nharm == 2:
            fv = np.stack([fv, np.zeros_like(fv)], 1)
    return DofMap(nu * ncomp * nharm, dofs.astype(np.int32),
                  np.ones(dofs.shape, np.int8), ncomp, nharm, fixed_values=fv)


TET4_EDGES = np.array([[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]])
TRI3_EDGES_GETDP = np.array([[0, 1], [0, 2], [1, 2]])


def edge_dofmap(m: Mesh) -> DofMap:
    """BF_Edge on EdgesOf[All], n x a = 0 on EdgesOf[boundary].

    Edge numbers are given on first touch: the constraint's boundary group
    creates its edges first (boundary elements in mesh order), then the
    volume loop (ExtendedGroup.cpp:227-230, GeoEntity.cpp:436-485).  The
    edge is stored as (min node, max node); its sign in an element is +1
    when the element's local edge runs from the lower to the higher global
    node number (GeoEntity.h:214-215 local edges (1,2),(1,3),(1,4),(2,3),
    (2,4),(3,4); triangle (1,2),(1,3),(2,3)).
    """
    nn = m.n_nodes
    be = m.bnd[:, TRI3_EDGES_GETDP].reshape(-1, 2)
    ve = m.elems[:, TET4_EDGES].reshape(-1, 2)
    # touch order: the first volume element's DOF lookup creates its edges,
    # then its constraint treatment generates the boundary group (all
    # boundary elements), then the element loop continues
    alle = np.concatenate([ve[:6], be, ve])
    key = np.minimum(alle[:, 0], alle[:, 1]).astype(np.int64) * nn + \
        np.maximum(alle[:, 0], alle[:, 1])
    uk, first = np.unique(key, return_index=True)
    # first-touch number of every unique edge
    order = np.argsort(first, kind="stable")
    edge_num = np.empty(len(uk), np.int64)
    edge_num[order] = np.arange(len(uk))
    vpos = np.searchsorted(uk, key[6 + len(be):])
    bpos = np.searchsorted(uk, key[6:6 + len(be)])
    fixed = np.zeros(len(uk), bool)
    fixed[bpos] = True
    # unknowns in increasing edge number
    en_fixed = np.zeros(len(uk), bool)
    en_fixed[edge_num[fixed]] = True
    num_by_edge = np.full(len(uk), -1, np.int64)
    num_by_edge[~en_fixed] = np.arange((~en_fixed).sum())
    dofs = num_by_edge[edge_num[vpos]].reshape(-1, 6)
    sign = np.where(ve[:, 0] < ve[:, 1], 1, -1).reshape(-1, 6).astype(np.int8)
    edges = np.stack([uk // nn, uk % nn], 1)[order]
    return DofMap(int((~en_fixed).sum()), dofs.astype(np.int32), sign,
                  edges=edges)


def cell_aggregates(p: Problem, dm: DofMap, cells: int):
    """Aggregates of the unknowns of a nodal scalar problem for the
    two-level preconditioners: the cells of a uniform grid of `cells` per
    side over the mesh's bounding box, each unknown in the cell that holds
    its node, empty cells dropped.  Returns (agg, n_agg)."""
    elems = p.mesh.elems
    if dm.elem_dofs.shape[1] != elems.shape[1] or dm.ncomp != 1 or dm.nharm != 1:
        raise ValueError("cell_aggregates: nodal scalar problems only")
    node_of = np.full(dm.n_dof, -1, np.int64)
    m = dm.elem_dofs >= 0
    node_of[dm.elem_dofs[m]] = elems[m]
    if np.any(node_of < 0):
        raise ValueError("cell_aggregates: an unknown belongs to no element")
    xyz = p.mesh.nodes[node_of]
    lo = p.mesh.nodes.min(axis=0)
    span = p.mesh.nodes.max(axis=0) - lo
    key = np.zeros(dm.n_dof, np.int64)
    for d in range(xyz.shape[1]):
        if span[d] <= 0:
            continue
        c = np.clip(((xyz[:, d] - lo[d]) / span[d] * cells).astype(np.int64), 0, cells - 1)
        key = key * cells + c
    _, agg = np.unique(key, return_inverse=True)
    agg = agg.reshape(-1).astype(np.int32)
    return agg, int(agg.max()) + 1


def dofmap_for(p: Problem) -> DofMap:
    g = dirichlet_coefs(p.params.get("dirichlet"))
    if p.formulation == "magnetostatics2d":
        return nodal_dofmap(p.mesh, dirichlet=g)
    if p.formulation == "eddy2d":
        return nodal_dofmap(p.mesh, nharm=2, dirichlet=g)
    if p.formulation == "nonlinear2d":
        return nodal_dofmap(p.mesh, dirichlet=g)
    if p.formulation == "elasticity":
        return nodal_dofmap(p.mesh, ncomp=3, dirichlet=g)
    if p.formulation == "curlcurl":
        return edge_dofmap(p.mesh)
    raise ValueError(p.formulation)


# --------------------------------------------------------------------------
# batches of independent problems (frequency / material sweeps)
# --------------------------------------------------------------------------

def eddy_sweep(n_problems: int = 512, seed: int = 7, n_min: int = 32,
               n_max: int = 160) -> list:
    """Independent complex eddy-current problems of uneven size: side n
    drawn uniformly from {n_min..n_max} cells, and per problem its own
    seeded jitter, 1-4 conductor disks and log-uniform frequency in
    [10 Hz, 10 kHz] (eddy_2d)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(n_min, n_max + 1, size=n_problems)
    return [eddy_2d(int(n), seed=int(seed * 100003 + k)) for k, n in enumerate(sizes)]


@dataclasses.dataclass
class Batch:
    """Independent problems as one system with diagonal blocks: problem k
    owns unknowns offsets[k]..offsets[k+1] (its own GetDP numbering shifted
    by offsets[k]) and nodes node_offsets[k]..node_offsets[k+1]."""

    problem: Problem
    dofmap: DofMap
    offsets: np.ndarray
    node_offsets: np.ndarray
    parts: list
    dofmaps: list


def concat_problems(problems: list) -> Batch:
    """One Problem / DofMap holding every problem's elements, for a single
    batched Generate; the per-element angular frequency (params['omega_e'])
    carries each problem's own frequency."""
    f = problems[0].formulation
    if any(p.formulation != f for p in problems):
        raise ValueError("a batch holds problems of one formulation")
    dms = [dofmap_for(p) for p in problems]
    off = np.zeros(len(problems) + 1, np.int64)
    noff = np.zeros(len(problems) + 1, np.int64)
    for k, (p, dm) in enumerate(zip(problems, dms)):
        off[k + 1] = off[k] + dm.n_dof
        noff[k + 1] = noff[k] + p.mesh.n_nodes
    if off[-1] >= 2 ** 31:
        raise ValueError("batch too large for 32-bit unknown numbers")
    nodes = np.concatenate([p.mesh.nodes for p in problems])
    elems = np.concatenate([p.mesh.elems + noff[k] for k, p in enumerate(problems)])
    edofs = np.concatenate([np.where(dm.elem_dofs >= 0, dm.elem_dofs + off[k], -1)
                            for k, dm in enumerate(dms)]).astype(np.int32)
    esign = np.concatenate([dm.elem_sign for dm in dms])
    region = np.concatenate([p.mesh.region for p in problems])
    mesh = Mesh(nodes, problems[0].mesh.kind, elems.astype(np.int32), region,
                problems[0].mesh.bnd_kind, np.zeros((0, problems[0].mesh.bnd.shape[1]), np.int32),
                np.zeros(0, np.int32))
    params = {}
    if f == "eddy2d":
        params["sigma"] = np.concatenate([p.params["sigma"] for p in problems])
        params["omega_e"] = np.concatenate(
            [np.full(p.mesh.n_elems, p.params["freq"] * 6.2831853071795865)
             for p in problems])
        params["freq"] = float("nan")
    prob = Problem(f"batch_{f}_{len(problems)}", mesh, f,
                   np.concatenate([p.coef for p in problems]),
                   np.concatenate([p.source for p in problems]), params)
    dm = DofMap(int(off[-1]), edofs, esign, dms[0].ncomp, dms[0].nharm)
    return Batch(prob, dm, off.astype(np.int32), noff, problems, dms)


# --------------------------------------------------------------------------
# GetDP input files (used to run the reference on the same problem)
# --------------------------------------------------------------------------

def write_msh22(m: Mesh, path: str) -> None:
    """Gmsh MSH 2.2 ASCII with physical tags; volume elements first."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n")
        f.write(f"{m.n_nodes}\n")
        for k, (x, y, z) in enumerate(m.nodes):
            f.write(f"{k + 1} {x:.17g} {y:.17g} {z:.17g}\n")
        f.write("$EndNodes\n$Elements\n")
        f.write(f"{m.n_elems + len(m.bnd)}\n")
        t = _MSH_TYPE[m.kind]
        eid = 1
        for e, r in zip(m.elems, m.region):
            f.write(f"{eid} {t} 2 {r} {r} " + " ".join(str(v + 1) for v in e) + "\n")
            eid += 1
        tb = _MSH_TYPE[m.bnd_kind]
        for e, r in zip(m.bnd, m.bnd_region):
            f.write(f"{eid} {tb} 2 {r} {r} " + " ".join(str(v + 1) for v in e) + "\n")
            eid += 1
        f.write("$EndElements\n")


_DUMP_OPS = ('Generate[A]; Write[A, File "b.bin"]; Solve[A]; SaveSolution[A];')


def _cvalue(p: Problem, comp: int) -> str:
    """The Value of a fixed-DOF constraint: 0., or the expression of the
    problem's Dirichlet coefficients for that component."""
    g = dirichlet_coefs(p.params.get("dirichlet"))
    return "0." if g is None else constraint_expr(g[comp])


def pro_text(p: Problem) -> str:
    """A GetDP problem file for p, using the canonical Galerkin terms the
    GPU kernels implement.  Per-element coefficients that vary element by
    element are written as one region per element (small meshes only)."""
    f = p.formulation
    if f in ("magnetostatics2d", "eddy2d"):
        eddy = f == "eddy2d"
        groups = ["Air = Region[2]; SrcP = Region[3]; SrcN = Region[4];"]
        if eddy:
            groups.append("Cond = Region[5];")
            groups.append("Dom = Region[{2,3,4,5}];")
        else:
            groups.append("Iron = Region[1];")
            groups.append("Dom = Region[{1,2,3,4}];")
        groups.append("Bnd = Region[10]; Src = Region[{3,4}];")
        fun = [f"mu0 = {MU0:.17g};"]
        if eddy:
            fun.append("nu[] = 1./mu0;")
            fun.append("sigma[Cond] = 5.8e7;")
            fun.append("sigma[Region[{2,3,4}]] = 0.;")
            fun.append(f"Freq = {p.params['freq']:.17g};")
        else:
            fun.append("nu[Iron] = 1./(1000.*mu0);")
            fun.append("nu[Region[{2,3,4}]] = 1./mu0;")
        fun.append("js[SrcP] = Vector[0,0,1.e6]; js[SrcN] = Vector[0,0,-1.e6];")
        eq = ["Integral { [ nu[] * Dof{d a}, {d a} ]; In Dom; Jacobian Vol; Integration I1; }"]
        if eddy:
            eq.append("Integral { DtDof [ sigma[] * Dof{a}, {a} ]; In Cond; Jacobian Vol; Integration I1; }")
        eq.append("Integral { [ -js[], {a} ]; In Src; Jacobian Vol; Integration I1; }")
        system = "{ Name A; NameOfFormulation F; Type Complex; Frequency Freq; }" if eddy \
            else "{ Name A; NameOfFormulation F; }"
        return f"""Group {{
  {' '.join(groups)}
}}
Function {{
  {chr(10).join('  ' + s for s in fun)}
}}
Constraint {{ {{ Name a; Case {{ {{ Region Bnd; Value {_cvalue(p, 0)}; }} }} }} }}
FunctionSpace {{
  {{ Name Hcurl_a; Type Form1P;
    BasisFunction {{ {{ Name se; NameOfCoef ae; Function BF_PerpendicularEdge;
      Support Dom; Entity NodesOf[All]; }} }}
    Constraint {{ {{ NameOfCoef ae; EntityType NodesOf; NameOfConstraint a; }} }} }}
}}
Jacobian {{ {{ Name Vol; Case {{ {{ Region All; Jacobian Vol; }} }} }} }}
Integration {{ {{ Name I1; Case {{ {{ Type Gauss;
  Case {{ {{ GeoElement Triangle; NumberOfPoints 3; }} }} }} }} }} }}
Formulation {{ {{ Name F; Type FemEquation;
  Quantity {{ {{ Name a; Type Local; NameOfSpace Hcurl_a; }} }}
  Equation {{
    {chr(10).join('    ' + s for s in eq)}
  }} }} }}
Resolution {{ {{ Name R; System {{ {system} }}
  Operation {{ {_DUMP_OPS} }} }} }}
"""
    if f == "nonlinear2d":
        ne = p.mesh.n_elems
        lines = []
        for k in range(ne):
            lines.append(f"  nu0[Region[{1000 + k}]] = {p.coef[k]:.17g};")
            lines.append(f"  js[Region[{1000 + k}]] = Vector[0, 0, {p.source[k]:.17g}];")
        b2, ks = p.params["b_sat2"], p.params["k_sat"]
        tol = p.params.get("nl_tol", 1e-8)
        itmax = p.params.get("nl_iter_max", 50)
        res_fmt = 'Format "Residual %03g: abs %14.12e rel %14.12e"'
        return f"""Group {{
  Vol = Region[{{{1000}:{1000 + ne - 1}}}]; Bnd = Region[10];
}}
Function {{
{chr(10).join(lines)}
  nu[] = nu0[] / (1. + {ks:.17g} * Exp[-SquNorm[$1] / {b2:.17g}]);
  dnudb2[] = nu0[] * ({ks:.17g} / {b2:.17g}) * Exp[-SquNorm[$1] / {b2:.17g}] /
             (1. + {ks:.17g} * Exp[-SquNorm[$1] / {b2:.17g}])^2;
  dhdb[] = TensorDiag[1, 1, 1] * nu[$1] + 2. * dnudb2[$1] * SquDyadicProduct[$1];
}}
Constraint {{ {{ Name a; Case {{ {{ Region Bnd; Value {_cvalue(p, 0)}; }} }} }} }}
FunctionSpace {{
  {{ Name Hcurl_a; Type Form1P;
    BasisFunction {{ {{ Name se; NameOfCoef ae; Function BF_PerpendicularEdge;
      Support Vol; Entity NodesOf[All]; }} }}
    Constraint {{ {{ NameOfCoef ae; EntityType NodesOf; NameOfConstraint a; }} }} }}
}}
Jacobian {{ {{ Name Vol; Case {{ {{ Region All; Jacobian Vol; }} }} }} }}
Integration {{ {{ Name I1; Case {{ {{ Type Gauss;
  Case {{ {{ GeoElement Triangle; NumberOfPoints 3; }} }} }} }} }} }}
Formulation {{ {{ Name F; Type FemEquation;
  Quantity {{ {{ Name a; Type Local; NameOfSpace Hcurl_a; }} }}
  Equation {{
    Integral {{ [ nu[{{d a}}] * {{d a}}, {{d a}} ]; In Vol; Jacobian Vol; Integration I1; }}
    Integral {{ [ dhdb[{{d a}}] * Dof{{d a}}, {{d a}} ]; In Vol; Jacobian Vol; Integration I1; }}
    Integral {{ [ -dhdb[{{d a}}] * {{d a}}, {{d a}} ]; In Vol; Jacobian Vol; Integration I1; }}
    Integral {{ [ -js[], {{a}} ]; In Vol; Jacobian Vol; Integration I1; }}
  }} }} }}
Resolution {{ {{ Name R; System {{ {{ Name A; NameOfFormulation F; }} }}
  Operation {{
    InitSolution[A];
    Generate[A]; Write[A, File "b.bin"]; Solve[A];
    Generate[A]; GetResidual[A, $res0];
    Evaluate[ $res = $res0, $iter = 0 ];
    Print[{{$iter, $res, $res / $res0}}, {res_fmt}];
    While[$res > 1e-300 && $res / $res0 > {tol:.17g} && $res / $res0 <= 1 && $iter < {itmax}]{{
      Solve[A]; Generate[A]; GetResidual[A, $res];
      Evaluate[ $iter = $iter + 1 ];
      Print[{{$iter, $res, $res / $res0}}, {res_fmt}];
    }}
    SaveSolution[A];
  }} }} }}
"""
    if f == "elasticity":
        ne = p.mesh.n_elems
        pois = p.params["poisson"]
        rhog = p.params["rho"] * p.params["g"]
        e_lines = "\n".join(f"  E[Region[{1000 + k}]] = {v:.17g};"
                            for k, v in enumerate(p.coef))
        comps = "xyz"
        terms = []
        for i in comps:
            for j in comps:
                terms.append(f"Integral {{ [ -C_{i}{j}[] * Dof{{d u{j}}}, {{d u{i}}} ]; "
                             f"In Vol; Jacobian Vol; Integration I1; }}")
        terms.append("Integral { [ CompZ[f[]], {uz} ]; In Vol; Jacobian Vol; Integration I1; }")
        spaces = []
        for c in comps:
            spaces.append(f"""  {{ Name H_u{c}; Type Form0;
    BasisFunction {{ {{ Name s{c}; NameOfCoef u{c}n; Function BF_Node;
      Support Vol; Entity NodesOf[All]; }} }}
    Constraint {{ {{ NameOfCoef u{c}n; EntityType NodesOf; NameOfConstraint Clamp{c}; }} }} }}""")
        clamps = " ".join(f"{{ Name Clamp{c}; Case {{ {{ Region Fix; Value {_cvalue(p, k)}; }} }} }}"
                          for k, c in enumerate(comps))
        return f"""Group {{
  Vol = Region[{{{1000}:{1000 + ne - 1}}}]; Fix = Region[20];
}}
Function {{
{e_lines}
  nu[] = {pois:.17g};
  a[] = E[]*(1.-nu[])/(1.+nu[])/(1.-2.*nu[]);
  c[] = E[]*nu[]/(1.+nu[])/(1.-2.*nu[]);
  b[] = E[]/2./(1.+nu[]);
  C_xx[] = Tensor[ a[],0  ,0  ,    0  ,b[],0  ,    0  ,0  ,b[] ];
  C_xy[] = Tensor[ 0  ,c[],0  ,    b[],0  ,0  ,    0  ,0  ,0   ];
  C_xz[] = Tensor[ 0  ,0  ,c[],    0  ,0  ,0  ,    b[],0  ,0   ];
  C_yx[] = Tensor[ 0  ,b[],0  ,    c[],0  ,0  ,    0  ,0  ,0   ];
  C_yy[] = Tensor[ b[],0  ,0  ,    0  ,a[],0  ,    0  ,0  ,b[] ];
  C_yz[] = Tensor[ 0  ,0  ,0  ,    0  ,0  ,c[],    0  ,b[],0   ];
  C_zx[] = Tensor[ 0  ,0  ,b[],    0  ,0  ,0  ,    c[],0  ,0   ];
  C_zy[] = Tensor[ 0  ,0  ,0  ,    0  ,0  ,b[],    0  ,c[],0   ];
  C_zz[] = Tensor[ b[],0  ,0  ,    0  ,b[],0  ,    0  ,0  ,a[] ];
  f[] = Vector[0, 0, {-rhog:.17g}];
}}
Constraint {{ {clamps} }}
FunctionSpace {{
{chr(10).join(spaces)}
}}
Jacobian {{ {{ Name Vol; Case {{ {{ Region All; Jacobian Vol; }} }} }} }}
Integration {{ {{ Name I1; Case {{ {{ Type Gauss;
  Case {{ {{ GeoElement Tetrahedron2; NumberOfPoints 4; }} }} }} }} }} }}
Formulation {{ {{ Name F; Type FemEquation;
  Quantity {{ {{ Name ux; Type Local; NameOfSpace H_ux; }}
             {{ Name uy; Type Local; NameOfSpace H_uy; }}
             {{ Name uz; Type Local; NameOfSpace H_uz; }} }}
  Equation {{
{chr(10).join('    ' + t for t in terms)}
  }} }} }}
Resolution {{ {{ Name R; System {{ {{ Name A; NameOfFormulation F; }} }}
  Operation {{ {_DUMP_OPS} }} }} }}
"""
    if f == "curlcurl":
        rg = p.params["reg"]
        ne = p.mesh.n_elems
        lines = []
        for k in range(ne):
            lines.append(f"  nu[Region[{1000 + k}]] = {p.coef[k]:.17g};")
            jx, jy, jz = p.source[k]
            lines.append(f"  js[Region[{1000 + k}]] = Vector[{jx:.17g}, {jy:.17g}, {jz:.17g}];")
        return f"""Group {{
  Dom = Region[{{{1000}:{1000 + ne - 1}}}]; Bnd = Region[30];
}}
Function {{
{chr(10).join(lines)}
}}
Constraint {{ {{ Name a; Case {{ {{ Region Bnd; Value 0.; }} }} }} }}
FunctionSpace {{
  {{ Name Hcurl_a; Type Form1;
    BasisFunction {{ {{ Name se; NameOfCoef ae; Function BF_Edge;
      Support Dom; Entity EdgesOf[All]; }} }}
    Constraint {{ {{ NameOfCoef ae; EntityType EdgesOf; NameOfConstraint a; }} }} }}
}}
Jacobian {{ {{ Name Vol; Case {{ {{ Region All; Jacobian Vol; }} }} }} }}
Integration {{ {{ Name I1; Case {{ {{ Type Gauss;
  Case {{ {{ GeoElement Tetrahedron; NumberOfPoints 4; }} }} }} }} }} }}
Formulation {{ {{ Name F; Type FemEquation;
  Quantity {{ {{ Name a; Type Local; NameOfSpace Hcurl_a; }} }}
  Equation {{
    Integral {{ [ nu[] * Dof{{d a}}, {{d a}} ]; In Dom; Jacobian Vol; Integration I1; }}
    Integral {{ [ {rg:.17g} * nu[] * Dof{{a}}, {{a}} ]; In Dom; Jacobian Vol; Integration I1; }}
    Integral {{ [ -js[], {{a}} ]; In Dom; Jacobian Vol; Integration I1; }}
  }} }} }}
Resolution {{ {{ Name R; System {{ {{ Name A; NameOfFormulation F; }} }}
  Operation {{ {_DUMP_OPS} }} }} }}
"""
    raise ValueError(f)


def post_text(p: Problem, points) -> str:
    """PostProcessing / PostOperation blocks for pro_text(p): the field and
    its curl printed on every element (Format Table, file post_elem.txt) and
    the field at each of `points` (file post_pts.txt)."""
    f = p.formulation
    if f not in ("magnetostatics2d", "eddy2d", "curlcurl"):
        raise ValueError(f)
    dom = "Dom"
    quants = (f"{{ Name av; Value {{ Local {{ [ {{a}} ]; In {dom}; Jacobian Vol; }} }} }}\n"
              f"    {{ Name b; Value {{ Local {{ [ {{d a}} ]; In {dom}; Jacobian Vol; }} }} }}")
    ops = [f'Print[ b, OnElementsOf {dom}, Format Table, File "post_elem.txt" ];']
    for (x, y, z) in points:
        ops.append(f'Print[ av, OnPoint {{{x:.17g}, {y:.17g}, {z:.17g}}}, Format Table, '
                   f'File > "post_pts.txt" ];')
        ops.append(f'Print[ b, OnPoint {{{x:.17g}, {y:.17g}, {z:.17g}}}, Format Table, '
                   f'File > "post_pts_b.txt" ];')
    return f"""PostProcessing {{ {{ Name P; NameOfFormulation F;
  Quantity {{
    {quants}
  }} }} }}
PostOperation {{ {{ Name Map; NameOfPostProcessing P;
  Operation {{
    {chr(10).join('    ' + o for o in ops)}
  }} }} }}
"""


def prepare_regions(p: Problem) -> None:
    """Formulations with per-element coefficients give every element its own
    physical region (1000 + element index), as pro_text expects."""
    if p.formulation in ("elasticity", "nonlinear2d", "curlcurl"):
        p.mesh.region = (1000 + np.arange(p.mesh.n_elems)).astype(np.int32)


def write_pro(p: Problem, path: str) -> None:
    """Write the problem file (after prepare_regions: write the mesh after
    this call)."""
    prepare_regions(p)
    with open(path, "w") as f:
        f.write(pro_text(p))
