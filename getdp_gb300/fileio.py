"""The on-disk formats either side of the path: Gmsh MSH 2.2 meshes in
(GetDP's reader: GeoData.cpp, Geo_ReadFileWithGmsh) and GetDP .res solution
files out (DofData.cpp:631-767, Dof_WriteFileRES0 / Dof_WriteFileRES, read
back by Dof_ReadFileRES).

Parsing is vectorised (numpy) so that a million-element mesh loads in well
under a second; the .res writer produces what GetDP's own reader accepts
(the reference's post-processing runs on it, tests/test_fileio.py).
"""
from __future__ import annotations

import dataclasses

import numpy as np

# Gmsh element type -> nodes per element (the types GetDP's examples use)
MSH_NODES = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 6: 6, 7: 5, 8: 3, 9: 6, 11: 10, 15: 1}


@dataclasses.dataclass
class MshData:
    """Nodes (with their Gmsh numbers) and elements grouped by type:
    elements[type] = (numbers, physical tags, elementary tags, 0-based node
    indices)."""

    node_numbers: np.ndarray
    nodes: np.ndarray
    elements: dict


def _section(data: bytes, name: bytes):
    a = data.index(b"$" + name)
    a = data.index(b"\n", a) + 1
    b = data.index(b"$End" + name, a)
    return a, b


def read_msh22(path: str) -> MshData:
    """Gmsh MSH 2.2, ASCII or binary (little-endian), with the library's
    native parser (gb300_msh_read); read_msh22_numpy is the same in numpy."""
    import ctypes
    from . import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(L.gb300_msh_read(path.encode(), ctypes.byref(h)))
    try:
        n = ctypes.c_longlong()
        pn, px = ctypes.c_void_p(), ctypes.c_void_p()
        _lib.check(L.gb300_msh_nodes(h, ctypes.byref(n), ctypes.byref(pn), ctypes.byref(px)))
        nn = n.value

        def arr(ptr, dtype, count):
            if count == 0:
                return np.zeros(0, dtype)
            return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(
                np.ctypeslib.as_ctypes_type(dtype))), shape=(count,)).copy()

        numbers = arr(pn.value, np.int64, nn)
        xyz = arr(px.value, np.float64, 3 * nn).reshape(nn, 3)
        cnt = ctypes.c_int()
        _lib.check(L.gb300_msh_group_count(h, ctypes.byref(cnt)))
        groups = {}
        for g in range(cnt.value):
            t, ne, nt, npe = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int()
            p1, p2, p3 = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
            _lib.check(L.gb300_msh_group(h, g, ctypes.byref(t), ctypes.byref(ne),
                                         ctypes.byref(nt), ctypes.byref(npe),
                                         ctypes.byref(p1), ctypes.byref(p2),
                                         ctypes.byref(p3)))
            k = ne.value
            groups.setdefault(t.value, []).append(
                (arr(p1.value, np.int64, k),
                 arr(p2.value, np.int32, k * nt.value).reshape(k, nt.value),
                 arr(p3.value, np.int64, k * npe.value).reshape(k, npe.value)))
    finally:
        L.gb300_msh_free(h)
    return _assemble(path, numbers, xyz, groups)


def read_msh22_numpy(path: str) -> MshData:
    """Gmsh MSH 2.2, ASCII or binary (little-endian), parsed with numpy."""
    with open(path, "rb") as f:
        data = f.read()
    a, b = _section(data, b"MeshFormat")
    head = data[a:b].split(b"\n")[0].split()
    if not head[0].startswith(b"2"):
        raise ValueError(f"{path}: MSH format {head[0].decode()} (2.x expected)")
    binary = int(head[1]) == 1
    a, b = _section(data, b"Nodes")
    nl = data.index(b"\n", a)
    nn = int(data[a:nl])
    if binary:
        rec = np.dtype([("num", "<i4"), ("xyz", "<f8", 3)])
        arr = np.frombuffer(data, rec, count=nn, offset=nl + 1)
        numbers, xyz = arr["num"].astype(np.int64), arr["xyz"].astype(np.float64)
    else:
        vals = np.array(data[nl + 1:b].split(), dtype=np.float64).reshape(nn, 4)
        numbers, xyz = vals[:, 0].astype(np.int64), vals[:, 1:].copy()
    a, b = _section(data, b"Elements")
    nl = data.index(b"\n", a)
    ne = int(data[a:nl])
    groups = {}
    if binary:
        off = nl + 1
        done = 0
        while done < ne:
            t, count, ntags = np.frombuffer(data, "<i4", 3, off)
            off += 12
            npe = MSH_NODES[int(t)]
            rec = np.frombuffer(data, "<i4", count * (1 + ntags + npe), off)
            off += 4 * rec.size
            rec = rec.reshape(count, 1 + ntags + npe)
            groups.setdefault(int(t), []).append((rec[:, 0], rec[:, 1:1 + ntags],
                                                  rec[:, 1 + ntags:]))
            done += count
    else:
        # all numbers of the section, then runs of records of one (type,
        # tag count) taken a whole block at a time
        tok = np.array(data[nl + 1:b].split(), dtype=np.int64)
        p, done = 0, 0
        while done < ne:
            t, ntags = int(tok[p + 1]), int(tok[p + 2])
            rl = 3 + ntags + MSH_NODES[t]
            left = (len(tok) - p) // rl
            block = tok[p:p + left * rl].reshape(left, rl)
            same = (block[:, 1] == t) & (block[:, 2] == ntags)
            cnt = int(np.argmin(same)) if not same.all() else left
            cnt = min(cnt, ne - done)
            m = block[:cnt]
            groups.setdefault(t, []).append((m[:, 0], m[:, 3:3 + ntags], m[:, 3 + ntags:]))
            p += cnt * rl
            done += cnt
    return _assemble(path, numbers, xyz, groups)


def _assemble(path, numbers, xyz, groups) -> MshData:
    nn = len(numbers)
    lookup = np.full(int(numbers.max()) + 1 if nn else 1, -1, np.int64)
    lookup[numbers] = np.arange(nn)
    elements = {}
    for t, parts in groups.items():
        num = np.concatenate([p[0] for p in parts]).astype(np.int64)
        tags = [p[1] for p in parts]
        width = max(x.shape[1] for x in tags)
        tags = np.concatenate([np.pad(x, ((0, 0), (0, width - x.shape[1]))) for x in tags])
        conn = lookup[np.concatenate([p[2] for p in parts]).astype(np.int64)]
        if (conn < 0).any():
            raise ValueError(f"{path}: an element refers to an unknown node")
        phys = tags[:, 0] if width > 0 else np.zeros(len(num), np.int64)
        elem = tags[:, 1] if width > 1 else np.zeros(len(num), np.int64)
        order = np.argsort(num, kind="stable")  # GetDP sorts elements by number
        elements[t] = (num[order], phys[order], elem[order], conn[order].astype(np.int32))
    return MshData(numbers, xyz, elements)


def write_res(path: str, x: np.ndarray, binary: bool = True, dofdata: int = 0,
              time: float = 0.0, time_imag: float = 0.0, step: int = 0,
              append: bool = False) -> None:
    """A GetDP .res file holding solution vector x of DofData `dofdata`
    (Dof_WriteFileRES0 header, then one $Solution block as
    Dof_WriteFileRES writes it)."""
    x = np.ascontiguousarray(x, np.float64)
    mode = "ab" if append else "wb"
    with open(path, mode) as f:
        if not append:
            f.write(("$ResFormat /* getdp-gb300, %s */\n1.1 %d\n$EndResFormat\n"
                     % ("binary" if binary else "ascii", 1 if binary else 0)).encode())
        f.write(("$Solution  /* DofData #%d */\n%d %.16g %.16g %d\n"
                 % (dofdata, dofdata, time, time_imag, step)).encode())
        if binary:
            f.write(x.tobytes())
            f.write(b"\n")
        else:
            f.write("".join("%.16g\n" % v for v in x).encode())
        f.write(b"$EndSolution\n")


def read_res(path: str, n: int) -> list:
    """Every $Solution block of a .res file: (dofdata, time, time_imag, step,
    values[n])."""
    with open(path, "rb") as f:
        data = f.read()
    a, b = _section(data, b"ResFormat")
    version, fmt = data[a:b].split()[:2]
    binary = int(fmt) == 1
    out = []
    pos = 0
    while True:
        k = data.find(b"$Solution", pos)
        if k < 0:
            break
        k = data.index(b"\n", k) + 1
        e = data.index(b"\n", k)
        h = data[k:e].split()
        k = e + 1
        if binary:
            vals = np.frombuffer(data, np.float64, n, k).copy()
            k += 8 * n
        else:
            end = data.index(b"$EndSolution", k)
            vals = np.array(data[k:end].split(), dtype=np.float64)[:n]
            k = end
        out.append((int(h[0]), float(h[1]), float(h[2]), int(h[3]), vals))
        pos = data.index(b"$EndSolution", k) + 12
    return out


# --------------------------------------------------------------------------
# .pre (DOF numbering) writer
# --------------------------------------------------------------------------
def dof_records(mesh, dm):
    """Every DOF the element tables touch, as (NumType, Entity, Harmonic,
    Type, NumDof, value) sorted by (NumType, Entity, Harmonic): GetDP's DOF
    tree order (DofData.cpp:36-45).  Nodal spaces: NumType = component + 1,
    Entity = node number; edge spaces: Entity = edge number (first-touch
    order, dm.edges).  Type 1 unknown (NumDof 1-based), 2 fixed (with its
    value: dm.fixed_values, or 0)."""
    ed = np.asarray(dm.elem_dofs, np.int64)
    ne, nloc = ed.shape
    fv = None if dm.fixed_values is None else np.asarray(dm.fixed_values, np.float64)
    if dm.edges is not None:  # Whitney edges: local edge k of the element
        from .workloads import TET4_EDGES
        nn = mesh.n_nodes
        ve = mesh.elems[:, TET4_EDGES].reshape(-1, 2).astype(np.int64)
        key = np.minimum(ve[:, 0], ve[:, 1]) * nn + np.maximum(ve[:, 0], ve[:, 1])
        ekey = dm.edges[:, 0].astype(np.int64) * nn + dm.edges[:, 1]
        order = np.argsort(ekey)
        ent = order[np.searchsorted(ekey[order], key)] + 1
        numtype = np.ones_like(ent)
        flat = ed.ravel()
        harm = [(0, flat)]
    else:
        nv = mesh.elems.shape[1]
        comp = np.arange(nloc) // nv
        ent = (mesh.elems[:, np.arange(nloc) % nv].astype(np.int64) + 1).ravel()
        numtype = np.broadcast_to(comp + 1, (ne, nloc)).ravel()
        flat = ed.ravel()
        harm = [(h, flat) for h in range(dm.nharm)]
    # one occurrence of each (NumType, Entity) the tables touch, in key order:
    # the keys are dense, so an index over their range replaces a sort (any
    # occurrence will do: every occurrence of a DOF carries the same number)
    numtype = np.ascontiguousarray(numtype, np.int64)
    if len(ent) == 0:
        return np.zeros((0, 6))
    span_e = int(ent.max()) + 1
    key = numtype * span_e + ent
    idx = np.full(int(key.max()) + 1, -1, np.int64)
    idx[key] = np.arange(len(key))
    sel = idx[idx >= 0]
    nh = len(harm)
    sel = np.repeat(sel, nh)  # harmonics of one DOF next to each other
    h = np.tile(np.arange(nh), len(sel) // nh)
    d = flat[sel]
    unk = d >= 0
    num = np.where(unk, d + h + 1, 0)  # 1-based; harmonic 1 is the next number
    if fv is None:
        val = np.zeros(len(d))
    else:
        k = np.maximum(-d - 1, 0)
        if fv.ndim == 2:
            val = fv[k, h]
        else:
            val = np.where(h == 0, fv[k], 0.0)
        val = np.where(unk, 0.0, val)
    return np.stack([numtype[sel], ent[sel], h, np.where(unk, 1, 2), num, val], 1)


def write_pre(path: str, mesh, dm, resolution: str = "R", n_spaces: int = None) -> None:
    """The .pre file GetDP writes for a one-system resolution
    (Dof_WriteFilePRE, DofData.cpp:363-462): the $Resolution header, one
    $DofData block (resolution and system index 0, the function spaces
    0..n-1, time function 0), every DOF of the tree with its number (unknown)
    or value (fixed, "%.16g" as LinAlg_PrintScalar prints it)."""
    r = dof_records(mesh, dm)
    if n_spaces is None:
        n_spaces = int(r[:, 0].max()) if len(r) else 1
    n_unknown = int(np.sum(r[:, 3] == 1))
    head = [f"$Resolution /* '{resolution}' */", "0 1", "$EndResolution",
            "$DofData /* #0 */", "0 0",
            " ".join([str(n_spaces)] + [str(i) for i in range(n_spaces)]),
            "1 0", "1 0", f"{len(r)} {n_unknown}"]
    L = _native()
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if L is not None:
            rec5 = np.ascontiguousarray(r[:, :5], np.int64)
            vals = np.ascontiguousarray(r[:, 5], np.float64)
            f.write(_native_text(L.gb300_format_dof_records, len(r), 160,
                                 rec5, vals))
        else:
            ints = r[:, :5].astype(np.int64).tolist()
            f.write("".join(f"{nt} {ent} {h} 1 {num} 1\n" if typ == 1 else
                            f"{nt} {ent} {h} 2 {'%.16g' % v} 0\n"
                            for (nt, ent, h, typ, num), v in
                            zip(ints, r[:, 5].tolist())).encode())
        f.write(b"$EndDofData\n")
        if dm.edges is not None:
            _write_elements_x_edges(f, mesh, dm, L)


def _native():
    """The library's text formatters, where the library is built (the
    formatting in Python below gives the same bytes)."""
    try:
        from . import _lib
        return _lib.load()
    except (ImportError, OSError):
        return None


def _native_text(fn, nrows: int, per_row: int, *args) -> bytes:
    import ctypes
    from . import _lib
    cap = nrows * per_row + 64
    buf = np.empty(cap, np.uint8)
    n = ctypes.c_longlong(0)
    ptrs = [a.ctypes.data_as(ctypes.c_void_p) if isinstance(a, np.ndarray) else a for a in args]
    _lib.check(fn(nrows, *ptrs, buf.ctypes.data_as(ctypes.c_void_p), cap, ctypes.byref(n)))
    return buf[:n.value].tobytes()


def _write_elements_x_edges(f, mesh, dm, L):
    """$ElementsXEdges (Geo_WriteFilePRE, GeoEntity.cpp:526-552): every
    element with edges, in mesh order (volume elements, then the boundary
    elements whose edges the constraint created), with its edges' numbers,
    negative where the element runs the edge from the higher to the lower
    node number (GeoEntity.h:214-215 local edges)."""
    blocks = _edge_blocks(mesh, dm)
    if L is None:
        f.write(("\n".join(_elements_x_edges(blocks)) + "\n").encode())
        return
    import ctypes
    f.write(f"$ElementsXEdges\n0 {sum(len(b) for b in blocks)}\n".encode())
    i = 0
    for blk in blocks:
        v = np.ascontiguousarray(blk, np.int64)
        f.write(_native_text(L.gb300_format_int_rows, len(v), 40 + 21 * v.shape[1],
                             ctypes.c_int(v.shape[1]), v, ctypes.c_longlong(i)))
        i += len(v)
    f.write(b"$EndElementsXEdges\n")


def _edge_blocks(mesh, dm):
    """The signed edge numbers of every element with edges (volume
    elements, then boundary elements), one array per element kind."""
    from .workloads import TET4_EDGES, TRI3_EDGES_GETDP
    nn = mesh.n_nodes
    ekey = dm.edges[:, 0].astype(np.int64) * nn + dm.edges[:, 1]
    order = np.argsort(ekey)

    def signed(conn, loc):
        ve = conn[:, loc].reshape(-1, 2).astype(np.int64)
        key = np.minimum(ve[:, 0], ve[:, 1]) * nn + np.maximum(ve[:, 0], ve[:, 1])
        num = order[np.searchsorted(ekey[order], key)] + 1
        return np.where(ve[:, 0] < ve[:, 1], num, -num).reshape(len(conn), -1)

    blocks = [signed(mesh.elems, TET4_EDGES)]
    if len(mesh.bnd):
        blocks.append(signed(mesh.bnd, TRI3_EDGES_GETDP))
    return blocks


def _elements_x_edges(blocks):
    """The $ElementsXEdges block as text lines (the Python formatting)."""
    lines = ["$ElementsXEdges", f"0 {sum(len(b) for b in blocks)}"]
    i = 0
    for blk in blocks:
        w = blk.shape[1]
        for row in blk.tolist():
            lines.append(f"{i} {w} " + " ".join(map(str, row)))
            i += 1
    lines.append("$EndElementsXEdges")
    return lines
