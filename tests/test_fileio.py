"""MSH 2.2 reading and .res writing (the formats on either side of the
path): round trips, the reference's own example mesh, and the reference's
post-processing reading a .res file written here."""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from getdp_gb300 import fileio as FIO
from getdp_gb300 import workloads as W
from oracle import refsrc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref", "getdp_ilu64")
GETDP_SRC = refsrc.source_dir() or ""


@pytest.mark.parametrize("p", [W.magnetostatics_2d(n=9, seed=2), W.curlcurl_edge(n=3, seed=1),
                               W.elasticity_p2(n=2, seed=1)],
                         ids=["tri3", "tet4", "tet10"])
@pytest.mark.parametrize("reader", ["native", "numpy"])
def test_msh_round_trip(p, reader, tmp_path):
    path = str(tmp_path / "m.msh")
    W.write_msh22(p.mesh, path)
    d = FIO.read_msh22(path) if reader == "native" else FIO.read_msh22_numpy(path)
    assert np.array_equal(d.nodes, p.mesh.nodes)
    assert np.array_equal(d.node_numbers, np.arange(1, p.mesh.n_nodes + 1))
    tv = W._MSH_TYPE[p.mesh.kind]
    num, phys, _, conn = d.elements[tv]
    assert np.array_equal(conn, p.mesh.elems)
    assert np.array_equal(phys, p.mesh.region)
    tb = W._MSH_TYPE[p.mesh.bnd_kind]
    assert np.array_equal(d.elements[tb][3], p.mesh.bnd)


def test_msh_binary(tmp_path):
    # a binary file written here in the MSH 2.2 binary layout
    p = W.magnetostatics_2d(n=5, seed=3)
    m = p.mesh
    path = str(tmp_path / "b.msh")
    with open(path, "wb") as f:
        f.write(b"$MeshFormat\n2.2 1 8\n")
        f.write(np.array([1], "<i4").tobytes() + b"\n$EndMeshFormat\n$Nodes\n")
        f.write(f"{m.n_nodes}\n".encode())
        rec = np.zeros(m.n_nodes, np.dtype([("num", "<i4"), ("xyz", "<f8", 3)]))
        rec["num"] = np.arange(1, m.n_nodes + 1)
        rec["xyz"] = m.nodes
        f.write(rec.tobytes() + b"\n$EndNodes\n$Elements\n")
        f.write(f"{m.n_elems}\n".encode())
        f.write(np.array([2, m.n_elems, 2], "<i4").tobytes())
        body = np.concatenate([np.arange(1, m.n_elems + 1)[:, None], m.region[:, None],
                               m.region[:, None], m.elems + 1], 1).astype("<i4")
        f.write(body.tobytes() + b"\n$EndElements\n")
    for rd in (FIO.read_msh22, FIO.read_msh22_numpy):
        d = rd(path)
        assert np.array_equal(d.nodes, m.nodes)
        assert np.array_equal(d.elements[2][3], m.elems)
        assert np.array_equal(d.elements[2][1], m.region)


@pytest.mark.skipif(not os.path.exists(os.path.join(GETDP_SRC, "examples", "magnet.msh")),
                    reason="reference example not present")
def test_reads_reference_example_mesh():
    d = FIO.read_msh22(os.path.join(GETDP_SRC, "examples", "magnet.msh"))
    assert d.nodes.shape[1] == 3 and len(d.nodes) > 0
    total = sum(len(v[0]) for v in d.elements.values())
    with open(os.path.join(GETDP_SRC, "examples", "magnet.msh"), "rb") as f:
        data = f.read()
    a = data.index(b"$Elements")
    assert total == int(data[a:].split(b"\n")[1])


@pytest.mark.parametrize("binary", [True, False])
def test_res_round_trip(binary, tmp_path):
    x = np.random.default_rng(1).standard_normal(37)
    path = str(tmp_path / "s.res")
    FIO.write_res(path, x, binary=binary)
    FIO.write_res(path, 2 * x, binary=binary, step=1, time=0.5, append=True)
    sols = FIO.read_res(path, len(x))
    assert len(sols) == 2
    if binary:
        assert np.array_equal(sols[0][4], x) and np.array_equal(sols[1][4], 2 * x)
    else:  # GetDP prints %.16g: one unit in the 17th digit may differ
        assert np.allclose(sols[0][4], x, rtol=1e-15, atol=0)
        assert np.allclose(sols[1][4], 2 * x, rtol=1e-15, atol=0)
    assert sols[1][1] == 0.5 and sols[1][3] == 1


@pytest.mark.skipif(not os.path.exists(REF), reason="reference binary not built")
@pytest.mark.parametrize("binary", [True, False])
def test_reference_post_processing_reads_our_res(binary):
    # the reference prints the same curl values from our .res as from its own
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_post_golden import parse_table
    d = dict(np.load(os.path.join(ROOT, "tests", "golden", "post_ms2d_n8.npz")))
    p = W.magnetostatics_2d(n=8, seed=11)
    with tempfile.TemporaryDirectory() as tmp:
        W.write_pro(p, os.path.join(tmp, "p.pro"))
        with open(os.path.join(tmp, "p.pro"), "a") as f:
            f.write(W.post_text(p, []))
        W.write_msh22(p.mesh, os.path.join(tmp, "p.msh"))
        FIO.write_res(os.path.join(tmp, "ours.res"), d["x"], binary=binary)
        r = subprocess.run([REF, "p.pro", "-pre", "R", "-msh", "p.msh", "-pos", "Map",
                            "-res", "ours.res", "-v", "2"], cwd=tmp,
                           stdin=subprocess.DEVNULL, capture_output=True, text=True,
                           timeout=300)
        out = os.path.join(tmp, "post_elem.txt")
        assert os.path.exists(out), r.stdout[-2000:] + r.stderr[-2000:]
        _, _, vals = parse_table(out, 3, 9)
    got = vals.reshape(-1, 1, 3, 3)
    if binary:
        assert np.array_equal(got, d["elem_vals"])
    else:  # the solution went through %.16g
        assert np.abs(got - d["elem_vals"]).max() <= 1e-14 * np.abs(d["elem_vals"]).max()


@pytest.mark.skipif(not os.path.exists(REF), reason="reference binary not built")
@pytest.mark.parametrize("gen,kw", [
    (W.magnetostatics_2d, dict(n=6, seed=3)),
    (W.magnetostatics_2d, dict(n=5, seed=1, dirichlet=1)),
    (W.eddy_2d, dict(n=4, seed=4, freq=500.0, dirichlet=1)),
    (W.elasticity_p2, dict(n=2, seed=21)),
    (W.elasticity_p2, dict(n=2, seed=23, dirichlet=2)),
    (W.curlcurl_edge, dict(n=3, seed=31)),
], ids=["ms2d", "ms2d_dir", "eddy_dir", "el_p2", "el_p2_dir", "cc_edge"])
def test_pre_writer_matches_reference_bytes(gen, kw, tmp_path):
    # the reference writes its .pre at pre-processing; ours from the DofMap
    p = gen(**kw)
    dm = W.dofmap_for(p)
    W.write_pro(p, str(tmp_path / "p.pro"))
    W.write_msh22(p.mesh, str(tmp_path / "p.msh"))
    r = subprocess.run([REF, "p.pro", "-pre", "R", "-msh", "p.msh", "-v", "1"], cwd=tmp_path,
                       stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=300)
    assert (tmp_path / "p.pre").exists(), r.stdout[-2000:] + r.stderr[-2000:]
    FIO.write_pre(str(tmp_path / "ours.pre"), p.mesh, dm)
    assert (tmp_path / "ours.pre").read_bytes() == (tmp_path / "p.pre").read_bytes()


def test_pre_writer_round_trips_the_numbering(tmp_path):
    # parsed back, the records give every element's unknown numbers
    p = W.elasticity_p2(n=3, seed=2)
    dm = W.dofmap_for(p)
    FIO.write_pre(str(tmp_path / "p.pre"), p.mesh, dm)
    lines = (tmp_path / "p.pre").read_text().splitlines()
    nrec, nunk = map(int, lines[8].split())
    assert nunk == dm.n_dof
    num = {}
    for l in lines[9:9 + nrec]:
        t = l.split()
        if t[3] == "1":
            num[(int(t[0]), int(t[1]))] = int(t[4]) - 1
    nv = p.mesh.elems.shape[1]
    for k in range(30):
        key = [(k // nv + 1, int(v) + 1) for v in p.mesh.elems[:, k % nv]]
        got = np.array([num.get(kk, -1) for kk in key])
        assert np.array_equal(got, np.where(dm.elem_dofs[:, k] >= 0, dm.elem_dofs[:, k], -1))


def test_native_pre_formatting_equals_python():
    """The library's formatters of the .pre blocks give the bytes of the
    Python formatting (records of both types, "%.16g" of awkward values,
    signed edge rows), and refuse a buffer that is too small."""
    import ctypes
    from getdp_gb300 import _lib
    L = _lib.load(build_if_missing=True)
    rng = np.random.default_rng(3)
    vals = np.concatenate([[0.0, -0.0, 1.0, -1.5, 1e-300, -2.5e-308, 1e300, np.pi,
                            1 / 3, 123456789.0123456789, 5e-5, 1e16, 1e15 + 0.5],
                           rng.standard_normal(200) * 10.0 ** rng.integers(-20, 20, 200)])
    n = len(vals)
    rec5 = np.column_stack([rng.integers(1, 4, n), rng.integers(1, 10 ** 9, n),
                            rng.integers(0, 2, n), rng.integers(1, 3, n),
                            rng.integers(1, 10 ** 7, n)]).astype(np.int64)
    got = FIO._native_text(L.gb300_format_dof_records, n, 160, rec5, vals)
    want = "".join(f"{nt} {ent} {h} 1 {num} 1\n" if typ == 1 else
                   f"{nt} {ent} {h} 2 {'%.16g' % v} 0\n"
                   for (nt, ent, h, typ, num), v in zip(rec5.tolist(), vals.tolist()))
    assert got == want.encode()
    rows = rng.integers(-10 ** 6, 10 ** 6, (50, 6)).astype(np.int64)
    got = FIO._native_text(L.gb300_format_int_rows, len(rows), 40 + 21 * 6,
                           ctypes.c_int(6), rows, ctypes.c_longlong(7))
    want = "".join(f"{7 + i} 6 " + " ".join(map(str, r)) + "\n"
                   for i, r in enumerate(rows.tolist()))
    assert got == want.encode()
    buf = np.empty(8, np.uint8)
    m = ctypes.c_longlong(0)
    rc = L.gb300_format_dof_records(n, rec5.ctypes.data_as(ctypes.c_void_p),
                                    vals.ctypes.data_as(ctypes.c_void_p),
                                    buf.ctypes.data_as(ctypes.c_void_p), 8, ctypes.byref(m))
    assert rc == 6  # GB300_ERR_CAPACITY
