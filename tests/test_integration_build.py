"""The drop-in integration, checked where the GetDP sources are present
(the development host; skipped elsewhere).

* build_getdp.sh compiles the unchanged GetDP sources with LinAlg_GB300.cpp in
  place of the Sparskit backend and the batched Generate hook
  (Generate_GB300.cpp, hooked into a patched copy of Treatment_Formulation.cpp)
  and links the program against libgetdp_gb300.so; the program runs the
  reference's own example (a copy of examples/magnet.*) through its parser and
  pre-processing into the backend (on a host without a GPU it stops there,
  with the backend's message).
* The same objects linked against a test double of the C ABI
  (tests/fake_gb300, host memory) run an unchanged 2D magnetostatics .pro
  through Generate: the element batch the hook gathers from GetDP's own data
  structures (node coordinates, unknown numbers, fixed DOFs and their values,
  the reluctivity of every element) is the one the workload's tables give.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import refsrc

GETDP_SRC = refsrc.source_dir() or ""
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

pytestmark = pytest.mark.skipif(
    not os.path.exists(os.path.join(GETDP_SRC, "src", "kernel", "LinAlg.h")),
    reason="GetDP sources not present")


@pytest.fixture(scope="module")
def getdp_build():
    """GetDP with the GB300 backend (objects kept between runs)."""
    from getdp_gb300 import build
    build.build()
    out = os.path.join(ROOT, "getdp_gb300", "_build", "getdp_backend")
    r = subprocess.run(["bash", os.path.join(ROOT, "getdp_gb300", "getdp_backend",
                                             "build_getdp.sh"), GETDP_SRC, out],
                       capture_output=True, text=True, timeout=2400)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return out


def test_getdp_builds_and_links_with_the_gb300_backend(getdp_build, tmp_path):
    exe = os.path.join(getdp_build, "getdp")
    assert os.path.exists(exe)
    # the reference's own example (it includes ../templates), run in a
    # scratch copy
    shutil.copytree(os.path.join(GETDP_SRC, "examples"), tmp_path / "examples")
    shutil.copytree(os.path.join(GETDP_SRC, "templates"), tmp_path / "templates")
    work = tmp_path / "examples"
    r = subprocess.run([exe, "magnet.pro", "-solve", "#1", "-v", "3"], cwd=work,
                       stdin=subprocess.DEVNULL, capture_output=True, text=True, timeout=300)
    log = r.stdout + r.stderr
    assert "Pre-processing" in log or "P r e" in log or "Pre" in log, log[-2000:]
    try:
        import torch  # noqa: F401  (only to tell whether a GPU is visible)
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert "GB300 backend: no CUDA device available" in log, log[-2000:]


def _read_dump(path):
    with open(path, "rb") as f:
        ne, nf = np.frombuffer(f.read(8), np.int32)
        nodes = np.frombuffer(f.read(8 * 9 * ne), np.float64).reshape(ne, 3, 3)
        edofs = np.frombuffer(f.read(4 * 3 * ne), np.int32).reshape(ne, 3)
        coef = np.frombuffer(f.read(8 * ne), np.float64)
        fixed = np.frombuffer(f.read(8 * nf), np.float64)
    return nodes, edofs, coef, fixed


@pytest.mark.parametrize("dirichlet", [None, 1])
def test_generate_hook_gathers_the_element_batch(getdp_build, tmp_path, dirichlet):
    from getdp_gb300 import workloads as W
    # the test double of the C ABI, and GetDP's objects linked against it
    fake = tmp_path / "fake"
    fake.mkdir()
    subprocess.run(["g++", "-O1", "-std=c++11", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "include"),
                    os.path.join(HERE, "fake_gb300", "fake_gb300.cpp"),
                    "-o", str(fake / "libgetdp_gb300.so")], check=True)
    objs = [os.path.join(getdp_build, "obj", f)
            for f in sorted(os.listdir(os.path.join(getdp_build, "obj")))]
    exe = str(tmp_path / "getdp_fake")
    subprocess.run(["g++", "-o", exe, *objs, "-L", str(fake), "-lgetdp_gb300",
                    f"-Wl,-rpath,{fake}", "-lm"], check=True)
    # an unchanged 2D a_z problem, Generate only
    p = W.magnetostatics_2d(12, seed=3, dirichlet=dirichlet)
    dm = W.dofmap_for(p)
    text = W.pro_text(p).replace(W._DUMP_OPS, "Generate[A];")
    (tmp_path / "p.pro").write_text(text)
    W.write_msh22(p.mesh, str(tmp_path / "p.msh"))
    env = dict(os.environ, GB300_GENERATE_DUMP=str(tmp_path / "batch.bin"))
    r = subprocess.run([exe, "p.pro", "-solve", "R", "-msh", "p.msh", "-v", "4"],
                       cwd=tmp_path, env=env, stdin=subprocess.DEVNULL,
                       capture_output=True, text=True, timeout=300)
    log = r.stdout + r.stderr
    assert "element matrices assembled on the GPU" in log, log[-3000:]
    nodes, edofs, coef, fixed = _read_dump(tmp_path / "batch.bin")
    # GetDP visits the elements in number order: the volume elements first
    ne = p.mesh.n_elems
    assert len(coef) == ne
    assert np.array_equal(nodes, p.mesh.nodes[p.mesh.elems])
    assert np.array_equal(coef, p.coef)  # nu per region, evaluated by GetDP
    unk = dm.elem_dofs >= 0
    assert np.array_equal(edofs >= 0, unk)
    assert np.array_equal(edofs[unk], dm.elem_dofs[unk])
    # fixed DOFs: GetDP's values (0 without Dirichlet data)
    want = np.zeros(dm.elem_dofs.shape) if dm.fixed_values is None else \
        np.asarray(dm.fixed_values)[np.maximum(-dm.elem_dofs - 1, 0)]
    got = fixed[np.maximum(-edofs - 1, 0)]
    assert np.array_equal(got[~unk], want[~unk])
