"""The drop-in integration, checked where the GetDP sources are present
(the development host; skipped elsewhere): build_getdp.sh compiles the
unchanged GetDP sources with LinAlg_GB300.cpp in place of the Sparskit
backend and links the program against libgetdp_gb300.so; the program then
runs the reference's own example (a copy of examples/magnet.*) through its
parser and pre-processing into the backend."""
import os
import shutil
import subprocess

import pytest

from oracle import refsrc

GETDP_SRC = refsrc.source_dir() or ""
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

pytestmark = pytest.mark.skipif(
    not os.path.exists(os.path.join(GETDP_SRC, "src", "kernel", "LinAlg.h")),
    reason="GetDP sources not present")


def test_getdp_builds_and_links_with_the_gb300_backend(tmp_path):
    from getdp_gb300 import build
    build.build()
    out = tmp_path / "getdp_build"
    r = subprocess.run(["bash", os.path.join(ROOT, "getdp_gb300", "getdp_backend",
                                             "build_getdp.sh"), GETDP_SRC, str(out)],
                       capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    exe = out / "getdp"
    assert exe.exists()
    # the reference's own example (it includes ../templates), run in a
    # scratch copy
    shutil.copytree(os.path.join(GETDP_SRC, "examples"), tmp_path / "examples")
    shutil.copytree(os.path.join(GETDP_SRC, "templates"), tmp_path / "templates")
    work = tmp_path / "examples"
    r = subprocess.run([str(exe), "magnet.pro", "-solve", "#1", "-v", "3"], cwd=work,
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
