"""Build tests/getdp_stub/_build/drive_linalg: GetDP's LinAlg call sequence
through the unchanged backend file getdp_gb300/getdp_backend/LinAlg_GB300.cpp,
compiled against the stand-in GetDP headers of this folder and linked with
the library.  Test infrastructure: it runs where GetDP's sources are absent
(the GPU machine), so that the backend's C++ itself is exercised on a GPU.

The prototypes of the stand-in LinAlg.h are the definitions LinAlg_GB300.cpp
itself makes (written to _build/linalg_protos.h)."""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
BACKEND = os.path.join(ROOT, "getdp_gb300", "getdp_backend", "LinAlg_GB300.cpp")
OUT = os.path.join(HERE, "_build")
EXE = os.path.join(OUT, "drive_linalg")

_DEF = re.compile(r"^((?:void|int|double|bool)\s+LinAlg_\w+\s*\([^)]*\))\s*\{", re.M)


def prototypes(text: str) -> str:
    """Declarations of the LinAlg_* functions a backend file defines."""
    return "".join(f"{m.group(1)};\n" for m in _DEF.finditer(text))


def build() -> str:
    from getdp_gb300 import build as B
    lib = B.build()
    srcs = [BACKEND, os.path.join(HERE, "stub.cpp"), os.path.join(HERE, "drive_linalg.cpp")]
    deps = srcs + [lib, os.path.join(ROOT, "include", "getdp_gb300.h")] + \
        [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".h")]
    if os.path.exists(EXE) and os.path.getmtime(EXE) >= max(os.path.getmtime(d) for d in deps):
        return EXE
    os.makedirs(OUT, exist_ok=True)
    with open(BACKEND) as f:
        protos = prototypes(f.read())
    hdr = os.path.join(OUT, "linalg_protos.h")
    with open(hdr, "w") as f:
        f.write("/* generated from LinAlg_GB300.cpp */\n" + protos)
    cmd = ["g++", "-O2", "-std=c++17", "-w", "-I", OUT, "-I", HERE,
           "-I", os.path.join(ROOT, "include"), *srcs, "-o", EXE,
           "-L", os.path.dirname(lib), "-lgetdp_gb300",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"drive_linalg build failed:\n{r.stdout}\n{r.stderr}")
    return EXE


if __name__ == "__main__":
    print(build())
