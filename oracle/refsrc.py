"""ORACLE — test infrastructure only.

Where the reference GetDP sources are, for the tests that read its own files
(the example mesh, the sources the drop-in build compiles): the
``GETDP_SOURCE_DIR`` environment variable, else the directory that
``oracle/build_ref.sh`` compiled the reference from (recorded in
``oracle/_ref/source_dir``).  ``None`` where neither exists, e.g. on a host
that only received the built library.
"""
from __future__ import annotations

import os

HERE = os.path.dirname(os.path.abspath(__file__))


def source_dir():
    cands = [os.environ.get("GETDP_SOURCE_DIR")]
    rec = os.path.join(HERE, "_ref", "source_dir")
    if os.path.exists(rec):
        with open(rec) as f:
            cands.append(f.read().strip())
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "src", "kernel")):
            return c
    return None
