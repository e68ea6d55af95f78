"""The C-ABI library loads and exports every entry point include/*.h
declares (no GPU needed: nothing is called)."""
import ctypes
import glob
import os
import re

import pytest

from getdp_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(gb300_\w+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    build.build()
    return ctypes.CDLL(build.LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gb300_solve" in names and "gb300_generate_values" in names
    assert len(names) > 30


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    # the Python binding declares a signature for every exported function
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_library_is_built_for_sm_103a():
    assert build.ARCH == "-gencode=arch=compute_103a,code=sm_103a"
    assert os.path.getsize(build.LIB) > 0
