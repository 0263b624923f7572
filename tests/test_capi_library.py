"""The C-ABI library builds for sm_103a, loads, and exports every entry
point include/gomc_gb300.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "gomc_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from gomc_gb300 import _lib, build
    build.build()
    L = ctypes.CDLL(build.LIB)
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(L, n), n
    # the Python binding declares the same set
    assert set(names) == set(_lib.SIGNATURES)


def test_library_is_sm103a_only():
    from gomc_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
