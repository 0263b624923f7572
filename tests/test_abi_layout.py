"""The ctypes mirrors of the C ABI's structs have the header's layout.

A C program compiled with the host compiler against include/gomc_gb300.h
prints sizeof and every field's offsetof; each must equal the ctypes
Structure's, so that a field added on one side only fails here rather than
shifting the parameters a caller passes.  No GPU is involved.
"""
import ctypes
import os
import shutil
import subprocess

import pytest

from gomc_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# ctypes class -> C typedef
MIRRORS = {
    _lib.SystemDesc: "gb_system_desc",
    _lib.Config: "gb_config",
    _lib.McParams: "gb_mc_params",
    _lib.McShape: "gb_mc_shape",
    _lib.ServerConfig: "gb_server_config",
    _lib.GemcDesc: "gb_gemc_desc",
    _lib.GemcConfig: "gb_gemc_config",
    _lib.GomcChk: "gb_gomc_chk",
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>',
             '#include "gomc_gb300.h"', 'int main(void) {']
    for cls, name in MIRRORS.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (name, name))
        for field in cls._fields_:
            f = field[0]
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));'
                         % (name, f, name, f))
    lines += ['  return 0;', '}']
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True,
                         text=True).stdout
    table = {}
    for line in out.splitlines():
        name, key, val = line.split()
        table[(name, key)] = int(val)
    return table


@pytest.mark.parametrize("cls", list(MIRRORS), ids=lambda c: c.__name__)
def test_struct_layout_matches_header(c_layout, cls):
    name = MIRRORS[cls]
    assert ctypes.sizeof(cls) == c_layout[(name, "sizeof")], name
    for field in cls._fields_:
        f = field[0]
        assert getattr(cls, f).offset == c_layout[(name, f)], (name, f)
