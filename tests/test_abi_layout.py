"""The ctypes mirrors of the C-ABI structs (topo_le_params, topo_le_stats in
include/topopt_gb300.h; LEParams, LEStats in the package's _lib.py) against
the C layout: a small C program compiled with the host compiler prints the
size and every field offset, and each must equal the ctypes one."""
import os
import shutil
import subprocess

import pytest

from topopt_in_petsc_transient_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {"topo_le_params": _lib.LEParams, "topo_le_stats": _lib.LEStats}


def _program(tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "topopt_gb300.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append('    printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('    printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["    return 0;", "}"]
    src = tmp_path / "abi_layout.c"
    src.write_text("\n".join(lines) + "\n")
    return src


def test_ctypes_structs_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    exe = str(tmp_path / "abi_layout")
    r = subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(_program(tmp_path)), "-o", exe],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60).stdout.split("\n")
    c = {}
    for line in out:
        if line.strip():
            *key, val = line.split()
            c[" ".join(key)] = int(val)
    for cname, py in STRUCTS.items():
        import ctypes
        assert c["%s size" % cname] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert c["%s %s" % (cname, fname)] == getattr(py, fname).offset, (cname, fname)
