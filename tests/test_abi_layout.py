"""The ctypes mirrors of the header's structs have the C layout: a tiny C
program compiled from include/pycbf_gb300.h prints every struct's size and
field offsets, which must equal ctypes' (CPU only; needs a C compiler)."""
import ctypes as ct
import os
import shutil
import subprocess
import tempfile

import pytest

from pycbf_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {
    "pycbf_gb_rfinfo": _lib.RFInfo,
    "pycbf_gb_synthetic": _lib.SyntheticGeom,
    "pycbf_gb_batch_job": _lib.BatchJob,
    "pycbf_gb_batch_info": _lib.BatchInfo,
}


def test_struct_layouts_match_the_header():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "pycbf_gb300.h"',
             "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    work = os.path.join(ROOT, "pycbf_gb300", "_build")  # the build's scratch folder
    os.makedirs(work, exist_ok=True)
    with tempfile.TemporaryDirectory(dir=work) as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as fp:
            fp.write("\n".join(lines))
        subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                       check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        name, key, val = line.split()
        got[(name, key)] = int(val)
    for cname, cls in STRUCTS.items():
        assert got[(cname, "size")] == ct.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)
