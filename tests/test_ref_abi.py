"""Layouts of the reference structs the drop-in entry point reads.

include/cgfd3d_ref_abi.h restates the layouts of the CGFD3D structs; the
ctypes mirrors in cgfd3d_gb300/refabi.py restate them again for Python.  A
compiled probe prints sizeof/offsetof for every field; the ctypes offsets must
match the restated header everywhere, and where the reference tree is present
the restated header must match the reference's own headers.
"""

import os
import subprocess
import tempfile

import pytest

from cgfd3d_gb300 import refabi

from helpers import ref_tree

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = ref_tree() or ""


def _fields():
    out = []
    for cname, cls in refabi.STRUCTS.items():
        out.append((cname, None, C_sizeof(cls)))
        for name, _ in cls._fields_:
            out.append((cname, name, getattr(cls, name).offset))
    return out


def C_sizeof(cls):
    import ctypes
    return ctypes.sizeof(cls)


def _probe(includes, defines):
    lines = ["#include <stdio.h>", "#include <stddef.h>"] + includes + ["int main(void){"]
    for cname, field, _ in _fields():
        if field is None:
            lines.append('printf("%%s %%zu\\n", "%s", sizeof(%s));' % (cname, cname))
        else:
            cf = "lambda" if field == "lambda_" else field
            lines.append('printf("%%s.%%s %%zu\\n", "%s", "%s", offsetof(%s, %s));'
                         % (cname, field, cname, cf))
    lines.append("return 0;}")
    d = tempfile.mkdtemp()
    src = os.path.join(d, "probe.c")
    exe = os.path.join(d, "probe")
    with open(src, "w") as f:
        f.write("\n".join(lines))
    subprocess.run(["gcc", "-o", exe, src] + defines, check=True)
    res = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    vals = {}
    for ln in res.splitlines():
        k, v = ln.split()
        vals[k] = int(v)
    return vals


def _key(cname, field):
    return cname if field is None else "%s.%s" % (cname, field)


def test_ctypes_mirror_matches_restated_header():
    got = _probe(['#include "cgfd3d_ref_abi.h"'], ["-I" + os.path.join(REPO, "include")])
    for cname, field, off in _fields():
        assert got[_key(cname, field)] == off, (cname, field)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "forward")),
                    reason="reference tree not present")
def test_restated_header_matches_reference_headers():
    mine = _probe(['#include "cgfd3d_ref_abi.h"'], ["-I" + os.path.join(REPO, "include")])
    theirs = _probe(['#include "drv_rk_curv_col.h"'],
                    ["-I" + os.path.join(REPO, "oracle", "shim"),
                     "-I" + os.path.join(REF, "forward"), "-I" + os.path.join(REF, "lib")])
    assert mine == theirs
