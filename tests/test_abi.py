"""The C ABI: exported symbols and struct layouts (no GPU needed).

Every function include/cgfd3d_gpu.h declares must be exported by the CUDA
library, the drop-in library must export drv_rk_curv_col_allstep, and the
ctypes mirror of cgfd_problem_t (cgfd3d_gb300/abi.py) must match the C
header's layout.
"""

import ctypes
import os
import re
import subprocess
import tempfile

from cgfd3d_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(REPO, "include", "cgfd3d_gpu.h")
BUILD = os.path.join(REPO, "cgfd3d_gb300", "_build")


def declared_functions():
    text = open(HDR).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cgfd_[a-z0-9_]+)\s*\(", text)))


def exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib], check=True,
                         capture_output=True, text=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_every_declared_function_is_exported():
    names = declared_functions()
    assert len(names) >= 15
    syms = exported(os.path.join(BUILD, "libcgfd3d_gpu.so"))
    missing = [n for n in names if n not in syms]
    assert not missing, missing


def test_library_loads_without_gpu():
    lib = ctypes.CDLL(os.path.join(BUILD, "libcgfd3d_gpu.so"))
    lib.cgfd_abi_version.restype = ctypes.c_int
    assert lib.cgfd_abi_version() == abi.CGFD_ABI_VERSION
    dl = ctypes.CDLL(os.path.join(BUILD, "libcgfd3d_dropin.so"))
    assert hasattr(dl, "drv_rk_curv_col_allstep")


def test_problem_struct_layout():
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cgfd3d_gpu.h"',
             "int main(void){",
             'printf("size %zu\\n", sizeof(cgfd_problem_t));',
             'printf("face %zu\\n", sizeof(cgfd_pml_face_t));']
    for name, _ in abi.Problem._fields_:
        cn = "lambda" if name == "lambda_" else name
        lines.append('printf("%s %%zu\\n", offsetof(cgfd_problem_t, %s));' % (name, cn))
    lines.append("return 0;}")
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "p.c"), "w") as f:
        f.write("\n".join(lines))
    subprocess.run(["gcc", "-I" + os.path.join(REPO, "include"), "-o",
                    os.path.join(d, "p"), os.path.join(d, "p.c")], check=True)
    got = dict(ln.split() for ln in subprocess.run(
        [os.path.join(d, "p")], capture_output=True, text=True, check=True).stdout.splitlines())
    assert int(got["size"]) == ctypes.sizeof(abi.Problem)
    assert int(got["face"]) == ctypes.sizeof(abi.PmlFace)
    for name, _ in abi.Problem._fields_:
        assert int(got[name]) == getattr(abi.Problem, name).offset, name
