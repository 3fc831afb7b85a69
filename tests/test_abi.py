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


def test_dropin_header_functions_are_exported():
    text = re.sub(r"/\*.*?\*/", "", open(os.path.join(REPO, "include", "cgfd3d_dropin.h")).read(),
                  flags=re.S)
    names = sorted(set(re.findall(r"\b(cgfd_[a-z0-9_]+)\s*\(", text)))
    assert names == ["cgfd_gpu_last_error"]
    syms = exported(os.path.join(BUILD, "libcgfd3d_dropin.so"))
    assert "drv_rk_curv_col_allstep" in syms
    assert not [n for n in names if n not in syms]


def test_dropin_failure_code_is_kept_for_exit_handlers():
    """An unsupported configuration (an RK scheme other than RK4) ends the
    process with status 1, as the reference's errors do, before any device
    call; cgfd_gpu_last_error() then reports CGFD_EINVAL to an atexit
    handler."""
    prog = r"""
#include <stdio.h>
#include <stdlib.h>
#include "cgfd3d_ref_abi.h"
#include "cgfd3d_dropin.h"
#include "cgfd3d_gpu.h"
static void report(void) { printf("code %d\n", cgfd_gpu_last_error()); fflush(stdout); }
int main(void)
{
  fd_t fd = {0};
  fd.num_rk_stages = 3;
  fd.num_of_pairs = 8;
  printf("before %d\n", cgfd_gpu_last_error());
  atexit(report);
  drv_rk_curv_col_allstep(&fd, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL, NULL,
                          NULL, 0.01f, 1, 0.0f, NULL, NULL, 0, 0, 0);
  printf("returned\n");
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        with open(src, "w") as f:
            f.write(prog)
        subprocess.run(["gcc", "-O1", "-I" + os.path.join(REPO, "include"), "-o", exe, src,
                        "-L" + BUILD, "-lcgfd3d_dropin", "-Wl,-rpath," + BUILD], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
    assert "before 0" in r.stdout and "returned" not in r.stdout
    assert "code %d" % 1 in r.stdout      # CGFD_EINVAL
    assert "is not supported" in r.stderr


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
