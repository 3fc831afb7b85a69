"""Host logic of slice/snapshot output (no GPU): box layout, float counts,
the snapshot schedule of the reference's writer."""

import ctypes
import os
import subprocess
import tempfile

from cgfd3d_gb300 import abi, output

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class _P:
    ni1, ni2, nj1, nj2, nk1, nk2 = 3, 22, 3, 17, 3, 12
    nx, ny, nz = 26, 21, 16
    ncmp = 9
    medium_type = abi.CGFD_MEDIUM_ELASTIC_ISO


def test_box_struct_layout():
    src = ('#include <stdio.h>\n#include "cgfd3d_gpu.h"\n'
           'int main(void){printf("%zu\\n", sizeof(cgfd_box_t));return 0;}\n')
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "b.c"), "w") as f:
        f.write(src)
    subprocess.run(["gcc", "-I" + os.path.join(REPO, "include"), "-o",
                    os.path.join(d, "b"), os.path.join(d, "b.c")], check=True)
    got = int(subprocess.run([os.path.join(d, "b")], capture_output=True, text=True,
                             check=True).stdout)
    assert got == ctypes.sizeof(abi.Box) == 44


def test_slice_boxes_follow_the_reference_writer():
    p = _P()
    bx, by, bz = output.slice_boxes(p, x=[5], y=[7], z=[12])
    assert (bx.i1, bx.ni, bx.j1, bx.nj, bx.k1, bx.nk) == (5, 1, 3, 15, 3, 10)
    assert (by.i1, by.ni, by.j1, by.nj, by.k1, by.nk) == (3, 20, 7, 1, 3, 10)
    assert (bz.i1, bz.ni, bz.j1, bz.nj, bz.k1, bz.nk) == (3, 20, 3, 15, 12, 1)
    assert all(b.c1 == 0 and b.c2 == 8 for b in (bx, by, bz))
    p.medium_type, p.ncmp = abi.CGFD_MEDIUM_VISCOELASTIC_ISO, 27
    assert output.slice_boxes(p, z=[12])[0].c2 == 8


def test_box_floats_from_the_library():
    from cgfd3d_gb300 import _lib
    L = _lib.lib()          # loads without a GPU; cgfd_box_floats makes no CUDA call
    arr = (abi.Box * 2)(abi.Box(0, 8, 3, 20, 1, 3, 15, 1, 3, 1, 1),
                        abi.Box(3, 5, 0, 4, 2, 0, 3, 3, 0, 2, 5))
    assert L.cgfd_box_floats(arr, 2) == 9 * 20 * 15 + 3 * 4 * 3 * 2
    arr[1].dk = 0
    assert L.cgfd_box_floats(arr, 2) == 0
    arr[1].dk, arr[1].c2 = 1, 2
    assert L.cgfd_box_floats(arr, 2) == 0


def _due_c(it, nt_total, it1, dit):
    """The C rule of io_snap_nc_put, with C's truncating division."""
    import math
    mod = math.fmod(it - it1, dit)
    num = int((it - it1) / dit)
    lim = int((nt_total - it1) / dit)
    return it >= it1 and num <= lim and mod == 0


def test_snapshot_schedule():
    for nt_total in (1, 7, 40):
        for it1 in (0, 3, 45):
            for dit in (1, 4, 7):
                got = [output.snapshot_due(it, nt_total, it1, dit) for it in range(nt_total)]
                assert got == [_due_c(it, nt_total, it1, dit) for it in range(nt_total)]
    assert [it for it in range(20) if output.snapshot_due(it, 20, 2, 5)] == [2, 7, 12, 17]


def test_sac_files_match_reference(tmp_path):
    """Station, station-strain and line SAC files equal, byte for byte, the
    files the reference's own writers made from the same seismograms."""
    import numpy as np
    z = np.load(os.path.join(REPO, "tests", "golden", "output", "sac_output.npz"))
    d = {k: z[k] for k in z.files if not k.startswith("file:")}
    names = [str(n) for n in d["names"]]
    evt, dt = str(d["evtnm"]), float(d["dt"])
    output.write_station_sac(str(tmp_path), evt, names, d["xyz"], d["seismo"], dt)
    output.write_station_strain_sac(str(tmp_path), evt, names, d["xyz"], d["seismo"],
                                    d["lam"], d["mu"], dt)
    output.write_line_sac(str(tmp_path), evt, str(d["line_name"]), d["line_seq"],
                          d["line_xyz"], d["line_seismo"], dt)
    want = {k[5:]: z[k].tobytes() for k in z.files if k.startswith("file:")}
    got = {fn: open(os.path.join(tmp_path, fn), "rb").read() for fn in os.listdir(tmp_path)}
    assert sorted(got) == sorted(want)
    for fn in want:
        assert got[fn] == want[fn], fn


def test_sac_header_fields():
    """Header fields of the SAC format at their published offsets."""
    import struct
    b = output.sac_bytes([1.0, 2.0, 3.0, 4.0], 0.5, 10.0, 20.0, 30.0, 0.5)
    assert len(b) == 632 + 16
    f = struct.unpack("<70f", b[:280])
    i = struct.unpack("<40i", b[280:440])
    assert f[0] == 0.5 and f[5] == 0.0 and f[6] == 1.5 and f[1] == -12345.0
    assert (f[31], f[32], f[33], f[34]) == (10.0, 20.0, 30.0, 0.5)
    assert i[6] == 6 and i[9] == 4 and i[15] == 1 and i[35] == 1 and i[0] == -12345
    assert b[440:448] == b"-12345\0\0" and b[448:464] == b"-12345  " + b"\0" * 8
    assert struct.unpack("<4f", b[632:]) == (1.0, 2.0, 3.0, 4.0)
