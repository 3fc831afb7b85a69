"""Reference outputs of the flat benchmark configuration at its stated size.

The configuration: isotropic elastic model on a 100 x 100 x 60 grid,
dx = dy = dz = 100 m, flat free surface (traction image), homogeneous
Vp/Vs/rho = 6000/3464/2700, CFS-PML with 10 layers on the five non-surface
faces (alpha_max = pi * fc = 6.283, beta_max = 2, ref_vel = 6000), explosive
moment source (Mxx = Myy = Mzz = 1e16) at the grid centre 2 km deep (20
cells), Ricker wavelet fc = 2 Hz, t0 = 0.6 s, 20 receivers on a surface line
(grid index start (10, 50, 59), step (4, 0, 0)) and the same 20 points as
stations, dt = 0.005 s, number_of_time_steps = 500 -- which the reference
runs as 501 steps (forward/main_curv_col_el_3d.c:615, nt_total = steps + 1).

The reference CPU build (oracle/_ref/cgfd3d_ref_dump, built by
``make -C oracle``) runs it from a par file, a source file and a station
file this script writes (tests/golden/make_golden.py's writers), and the
capture wrapper dumps every input and output of the time loop.  The
fixture keeps the inputs (constant volumes compress to almost nothing), the
line and station seismograms (9 components x 501 samples), and from the
final wavefield four planes through the source instead of the whole volume:
the free surface k = nk2, the source plane k = nk2 - 20, and the vertical
planes j = 53 and i = 53 (padded indices).  A second run of the same case
with number_of_time_steps = 250 adds the same planes after 251 steps
(out.t251.plane.*), a snapshot taken while the wavefield still fills the
model; its seismograms are checked to be the first 251 samples of the long
run's.

This script needs the reference tree and runs only where it exists:

    python tests/golden/configs/make_config_golden.py [--ref <reference tree>]

The reference tree defaults to $CGFD_REF_TREE.
"""

import argparse
import json
import math
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.dirname(HERE)
REPO = os.path.dirname(os.path.dirname(GOLDEN))
sys.path.insert(0, GOLDEN)

import make_golden  # noqa: E402  (writers and the dump reader)

C0 = dict(
    ni=100, nj=100, nk=60, dh=100.0, topo=False, medium="elastic_iso",
    media_override=(6000.0, 3464.0, 2700.0),
    pml=dict(x_left=10, x_right=10, y_front=10, y_back=10, z_bottom=10),
    pml_alpha_max=math.pi * 2.0,
    free=True, seed=None, steps=500, dt=0.005,
    src=dict(kind="moment", loc=(50.0, 50.0, 20.0), spatial="point",
             m=(1e16, 1e16, 1e16, 0.0, 0.0, 0.0), fc=2.0, t0=0.6),
    stations=[(10.0 + 4 * n, 50.0, 0.0, 1) for n in range(20)],
    lines=[dict(start=(10, 50, 59), incre=(4, 0, 0), count=20)],
)

# planes of the final wavefield kept in the fixture (padded indices)
PLANES = {"k": [62, 42], "j": [53], "i": [53]}


def planes_of(wav, ncmp, nx, ny, nz):
    """The kept planes of one wavefield level (ncmp x nz x ny x nx)."""
    w = np.asarray(wav, np.float32).reshape(ncmp, nz, ny, nx)
    out = {}
    for k in PLANES["k"]:
        out["k%d" % k] = np.ascontiguousarray(w[:, k, :, :])
    for j in PLANES["j"]:
        out["j%d" % j] = np.ascontiguousarray(w[:, :, j, :])
    for i in PLANES["i"]:
        out["i%d" % i] = np.ascontiguousarray(w[:, :, :, i])
    return out


def run_reference(c, ref_bin):
    """One reference run of case c: the trimmed dump (inputs, outputs, the
    final state as out.wav.final)."""
    work = tempfile.mkdtemp(prefix="cgfd_c0_")
    try:
        os.makedirs(os.path.join(work, "out"))
        os.makedirs(os.path.join(work, "tmp"))
        make_golden.write_par(os.path.join(work, "par.json"), c, work)
        make_golden.write_src(os.path.join(work, "case.src"), c)
        make_golden.write_station(os.path.join(work, "case.station"), c)
        env = dict(os.environ)
        env["CGFD_DUMP_FILE"] = os.path.join(work, "dump.bin")
        env["CGFD_DUMP_MEDIA"] = "%g,%g,%g" % c["media_override"]
        r = subprocess.run([ref_bin, os.path.join(work, "par.json"), "0"],
                           cwd=work, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout[-4000:] + r.stderr[-4000:])
            raise RuntimeError("reference run failed")
        return make_golden.trim(make_golden.read_dump(os.path.join(work, "dump.bin")))
    finally:
        shutil.rmtree(work, ignore_errors=True)


def run_c0(ref_bin, out_path):
    """The 501-step run, plus the planes of a 251-step run of the same case
    (a snapshot while the wavefield is still strong) as out.t251.plane.*;
    the shorter run's seismograms must be the prefix of the longer one's."""
    d = run_reference(C0, ref_bin)
    mid = run_reference(dict(C0, steps=250), ref_bin)
    nt = int(mid["nt_total"][0])
    assert nt == 251
    g = mid["gd.dims"]
    nx, ny, nz = int(g[3]), int(g[4]), int(g[5])
    ncmp = int(mid["wav.ncmp"][0])
    line = d["out.line.0.seismo"].reshape(-1, ncmp, int(d["line.max_nt"][0]))
    line_mid = mid["out.line.0.seismo"].reshape(-1, ncmp, nt)
    assert np.array_equal(line[:, :, :nt], line_mid), "251-step run is not a prefix"
    for name, v in planes_of(mid["out.wav.final"], ncmp, nx, ny, nz).items():
        d["out.t251.plane." + name] = v
    return finish_c0(d, out_path)


def finish_c0(d, out_path):
    c = C0
    g = d["gd.dims"]
    nx, ny, nz = int(g[3]), int(g[4]), int(g[5])
    ncmp = int(d["wav.ncmp"][0])
    final = d.pop("out.wav.final")
    for name, v in planes_of(final, ncmp, nx, ny, nz).items():
        d["out.wav.plane." + name] = v
    for k in [k for k in d if k.startswith("out.pml.")]:
        d.pop(k)
    d["case.json"] = np.frombuffer(json.dumps(c).encode(), dtype=np.uint8)
    np.savez_compressed(out_path, **d)
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CGFD_REF_TREE", ""))
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(a.ref):
        sys.exit("give the reference tree with --ref or $CGFD_REF_TREE")
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8",
                    "REF=" + a.ref], check=True, capture_output=True)
    ref_bin = os.path.join(REPO, "oracle", "_ref", "cgfd3d_ref_dump")
    out = os.path.join(HERE, "c0_flat_explosion_501.npz")
    d = run_c0(ref_bin, out)
    print("c0_flat_explosion_501:", len(d), "arrays,", os.path.getsize(out) // 1024, "KiB")


if __name__ == "__main__":
    main()
