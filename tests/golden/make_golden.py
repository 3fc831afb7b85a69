"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the CGFD3D reference CPU solver (built by ``make -C oracle`` into
``oracle/_ref/cgfd3d_ref_dump`` from the reference sources) on small
deterministic cases and stores, per case, every input array that
``drv_rk_curv_col_allstep`` (forward/drv_rk_curv_col.c:28) reads and every
output it produces, as a compressed ``<case>.npz``.

The reference's own setup code builds each case from a par file, a source
file, a station file and (for topography) a ``.gdlay`` grid-layer file that
this script writes.  With ``seed`` set, the capture wrapper (oracle/ref_dump.c)
perturbs the media and seeds the wavefield and the PML auxiliary variables
with noise before the time loop, so every tap of every operator and every
boundary branch is exercised from the first step.

This script needs the reference tree and runs only where it exists; the
fixtures it writes are committed and are all the tests need elsewhere.

    python tests/golden/make_golden.py [--ref <reference tree>] [case ...]

The reference tree defaults to $CGFD_REF_TREE.
"""

import argparse
import json
import math
import os
import shutil
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

# --------------------------------------------------------------------------
# cases
# --------------------------------------------------------------------------

CASES = {
    # curvilinear topography, every boundary branch, seeded noise state,
    # Gaussian force + moment source, off-grid receivers, one line
    "iso_topo_noise": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_iso",
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        free=True, seed=12345, steps=9, dt=0.004,
        src=dict(kind="force+moment", loc=(8.3, 7.6, 4.0), spatial="gauss",
                 f=(1e15, -2e15, 3e15), m=(1e16, 2e16, -1e16, 0.5e16, -0.3e16, 0.2e16),
                 fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1), (12.0, 6.0, 3.4, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    # flat free surface, homogeneous medium, explosive point source, zero
    # initial state: a physically meaningful run with surface seismograms
    "iso_flat_explosion": dict(
        ni=30, nj=28, nk=24, dh=100.0, topo=False, medium="elastic_iso",
        media_override=(6000.0, 3464.0, 2700.0),
        pml=dict(x_left=6, x_right=6, y_front=6, y_back=6, z_bottom=6),
        free=True, seed=None, steps=120, dt=0.005,
        src=dict(kind="moment", loc=(15.0, 14.0, 8.0), spatial="point",
                 m=(1e16, 1e16, 1e16, 0.0, 0.0, 0.0), fc=10.0, t0=0.12),
        stations=[(5.0 + 2 * n, 14.0, 0.0, 1) for n in range(10)],
        lines=[dict(start=(0, 14, 23), incre=(3, 0, 0), count=10)],
    ),
    # VTI medium (the reference's built-in VTI test medium, perturbed +-10 %
    # per point by the seed) on the same curvilinear topography
    "vti_topo_noise": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_vti",
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        free=True, seed=4242, steps=9, dt=0.004,
        src=dict(kind="force+moment", loc=(8.3, 7.6, 4.0), spatial="gauss",
                 f=(1e15, -2e15, 3e15), m=(1e16, 2e16, -1e16, 0.5e16, -0.3e16, 0.2e16),
                 fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1), (12.0, 6.0, 3.4, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    # GMB visco-elastic isotropic medium with three Maxwell bodies (the
    # reference's built-in test medium: Qp 80, Qs 40), seeded noise state
    # including the memory variables
    "visco_topo_noise": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="viscoelastic_iso",
        visco=dict(type="gmb", number_of_maxwell=3, min_freq=0.5, max_freq=5.0,
                   refer_freq=1.58),
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        free=True, seed=9191, steps=9, dt=0.004,
        src=dict(kind="force+moment", loc=(8.3, 7.6, 4.0), spatial="gauss",
                 f=(1e15, -2e15, 3e15), m=(1e16, 2e16, -1e16, 0.5e16, -0.3e16, 0.2e16),
                 fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1), (12.0, 6.0, 3.4, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    # force sources whose spread reaches the free surface (the reference
    # then injects them through the traction image and vlow layers,
    # forward/src_t.c:153-314): a Gaussian force one cell below the
    # topography, and a point force at the flat surface
    "iso_surface_force": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_iso",
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        free=True, seed=2468, steps=9, dt=0.004,
        src=dict(kind="force", loc=(8.4, 7.3, 1.0), spatial="gauss",
                 f=(2e15, -1e15, 3e15), fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    "iso_surface_point_force": dict(
        ni=24, nj=20, nk=16, dh=100.0, topo=False, medium="elastic_iso",
        media_override=(6000.0, 3464.0, 2700.0),
        pml=dict(x_left=5, x_right=5, y_front=5, y_back=5, z_bottom=5),
        free=True, seed=None, steps=30, dt=0.005,
        src=dict(kind="force", loc=(12.0, 10.0, 0.0), spatial="point",
                 f=(0.0, 0.0, 1e15), fc=10.0, t0=0.12),
        stations=[(4.0 + 2 * n, 10.0, 0.0, 1) for n in range(8)],
        lines=[],
    ),
    "vti_surface_force": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_vti",
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        free=True, seed=1357, steps=9, dt=0.004,
        src=dict(kind="force", loc=(8.4, 7.3, 2.0), spatial="gauss",
                 f=(2e15, -1e15, 3e15), fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    # Graves Q attenuation (visco_config graves_Qs) of an elastic medium on
    # the topography, Qs perturbed +-10 % around the reference's test value
    "iso_topo_graves": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_iso",
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        visco=dict(type="graves_Qs", Qs_freq=2.0),
        free=True, seed=4242, steps=9, dt=0.004,
        src=dict(kind="moment", loc=(8.3, 7.6, 4.0), spatial="gauss",
                 m=(1e16, 2e16, -1e16, 0.5e16, -0.3e16, 0.2e16), fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    # exponential sponge (ablexp) on five faces instead of CFS-PML, flat
    # free surface, noise state
    "iso_flat_ablexp": dict(
        ni=24, nj=20, nk=16, dh=100.0, topo=False, medium="elastic_iso",
        pml={}, ablexp=dict(x_left=5, x_right=6, y_front=4, y_back=5, z_bottom=6),
        free=True, seed=99, steps=10, dt=0.005,
        src=dict(kind="moment", loc=(12.0, 10.0, 6.0), spatial="gauss",
                 m=(1e16, 1e16, 1e16, 0.0, 0.0, 0.0), fc=8.0, t0=0.05),
        stations=[(4.0 + 2 * n, 10.0, 0.0, 1) for n in range(6)],
        lines=[],
    ),
    # VTI medium on the topography with the sponge and Graves Q together
    "vti_topo_ablexp_graves": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_vti",
        pml={}, ablexp=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        visco=dict(type="graves_Qs", Qs_freq=1.5),
        free=True, seed=8642, steps=9, dt=0.004,
        src=dict(kind="force+moment", loc=(8.3, 7.6, 4.0), spatial="gauss",
                 f=(1e15, -2e15, 3e15), m=(1e16, 2e16, -1e16, 0.5e16, -0.3e16, 0.2e16),
                 fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1)],
        lines=[],
    ),
    # fully anisotropic medium (21 constants; a stable transversely
    # isotropic stiffness with every constant offset, see oracle/ref_dump.c)
    # on the topography, seeded noise state, every boundary branch
    "aniso_topo_noise": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_aniso",
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        free=True, seed=97531, steps=9, dt=0.004,
        src=dict(kind="force+moment", loc=(8.3, 7.6, 4.0), spatial="gauss",
                 f=(1e15, -2e15, 3e15), m=(1e16, 2e16, -1e16, 0.5e16, -0.3e16, 0.2e16),
                 fc=8.0, t0=0.05),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1), (12.0, 6.0, 3.4, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    # distributed (dd) sources at grid points next to an ordinary moment
    # source: force and moment rates of 12 points (interior, PML, free
    # surface, one column) read by the reference from a raw container
    # (oracle/shim/netcdf_null.c), three steps per read, input ending before
    # the last steps
    "iso_topo_dd": dict(
        ni=18, nj=16, nk=14, dh=100.0, topo=True, medium="elastic_iso",
        pml=dict(x_left=4, x_right=4, y_front=4, y_back=4, z_bottom=4),
        free=True, seed=1122, steps=9, dt=0.004,
        src=dict(kind="moment", loc=(8.3, 7.6, 4.0), spatial="point",
                 m=(1e16, 2e16, -1e16, 0.5e16, -0.3e16, 0.2e16), fc=8.0, t0=0.05),
        dd=dict(points=[(8, 7, 5), (8, 7, 9), (8, 7, 11), (2, 5, 6), (15, 12, 3),
                        (5, 13, 13), (12, 3, 13), (10, 10, 1), (6, 9, 12), (14, 6, 8),
                        (3, 3, 2), (9, 11, 13)],
                nt_per_read=3, dt_in=0.002, t_end=0.03, seed=77),
        stations=[(3.25, 4.5, 0.0, 1), (10.7, 9.1, 0.0, 1)],
        lines=[dict(start=(2, 8, 13), incre=(2, 0, 0), count=6)],
    ),
    # no free surface: PML on all six faces (z2 face included), noise state
    "iso_box_pml6": dict(
        ni=16, nj=14, nk=12, dh=100.0, topo=False, medium="elastic_iso",
        pml=dict(x_left=3, x_right=3, y_front=3, y_back=3, z_bottom=3, z_top=3),
        free=False, seed=777, steps=9, dt=0.004,
        src=dict(kind="moment", loc=(7.0, 6.0, 5.0), spatial="gauss",
                 m=(1e16, -1e16, 0.0, 1e16, 0.0, 0.0), fc=8.0, t0=0.05),
        stations=[(4.5, 5.5, 2.0, 1)],
        lines=[],
    ),
}


def topo_surface(x, y, Lx, Ly):
    """Smooth hill plus two bumps, amplitude ~1.5 grid cells."""
    r2 = ((x - 0.55 * Lx) ** 2 + (y - 0.45 * Ly) ** 2) / (0.35 * Lx) ** 2
    return (150.0 * np.exp(-r2)
            + 30.0 * np.sin(2 * np.pi * x / Lx) * np.cos(2 * np.pi * y / Ly))


def write_gdlay(path, c):
    nx, ny = c["ni"] + 6, c["nj"] + 6
    dh = c["dh"]
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    x = (ii - 3) * dh
    y = (jj - 3) * dh
    Lx, Ly = (nx - 6) * dh, (ny - 6) * dh
    ncell = c["nk"] + 2
    ztop = topo_surface(x, y, Lx, Ly)
    zbot = np.full_like(ztop, -ncell * dh)
    with open(path, "w") as f:
        f.write("2\n%d\n1\n%d %d\n" % (ncell, nx, ny))
        for z in (zbot, ztop):
            for j in range(ny):
                for i in range(nx):
                    f.write("%.6f %.6f %.6f\n" % (x[j, i], y[j, i], z[j, i]))


def write_par(path, c, work):
    faces = {"x_left": "boundary_x_left", "x_right": "boundary_x_right",
             "y_front": "boundary_y_front", "y_back": "boundary_y_back",
             "z_bottom": "boundary_z_bottom", "z_top": "boundary_z_top"}
    par = {
        "number_of_total_grid_points_x": c["ni"],
        "number_of_total_grid_points_y": c["nj"],
        "number_of_total_grid_points_z": c["nk"],
        "number_of_mpiprocs_x": 1,
        "number_of_mpiprocs_y": 1,
        "size_of_time_step": c["dt"],
        "number_of_time_steps": c["steps"],
        "time_window_length": c["dt"] * c["steps"],
        "check_stability": 1,
    }
    for key, nlay in c["pml"].items():
        par[faces[key]] = {"cfspml": {"number_of_layers": nlay,
                                      "alpha_max": c.get("pml_alpha_max", 3.14),
                                      "beta_max": 2.0, "ref_vel": 6000.0}}
    for key, nlay in c.get("ablexp", {}).items():
        par[faces[key]] = {"ablexp": {"number_of_layers": nlay, "ref_vel": 6000.0}}
    if c["free"]:
        par["boundary_z_top"] = {"free": "timg"}
    if c["topo"]:
        par["grid_generation_method"] = {"layer_interp": {
            "in_grid_layer_file": os.path.join(work, "grid.gdlay"),
            "refine_factor": [1, 1, 1],
            "horizontal_start_index": [3, 3],
            "vertical_last_to_top": 0}}
    else:
        par["grid_generation_method"] = {"cartesian": {
            "origin": [0.0, 0.0, -(c["nk"] - 1) * c["dh"]],
            "inteval": [c["dh"], c["dh"], c["dh"]]}}
    par.update({
        "is_export_grid": 0,
        "grid_export_dir": work,
        "metric_calculation_method": {"calculate": 1},
        "is_export_metric": 0,
        "medium": {"type": c["medium"], "input_way": "code", "code": "x",
                   "equivalent_medium_method": "loc"},
        **({"visco_config": c["visco"]} if "visco" in c else {}),
        "is_export_media": 0,
        "media_export_dir": work,
        "in_source_file": os.path.join(work, "case.src"),
        "is_export_source": 0,
        "source_export_dir": work,
        "source_spatial_distribution_type": c["src"]["spatial"],
        **({"in_ddsource_file": os.path.join(work, "dd.raw"),
            "ddsource_add_at_point": 1,
            "ddsource_nt_per_read": c["dd"]["nt_per_read"]} if "dd" in c else {}),
        "output_dir": os.path.join(work, "out"),
        "tmp_dir": os.path.join(work, "tmp"),
        "in_station_file": os.path.join(work, "case.station"),
        "receiver_line": [
            {"name": "line%d" % n, "grid_index_start": list(l["start"]),
             "grid_index_incre": list(l["incre"]),
             "grid_index_count": l["count"]}
            for n, l in enumerate(c["lines"])],
        "snapshot": [],
        "check_nan_every_nummber_of_steps": 0,
        "output_all": 0,
    })
    with open(path, "w") as f:
        json.dump(par, f, indent=2)


def write_src(path, c):
    s = c["src"]
    cmp_type = {"force": 1, "moment": 2, "force+moment": 3}[s["kind"]]
    lines = ["case_event", "1", "0 1.0", "%d 0" % cmp_type, "0 1",
             "%g %g %g" % s["loc"],
             "0.0 ricker %g %g" % (s["fc"], s["t0"])]
    vals = []
    if "f" in s and cmp_type in (1, 3):
        vals += list(s["f"])
    if "m" in s and cmp_type in (2, 3):
        vals += list(s["m"])
    lines.append(" ".join("%g" % v for v in vals))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_dd(path, c):
    """Distributed-source input in the raw container of the NetCDF shim
    (oracle/shim/netcdf_null.c): grid-index locations, per-point force and
    moment rates sampled every dt_in from 0 to t_end (smooth random pulses)."""
    d = c["dd"]
    rng = np.random.default_rng(d["seed"])
    pts = np.array(d["points"], np.float32)
    n = len(pts)
    t = np.arange(0.0, d["t_end"] + 0.5 * d["dt_in"], d["dt_in"]).astype(np.float32)
    t[0] = 0.0
    pulses = {}
    for name in ("Fx", "Fy", "Fz", "Mxx_rate", "Myy_rate", "Mzz_rate", "Myz_rate",
                 "Mxz_rate", "Mxy_rate"):
        amp = (1e15 if name.startswith("F") else 1e17) * rng.standard_normal((n, 1))
        tc = rng.uniform(0.005, 0.02, (n, 1))
        w = rng.uniform(0.004, 0.01, (n, 1))
        pulses[name] = (amp * np.exp(-((t[None, :] - tc) / w) ** 2)).astype(np.float32)
    b = b"CGNCRAW1"
    atts = [("location_is_axis", 0), ("z_is_depth", 0)]
    b += struct.pack("<i", len(atts))
    for nm, v in atts:
        b += nm.encode().ljust(32, b"\0") + struct.pack("<i", v)
    dims = [("time", len(t)), ("number", n)]
    b += struct.pack("<i", len(dims))
    for nm, ln in dims:
        b += nm.encode().ljust(32, b"\0") + struct.pack("<q", ln)
    vars_ = [("time", [0], t), ("x", [1], pts[:, 0]), ("y", [1], pts[:, 1]),
             ("z", [1], pts[:, 2])] + [(nm, [1, 0], v) for nm, v in pulses.items()]
    b += struct.pack("<i", len(vars_))
    for nm, dd, data in vars_:
        b += nm.encode().ljust(32, b"\0") + struct.pack("<i4i", len(dd), *(dd + [0] * (4 - len(dd))))
        b += np.ascontiguousarray(data, "<f4").tobytes()
    with open(path, "wb") as f:
        f.write(b)


def write_station(path, c):
    with open(path, "w") as f:
        f.write("%d\n" % len(c["stations"]))
        for n, (x, y, z, depth) in enumerate(c["stations"]):
            f.write("r%d 0 %d %g %g %g\n" % (n, depth, x, y, z))


def read_dump(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        name = data[pos:pos + 48].split(b"\0", 1)[0].decode()
        kind = chr(data[pos + 48])
        (count,) = struct.unpack("<q", data[pos + 56:pos + 64])
        pos += 64
        dt = {"f": np.float32, "i": np.int32, "d": np.float64}[kind]
        nb = count * np.dtype(dt).itemsize
        out[name] = np.frombuffer(data[pos:pos + nb], dtype=dt).copy()
        pos += nb
    return out


def trim(d):
    """Keep the final wavefield and PML levels only.

    The reference swaps its pre/end level pointers after every step
    (forward/drv_rk_curv_col.c:530-542), so after nt_total steps the state
    sits in level 3 when nt_total is odd and in level 0 when it is even.
    """
    nt = int(d["nt_total"][0])
    lev = 3 if nt % 2 == 1 else 0
    out = {}
    for k, v in d.items():
        if k.startswith("out.wav.level"):
            if k == "out.wav.level%d" % lev:
                out["out.wav.final"] = v
            continue
        if k.startswith("out.pml.") and k.endswith(".aux"):
            n4 = v.size // 4
            out[k.replace(".aux", ".final")] = v[lev * n4:(lev + 1) * n4]
            continue
        out[k] = v
    return out


def run_case(name, c, ref_bin):
    work = tempfile.mkdtemp(prefix="cgfd_golden_")
    try:
        os.makedirs(os.path.join(work, "out"))
        os.makedirs(os.path.join(work, "tmp"))
        if c["topo"]:
            write_gdlay(os.path.join(work, "grid.gdlay"), c)
        write_par(os.path.join(work, "par.json"), c, work)
        write_src(os.path.join(work, "case.src"), c)
        write_station(os.path.join(work, "case.station"), c)
        if "dd" in c:
            write_dd(os.path.join(work, "dd.raw"), c)
        env = dict(os.environ)
        env["CGFD_DUMP_FILE"] = os.path.join(work, "dump.bin")
        if c.get("seed") is not None:
            env["CGFD_DUMP_SEED"] = str(c["seed"])
        if c.get("media_override") is not None:
            env["CGFD_DUMP_MEDIA"] = "%g,%g,%g" % c["media_override"]
        r = subprocess.run([ref_bin, os.path.join(work, "par.json"), "0"],
                           cwd=work, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout[-4000:] + r.stderr[-4000:])
            raise RuntimeError("reference run failed for %s" % name)
        d = trim(read_dump(os.path.join(work, "dump.bin")))
        d["case.json"] = np.frombuffer(json.dumps(c).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        return d
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CGFD_REF_TREE", ""))
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(a.ref):
        sys.exit("give the reference tree with --ref or $CGFD_REF_TREE")
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8",
                    "REF=" + a.ref], check=True, capture_output=True)
    ref_bin = os.path.join(REPO, "oracle", "_ref", "cgfd3d_ref_dump")
    for name in (a.cases or CASES):
        d = run_case(name, CASES[name], ref_bin)
        print(name, len(d), "arrays,",
              os.path.getsize(os.path.join(HERE, name + ".npz")) // 1024, "KiB")


if __name__ == "__main__":
    main()
