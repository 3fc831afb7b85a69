"""Generate tests/golden/media/layer_el_iso.npz from the reference's
layered-model discretisation.

Runs ``oracle/_ref/ref_probe layer`` (the reference's
media_layer2model_el_iso, media/media_layer2model.cpp:140-190, built by
``make -C oracle``) on a seeded elastic isotropic layered model (.md3lay
text, media/media_read_file.cpp:22-240) and a curvilinear grid, with the
equivalent-medium methods "loc", "har" and "ari": four interfaces, one of them flat and lying
exactly on a grid level (the points on it take the mean of the two layers),
velocity and density gradients with power laws, and grid points above the
top interface.  Stores the model, the grid and the reference's lambda, mu
and rho.

It also writes layer_el_vti.npz: three elastic VTI layered models
(elastic_vti_prem, elastic_vti_thomsen, elastic_vti_cij) on a smaller grid,
discretised by media_layer2model_el_vti (media/media_layer2model.cpp:192-247)
with every method for the Thomsen model and one or two for the others; keys
<type>_<method>_<c11|c33|c55|c66|c13|rho> and <type>_md3lay.

And layer_onecmp.npz: a one-component layered model (a Qs-like value with
gradients and powers) on the first grid, discretised by
media_layer2model_onecmp (media/media_layer2model.cpp:47-88) with each
method; keys md3lay, var_loc, var_har, var_ari.

And bin_model.npz: a model given as binary volumes (stored z fastest,
then x, then y; z decreasing; wider than the grid in x and y and shallower
than its bottom) interpolated on the first grid by media_bin2model_el_iso
and media_bin2model_vis_iso (media/media_bin2model.cpp:27-432); keys
order, size, spacing, origin, ext (xmin xmax ymin ymax), rho_vol, vp_vol,
vs_vol, qp_vol, qs_vol (file order) and rho, lam, mu, Qp, Qs.

And grid_el_iso.npz: an elastic isotropic 3-D grid model (.md3grd: three
layers of three grid levels, a layer boundary where two levels coincide and
one on a flat grid level, grid points below the last level) on the first
grid through media_grid2model_el_iso (media/media_grid2model.cpp:133-189)
with each method; keys md3grd, ext and rho_<m>, lam_<m>, mu_<m>.

And grid_el_vti.npz: elastic VTI grid models of the three parametrisations
(the same levels) through media_grid2model_el_vti with "loc"; keys
<type>_md3grd and <type>_<c11|c33|c55|c66|c13|rho>.

This script needs the reference build and runs only where it exists; the
fixtures it writes are committed and are all the tests need elsewhere.

    python tests/golden/media/make_media_golden.py
"""

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
PROBE = os.path.join(REPO, "oracle", "_ref", "ref_probe")


def grid(ni=22, nj=18, nk=16, dh=100.0):
    """Padded (nz, ny, nx) grid: flat levels every dh below z = -600 m, a
    gentle hill above, x/y skewed slightly with height."""
    nx, ny, nz = ni + 6, nj + 6, nk + 6
    i = np.arange(nx) - 3.0
    j = np.arange(ny) - 3.0
    k = np.arange(nz) - 3.0
    K, J, I = np.meshgrid(k, j, i, indexing="ij")
    X = I * dh + 3.0 * np.sin(0.3 * K)
    Y = J * dh - 2.0 * np.cos(0.2 * K)
    top = 150.0 * np.exp(-((I - ni / 2) ** 2 + (J - nj / 2) ** 2) / 40.0)
    z0 = -(nk - 1) * dh
    Z = z0 + K * dh
    upper = K >= nk - 6                       # the top levels follow the hill
    frac = np.clip((K - (nk - 7)) / 6.0, 0, 1)
    Z = np.where(upper, Z + frac * top, Z)
    return X.astype(np.float32), Y.astype(np.float32), Z.astype(np.float32)


def layers(X, Y, seed=5):
    """Four interfaces on a 12 x 10 mesh covering the grid; properties
    (rho, vp, vs) with gradients and power laws per layer."""
    rng = np.random.default_rng(seed)
    NX, NY = 12, 10
    minx, miny = float(X.min()) - 50.0, float(Y.min()) - 50.0
    dx = (float(X.max()) + 50.0 - minx) / (NX - 1)
    dy = (float(Y.max()) + 50.0 - miny) / (NY - 1)
    xs = minx + dx * np.arange(NX)
    ys = miny + dy * np.arange(NY)
    XX, YY = np.meshgrid(xs, ys)
    elev = np.stack([
        60.0 + 20.0 * np.sin(XX / 700.0) * np.cos(YY / 500.0),   # below the hill top
        -400.0 + 80.0 * np.sin(XX / 900.0 + 0.5),
        np.full_like(XX, -800.0),                               # a grid level
        -1200.0 + 60.0 * np.cos(YY / 600.0),
    ])
    base = [(2300, 3800, 2100), (2450, 4500, 2550), (2600, 5200, 2950), (2750, 6000, 3450)]
    recs = []
    for n, (rho, vp, vs) in enumerate(base):
        pert = lambda a, s: a * (1.0 + s * rng.uniform(-1, 1, XX.shape))
        recs.append(np.stack([elev[n], pert(rho, 0.02), np.full_like(XX, 0.05 * (n + 1)),
                              np.full_like(XX, 1.0 if n % 2 == 0 else 0.5),
                              pert(vp, 0.03), np.full_like(XX, 0.3 + 0.1 * n),
                              np.full_like(XX, 1.0),
                              pert(vs, 0.03), np.full_like(XX, 0.2),
                              np.full_like(XX, 1.0 if n < 2 else 0.8)], -1))
    return dict(NX=NX, NY=NY, MINX=minx, MINY=miny, DX=dx, DY=dy,
                rec=np.stack(recs).astype(np.float32))


VTI_TYPES = {
    # per property: base value per layer (4 layers), gradient, power
    "elastic_vti_prem": [((2300, 2450, 2600, 2750), 0.05, 1.0),     # rho
                         ((4000, 4600, 5300, 6100), 0.3, 1.0),      # vph
                         ((3800, 4450, 5200, 6000), 0.2, 0.8),      # vpv
                         ((2200, 2600, 3000, 3500), 0.0, 1.0),      # vsh
                         ((2100, 2550, 2950, 3450), 0.1, 1.0),      # vsv
                         ((0.95, 0.92, 0.97, 1.0), 0.0, 1.0)],      # eta
    "elastic_vti_thomsen": [((2300, 2450, 2600, 2750), 0.05, 1.0),  # rho
                            ((3800, 4500, 5200, 6000), 0.3, 1.0),   # vp0
                            ((2100, 2550, 2950, 3450), 0.2, 0.9),   # vs0
                            ((0.15, 0.10, 0.08, 0.05), 0.0, 1.0),   # epsilon
                            ((0.08, 0.05, 0.04, 0.02), 1e-5, 1.0),  # delta
                            ((0.10, 0.07, 0.05, 0.03), 0.0, 1.0)],  # gamma
    "elastic_vti_cij": [((2300, 2450, 2600, 2750), 0.05, 1.0),      # rho
                        ((3.9e10, 5.2e10, 7.3e10, 1.0e11), 2e6, 1.0),   # c11
                        ((3.3e10, 4.8e10, 7.0e10, 9.9e10), 1e6, 0.7),   # c33
                        ((1.0e10, 1.6e10, 2.3e10, 3.3e10), 0.0, 1.0),   # c55
                        ((1.2e10, 1.8e10, 2.5e10, 3.5e10), 5e5, 1.0),   # c66
                        ((1.2e10, 1.6e10, 2.4e10, 3.2e10), 0.0, 1.0)],  # c13
}

VTI_CASES = [("elastic_vti_prem", "loc"), ("elastic_vti_prem", "ari"),
             ("elastic_vti_thomsen", "loc"), ("elastic_vti_thomsen", "har"),
             ("elastic_vti_thomsen", "ari"),
             ("elastic_vti_cij", "loc"), ("elastic_vti_cij", "har")]


def vti_layers(X, Y, kind, seed=7):
    """Four interfaces (as layers()) with the six properties of a VTI
    parametrisation: elevation, then (value, gradient, power) each."""
    rng = np.random.default_rng(seed)
    base = layers(X, Y)
    XX_shape = base["rec"].shape[1:3]
    recs = []
    for n in range(4):
        cols = [base["rec"][n, :, :, 0]]
        for vals, grad, pw in VTI_TYPES[kind]:
            cols += [vals[n] * (1.0 + 0.02 * rng.uniform(-1, 1, XX_shape)),
                     np.full(XX_shape, grad), np.full(XX_shape, pw if n % 2 == 0 else 1.0)]
        recs.append(np.stack(cols, -1))
    out = dict(base)
    out["rec"] = np.stack(recs).astype(np.float32)
    return out


def write_md3lay(path, L, kind="elastic_isotropic"):
    rec = L["rec"]
    with open(path, "w") as f:
        f.write("# layered %s model\n" % kind.replace("_", " "))
        f.write("%s\n%d\n" % (kind, rec.shape[0]))
        f.write("%d %d %.9g %.9g %.9g %.9g\n" % (L["NX"], L["NY"], L["MINX"], L["MINY"],
                                                 L["DX"], L["DY"]))
        for n in range(rec.shape[0]):
            for j in range(L["NY"]):
                for i in range(L["NX"]):
                    f.write(" ".join("%.9g" % v for v in rec[n, j, i]) + "\n")


def main():
    X, Y, Z = grid()
    L = layers(X, Y)
    nz, ny, nx = X.shape
    with tempfile.TemporaryDirectory() as tmp:
        lay = os.path.join(tmp, "model.md3lay")
        write_md3lay(lay, L)
        # the values as the reference parses them (%f of the text)
        gpath, opath = os.path.join(tmp, "grid.bin"), os.path.join(tmp, "out.bin")
        with open(gpath, "wb") as f:
            f.write(struct.pack("<3i", nx, ny, nz))
            for A in (X, Y, Z):
                f.write(A.astype("<f4").tobytes())
        res = {}
        for meth in ("loc", "har", "ari"):
            subprocess.run([PROBE, "layer", lay, gpath, meth, opath], check=True,
                           stdout=subprocess.DEVNULL)
            o = np.fromfile(opath, "<f4").reshape(3, nz, ny, nx)
            sfx = "" if meth == "loc" else "_" + meth
            res.update({"lam" + sfx: o[0], "mu" + sfx: o[1], "rho" + sfx: o[2]})
        out = (res["lam"], res["mu"], res["rho"])
        md3lay = open(lay).read()
    np.savez_compressed(os.path.join(HERE, "layer_el_iso.npz"), x3d=X, y3d=Y, z3d=Z,
                        md3lay=np.frombuffer(md3lay.encode(), np.uint8), **res)
    print("points changed from loc: har %d, ari %d"
          % ((res["lam_har"] != res["lam"]).sum(), (res["lam_ari"] != res["lam"]).sum()))
    vti_main()
    one_main(X, Y, Z)
    bin_main(X, Y, Z)
    grid_main(X, Y, Z)
    grid_vti_main(X, Y, Z)
    on = int(np.isclose(Z, -800.0).sum())
    print("grid %s, %d points on the flat interface, rho range %.1f-%.1f"
          % (X.shape, on, out[2].min(), out[2].max()))


def one_main(X, Y, Z):
    rng = np.random.default_rng(11)
    base = layers(X, Y)
    shp = base["rec"].shape[1:3]
    recs = []
    for n, (q, g, pw) in enumerate([(60.0, 0.02, 1.0), (90.0, 0.05, 0.8), (140.0, 0.0, 1.0),
                                    (220.0, 0.01, 1.2)]):
        recs.append(np.stack([base["rec"][n, :, :, 0],
                              q * (1.0 + 0.05 * rng.uniform(-1, 1, shp)),
                              np.full(shp, g), np.full(shp, pw)], -1))
    L = dict(base)
    L["rec"] = np.stack(recs).astype(np.float32)
    nz, ny, nx = X.shape
    res = {}
    with tempfile.TemporaryDirectory() as tmp:
        lay = os.path.join(tmp, "qs.md3lay")
        write_md3lay(lay, L, "one_component")
        res["md3lay"] = np.frombuffer(open(lay).read().encode(), np.uint8)
        gpath, opath = os.path.join(tmp, "grid.bin"), os.path.join(tmp, "out.bin")
        with open(gpath, "wb") as f:
            f.write(struct.pack("<3i", nx, ny, nz))
            for A in (X, Y, Z):
                f.write(A.astype("<f4").tobytes())
        for meth in ("loc", "har", "ari"):
            subprocess.run([PROBE, "layer_one", lay, gpath, meth, opath], check=True,
                           stdout=subprocess.DEVNULL)
            res["var_" + meth] = np.fromfile(opath, "<f4").reshape(nz, ny, nx)
    np.savez_compressed(os.path.join(HERE, "layer_onecmp.npz"), **res)
    print("onecmp: har changed %d points" % (res["var_har"] != res["var_loc"]).sum())


def bin_main(X, Y, Z):
    rng = np.random.default_rng(17)
    order = np.array([2, 0, 1], np.int32)              # file dims: z, x, y
    dx, dy, dz = 110.0, 130.0, -85.0
    x0, y0, z0 = float(X.min()) - 250.0, float(Y.min()) - 200.0, 400.0
    nxb = int((float(X.max()) + 300.0 - x0) / dx) + 1
    nyb = int((float(Y.max()) + 250.0 - y0) / dy) + 1
    nzb = 20                                            # to z = -1215: the grid goes deeper
    size = np.array([nzb, nxb, nyb], np.int32)
    spacing = np.array([dz, dx, dy], np.float32)
    origin = np.array([z0, x0, y0], np.float32)
    zz = z0 + dz * np.arange(nzb)
    xx = x0 + dx * np.arange(nxb)
    yy = y0 + dy * np.arange(nyb)
    Yg, Xg, Zg = np.meshgrid(yy, xx, zz, indexing="ij")    # [y][x][z]: z fastest
    depth = np.clip(-Zg, 0, None)

    def field(base, grad, amp):
        return (base + grad * depth + amp * np.sin(Xg / 400.0 + 0.3 * Zg / 100.0)
                * np.cos(Yg / 500.0) + amp * 0.3 * rng.standard_normal(Xg.shape))

    vols = {"rho_vol": field(2200.0, 0.4, 40.0), "vp_vol": field(3600.0, 1.5, 150.0),
            "vs_vol": field(2000.0, 0.9, 80.0), "qp_vol": field(120.0, 0.08, 10.0),
            "qs_vol": field(60.0, 0.04, 5.0)}
    vols = {k: v.astype(np.float32) for k, v in vols.items()}
    ext = np.array([X.min(), X.max(), Y.min(), Y.max()], np.float32)
    nz, ny, nx = X.shape
    res = dict(order=order, size=size, spacing=spacing, origin=origin, ext=ext, **vols)
    with tempfile.TemporaryDirectory() as tmp:
        gpath = os.path.join(tmp, "grid.bin")
        with open(gpath, "wb") as f:
            f.write(struct.pack("<3i", nx, ny, nz))
            for A in (X, Y, Z):
                f.write(A.astype("<f4").tobytes())
        ppath = os.path.join(tmp, "params.bin")
        with open(ppath, "wb") as f:
            for a in (order, size, spacing, origin, ext):
                f.write(a.tobytes())
        files = {}
        for k, v in vols.items():
            files[k] = os.path.join(tmp, k + ".bin")
            v.tofile(files[k])
        opath = os.path.join(tmp, "out.bin")
        subprocess.run([PROBE, "bin", gpath, ppath, files["rho_vol"], files["vp_vol"],
                        files["vs_vol"], opath], check=True, stdout=subprocess.DEVNULL)
        o = np.fromfile(opath, "<f4").reshape(3, nz, ny, nx)
        res.update(rho=o[0], lam=o[1], mu=o[2])
        subprocess.run([PROBE, "bin_vis", gpath, ppath, files["qp_vol"], files["qs_vol"],
                        opath], check=True, stdout=subprocess.DEVNULL)
        o = np.fromfile(opath, "<f4").reshape(2, nz, ny, nx)
        res.update(Qp=o[0], Qs=o[1])
    np.savez_compressed(os.path.join(HERE, "bin_model.npz"), **res)
    print("bin: model %s (z, x, y), rho %.1f-%.1f" % (tuple(size), res["rho"].min(),
                                                     res["rho"].max()))


def grid_main(X, Y, Z):
    rng = np.random.default_rng(23)
    ext = np.array([X.min(), X.max(), Y.min(), Y.max()], np.float32)
    NX, NY = 12, 10
    # the mesh covers the grid exactly as the reader crops it: (xmin - MINX)
    # below one DX and ceil((xmax - MINX) / DX) = NX - 1
    dx = float(ext[1] - ext[0]) / (NX - 1.8)
    dy = float(ext[3] - ext[2]) / (NY - 1.8)
    minx, miny = float(ext[0]) - 0.3 * dx, float(ext[2]) - 0.3 * dy
    XX, YY = np.meshgrid(minx + dx * np.arange(NX), miny + dy * np.arange(NY))
    l2 = -390.0 + 80.0 * np.sin(XX / 900.0 + 0.5)
    levels = [60.0 + 20.0 * np.sin(XX / 700.0) * np.cos(YY / 500.0),
              -150.0 + 30.0 * np.sin(XX / 900.0), l2,
              l2, -600.0 + 20.0 * np.cos(YY / 600.0), np.full_like(XX, -800.0),
              np.full_like(XX, -800.0), -1100.0 + 60.0 * np.cos(YY / 600.0),
              np.full_like(XX, -1400.0)]
    props = [((2300, 2400), (3800, 4200), (2100, 2300)),
             ((2450, 2600), (4500, 5000), (2550, 2800)),
             ((2650, 2800), (5200, 6000), (2950, 3450))]
    lines = ["elastic_isotropic", "3", "3 3 3",          # (no comments: the reader takes none)
             "%d %d %.9g %.9g %.9g %.9g" % (NX, NY, minx, miny, dx, dy)]
    for ni, e in enumerate(levels):
        layer, t = ni // 3, (ni % 3) / 2.0
        vals = [lo + (hi - lo) * t for lo, hi in props[layer]]
        pert = [v * (1.0 + 0.02 * rng.uniform(-1, 1, XX.shape)) for v in vals]
        for j in range(NY):
            for i in range(NX):
                lines.append("%.9g %.9g %.9g %.9g" % (np.float32(e[j, i]), pert[0][j, i],
                                                       pert[1][j, i], pert[2][j, i]))
    text = "\n".join(lines) + "\n"
    nz, ny, nx = X.shape
    res = dict(md3grd=np.frombuffer(text.encode(), np.uint8), ext=ext)
    with tempfile.TemporaryDirectory() as tmp:
        grd = os.path.join(tmp, "model.md3grd")
        open(grd, "w").write(text)
        gpath, epath = os.path.join(tmp, "grid.bin"), os.path.join(tmp, "ext.bin")
        opath = os.path.join(tmp, "out.bin")
        with open(gpath, "wb") as f:
            f.write(struct.pack("<3i", nx, ny, nz))
            for A in (X, Y, Z):
                f.write(A.astype("<f4").tobytes())
        ext.tofile(epath)
        for meth in ("loc", "har", "ari"):
            subprocess.run([PROBE, "grid", grd, gpath, meth, epath, opath], check=True,
                           stdout=subprocess.DEVNULL)
            o = np.fromfile(opath, "<f4").reshape(3, nz, ny, nx)
            res.update({"rho_" + meth: o[0], "lam_" + meth: o[1], "mu_" + meth: o[2]})
    np.savez_compressed(os.path.join(HERE, "grid_el_iso.npz"), **res)
    print("grid: har changed %d points, rho %.1f-%.1f"
          % ((res["lam_har"] != res["lam_loc"]).sum(), res["rho_loc"].min(),
             res["rho_loc"].max()))


GRID_VTI = {
    # per layer (top value, bottom value) of the six parameters
    "elastic_vti_prem": [((2300, 2400), (4000, 4400), (3800, 4200), (2200, 2400), (2100, 2300),
                          (0.95, 0.93))] * 3,
    "elastic_vti_thomsen": [((2300, 2450), (3800, 4300), (2100, 2400), (0.15, 0.12),
                             (0.08, 0.06), (0.10, 0.08))] * 3,
    "elastic_vti_cij": [((2300, 2450), (3.9e10, 4.6e10), (3.3e10, 4.0e10), (1.0e10, 1.3e10),
                         (1.2e10, 1.5e10), (1.2e10, 1.4e10))] * 3,
}


def grid_vti_main(X, Y, Z):
    rng = np.random.default_rng(29)
    ext = np.array([X.min(), X.max(), Y.min(), Y.max()], np.float32)
    NX, NY = 12, 10
    dx = float(ext[1] - ext[0]) / (NX - 1.8)
    dy = float(ext[3] - ext[2]) / (NY - 1.8)
    minx, miny = float(ext[0]) - 0.3 * dx, float(ext[2]) - 0.3 * dy
    XX, YY = np.meshgrid(minx + dx * np.arange(NX), miny + dy * np.arange(NY))
    l2 = -390.0 + 80.0 * np.sin(XX / 900.0 + 0.5)
    levels = [60.0 + 20.0 * np.sin(XX / 700.0) * np.cos(YY / 500.0),
              -150.0 + 30.0 * np.sin(XX / 900.0), l2,
              l2, -600.0 + 20.0 * np.cos(YY / 600.0), np.full_like(XX, -800.0),
              np.full_like(XX, -800.0), -1100.0 + 60.0 * np.cos(YY / 600.0),
              np.full_like(XX, -1400.0)]
    nz, ny, nx = X.shape
    res = dict(ext=ext)
    with tempfile.TemporaryDirectory() as tmp:
        gpath, epath = os.path.join(tmp, "grid.bin"), os.path.join(tmp, "ext.bin")
        opath = os.path.join(tmp, "out.bin")
        with open(gpath, "wb") as f:
            f.write(struct.pack("<3i", nx, ny, nz))
            for A in (X, Y, Z):
                f.write(A.astype("<f4").tobytes())
        ext.tofile(epath)
        for kind, props in GRID_VTI.items():
            lines = [kind, "3", "3 3 3", "%d %d %.9g %.9g %.9g %.9g" % (NX, NY, minx, miny, dx, dy)]
            for ni, e in enumerate(levels):
                layer, t = ni // 3, (ni % 3) / 2.0
                scale = 1.0 + 0.08 * layer
                vals = [(lo + (hi - lo) * t) * (scale if c < 5 or kind != "elastic_vti_thomsen"
                                               else 1.0) for c, (lo, hi) in enumerate(props[layer])]
                pert = [v * (1.0 + 0.02 * rng.uniform(-1, 1, XX.shape)) for v in vals]
                for j in range(NY):
                    for i in range(NX):
                        lines.append(" ".join(["%.9g" % np.float32(e[j, i])] +
                                              ["%.9g" % p_[j, i] for p_ in pert]))
            text = "\n".join(lines) + "\n"
            res[kind + "_md3grd"] = np.frombuffer(text.encode(), np.uint8)
            grd = os.path.join(tmp, kind + ".md3grd")
            open(grd, "w").write(text)
            subprocess.run([PROBE, "grid_vti", grd, gpath, "loc", epath, opath], check=True,
                           stdout=subprocess.DEVNULL)
            o = np.fromfile(opath, "<f4").reshape(6, nz, ny, nx)
            for c, name in enumerate(("c11", "c33", "c55", "c66", "c13", "rho")):
                res[kind + "_" + name] = o[c]
    np.savez_compressed(os.path.join(HERE, "grid_el_vti.npz"), **res)
    print("grid vti: %d types" % len(GRID_VTI))


def vti_main():
    X, Y, Z = grid(ni=16, nj=14, nk=16)
    nz, ny, nx = X.shape
    res = dict(x3d=X, y3d=Y, z3d=Z)
    with tempfile.TemporaryDirectory() as tmp:
        gpath, opath = os.path.join(tmp, "grid.bin"), os.path.join(tmp, "out.bin")
        with open(gpath, "wb") as f:
            f.write(struct.pack("<3i", nx, ny, nz))
            for A in (X, Y, Z):
                f.write(A.astype("<f4").tobytes())
        for kind in VTI_TYPES:
            lay = os.path.join(tmp, kind + ".md3lay")
            write_md3lay(lay, vti_layers(X, Y, kind), kind)
            res[kind + "_md3lay"] = np.frombuffer(open(lay).read().encode(), np.uint8)
        for kind, meth in VTI_CASES:
            lay = os.path.join(tmp, kind + ".md3lay")
            subprocess.run([PROBE, "layer_vti", lay, gpath, meth, opath], check=True,
                           stdout=subprocess.DEVNULL)
            o = np.fromfile(opath, "<f4").reshape(6, nz, ny, nx)
            for c, name in enumerate(("c11", "c33", "c55", "c66", "c13", "rho")):
                res["%s_%s_%s" % (kind, meth, name)] = o[c]
    np.savez_compressed(os.path.join(HERE, "layer_el_vti.npz"), **res)
    print("vti: grid %s, %d cases" % (X.shape, len(VTI_CASES)))


if __name__ == "__main__":
    main()
