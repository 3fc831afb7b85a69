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

This script needs the reference build and runs only where it exists; the
fixture it writes is committed and is all the tests need elsewhere.

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


def write_md3lay(path, L):
    rec = L["rec"]
    with open(path, "w") as f:
        f.write("# layered elastic isotropic model\n")
        f.write("elastic_isotropic\n%d\n" % rec.shape[0])
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
    on = int(np.isclose(Z, -800.0).sum())
    print("grid %s, %d points on the flat interface, rho range %.1f-%.1f"
          % (X.shape, on, out[2].min(), out[2].max()))


if __name__ == "__main__":
    main()
