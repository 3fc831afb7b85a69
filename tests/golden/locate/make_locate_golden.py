"""Generate tests/golden/locate/locate_topo.npz from the reference's point
location on a curvilinear grid.

Runs ``oracle/_ref/ref_probe locate`` (the reference's gd_curv_set_minmax,
gd_curv_depth_to_axis and gd_curv_coord_to_glob_indx, built by ``make -C
oracle``) on a seeded topography grid with skewed grid lines and on query
points of every kind the location meets: points inside cells, grid nodes,
points on shared cell faces and edges, points given by depth below the
surface, points outside the grid and inside the ghost layers.  Stores the
grid, the queries and the reference's answers.

This script needs the reference build and runs only where it exists; the
fixture it writes is committed and is all the tests need elsewhere.

    python tests/golden/locate/make_locate_golden.py
"""

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
PROBE = os.path.join(REPO, "oracle", "_ref", "ref_probe")


def grid(ni=24, nj=20, nk=16, dh=100.0, seed=3):
    """Padded (nz, ny, nx) coordinates: a Gaussian hill with roughness on
    top, vertical lines stretched to a flat bottom, x and y lines skewed with
    depth and height so that cells are not boxes."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = ni + 6, nj + 6, nk + 6
    i = np.arange(nx) - 3.0
    j = np.arange(ny) - 3.0
    k = np.arange(nz) - 3.0
    K, J, I = np.meshgrid(k, j, i, indexing="ij")
    xb, yb = I * dh, J * dh
    Lx, Ly = (ni - 1) * dh, (nj - 1) * dh
    rough = rng.normal(0.0, 20.0, (ny, nx))
    top = 600.0 * np.exp(-((xb[0] - Lx / 2) ** 2 + (yb[0] - Ly / 2) ** 2) / (700.0 ** 2)) + rough
    bottom = -(nk - 1) * dh
    u = K / (nk - 1)                                  # 0 bottom, 1 surface
    Z = bottom + u * (top[None] - bottom)
    X = xb + 25.0 * np.sin(0.9 * u * np.pi) + 8.0 * np.cos(0.7 * J)
    Y = yb + 18.0 * np.sin(1.3 * u * np.pi + 0.4) - 6.0 * np.sin(0.5 * I)
    return X.astype(np.float32), Y.astype(np.float32), Z.astype(np.float32)


def trilinear(A, fi, fj, fk):
    i0, j0, k0 = int(np.floor(fi)), int(np.floor(fj)), int(np.floor(fk))
    a, b, c = fi - i0, fj - j0, fk - k0
    v = 0.0
    for dk, wk in ((0, 1 - c), (1, c)):
        for dj, wj in ((0, 1 - b), (1, b)):
            for di, wi in ((0, 1 - a), (1, a)):
                v += wi * wj * wk * float(A[k0 + dk, j0 + dj, i0 + di])
    return v


def queries(X, Y, Z, seed=11):
    rng = np.random.default_rng(seed)
    nz, ny, nx = X.shape
    ni1, ni2, nj1, nj2, nk1, nk2 = 3, nx - 4, 3, ny - 4, 3, nz - 4
    q = []

    def at(fi, fj, fk, depth=None):
        x, y, z = (trilinear(A, fi, fj, fk) for A in (X, Y, Z))
        if depth is None:
            q.append((x, y, z, 0))
        else:
            q.append((x, y, depth, 1))

    for _ in range(28):                                  # inside cells
        at(rng.uniform(ni1, ni2), rng.uniform(nj1, nj2), rng.uniform(nk1, nk2))
    for _ in range(8):                                   # grid nodes
        at(rng.integers(ni1, ni2 + 1), rng.integers(nj1, nj2 + 1), rng.integers(nk1, nk2 + 1))
    for _ in range(4):                                   # surface nodes
        at(rng.integers(ni1, ni2 + 1), rng.integers(nj1, nj2 + 1), nk2)
    for _ in range(6):                                   # on shared faces / edges
        fi = rng.integers(ni1 + 1, ni2) + (0.5 if rng.random() < 0.5 else 0.0)
        at(fi, rng.integers(nj1 + 1, nj2) + 0.5, rng.integers(nk1 + 1, nk2))
    for _ in range(4):                                   # close under the surface
        at(rng.uniform(ni1, ni2), rng.uniform(nj1, nj2), nk2 - rng.uniform(0, 0.3))
    for d in (0.0, 0.0, 40.0, 250.0, 900.0, 1300.0):     # by depth below the surface
        at(rng.uniform(ni1, ni2), rng.uniform(nj1, nj2), nk2, depth=d)
    at(ni1 + 4, nj1 + 5, nk2, depth=0.0)                 # depth at a surface node
    for fi, fj, fk in ((1.5, 8.0, 8.0), (10.0, 1.2, 9.0), (9.0, 9.0, 1.5)):
        at(fi, fj, fk)                                   # in the ghost layers
    xmax, zmax = float(X.max()), float(Z.max())
    q += [(xmax + 50.0, float(Y.mean()), float(Z.mean()), 0),
          (float(X.mean()), float(Y.mean()), zmax + 100.0, 0),
          (float(X.min()) - 1.0, float(Y.min()) - 1.0, 0.0, 1)]
    return np.array([v[:3] for v in q], np.float32), np.array([v[3] for v in q], np.int32)


def run_probe(X, Y, Z, pts, is_depth):
    nz, ny, nx = X.shape
    with tempfile.TemporaryDirectory() as tmp:
        inp, out = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
        with open(inp, "wb") as fh:
            fh.write(struct.pack("<4i", nx, ny, nz, len(pts)))
            for A in (X, Y, Z):
                fh.write(A.astype("<f4").tobytes())
            for p, d in zip(pts, is_depth):
                fh.write(struct.pack("<3fi", *[float(v) for v in p], int(d)))
        subprocess.run([PROBE, "locate", inp, out], check=True)
        raw = np.fromfile(out, dtype=np.uint8).reshape(len(pts), 32)
    ints = raw[:, :16].copy().view("<i4")
    flts = raw[:, 16:].copy().view("<f4")
    return ints, flts


def main():
    X, Y, Z = grid()
    pts, is_depth = queries(X, Y, Z)
    ints, flts = run_probe(X, Y, Z, pts, is_depth)
    np.savez_compressed(os.path.join(HERE, "locate_topo.npz"), x3d=X, y3d=Y, z3d=Z,
                        points=pts, is_depth=is_depth, found=ints[:, 0],
                        index=ints[:, 1:4], shift=flts[:, :3], z_axis=flts[:, 3])
    print("%d points, %d located" % (len(pts), int(ints[:, 0].sum())))


if __name__ == "__main__":
    main()
