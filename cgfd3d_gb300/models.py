"""Synthetic models of the benchmark configurations, built on the host.

The reference builds its inputs with its own setup code (grid, metrics,
media, PML coefficients, source tables, receivers) before it calls the time
loop.  This module restates the parts of that setup the benchmark workloads
need, vectorised with numpy:

  metrics           forward/gd_t.c:190-402 (centred 7-point operator of
                    forward/fd_t.c:152-176, cross products, mirrored ghosts)
  PML coefficients  forward/bdry_t.c:115-366 and :371-506
  source tables     forward/src_t.c:984-1174 (wavelet by name, Ricker
                    src_t.c:2158-2166), grid-index location src_t.c:768-775
  receivers         forward/io_funcs.c:233-414 (grid-index stations, floor)

Configurations (seeded, synthetic -- the reference publishes no dataset):

  "flat"  100x100x60, dh 100 m, flat free surface, Vp/Vs/rho 6000/3464/2700,
          CFS-PML 10 layers on 5 faces, explosive source at the centre 2 km
          deep, Ricker 2 Hz, 20 surface receivers, dt 0.005 s, 500 steps
  "topo"  400x400x200, surface 2000 exp(-r^2/(5 km)^2) + seeded Gaussian-
          correlated roughness (std 100 m, correlation 1 km), body-fitted
          grid at 100 m nominal spacing, three layers 4000/2310/2400,
          5500/3175/2650, 6500/3750/2900 with interfaces at 3 and 10 km
          depth, CFS-PML 12 layers, double couple from the seed, Ricker
          1.5 Hz, 400 surface receivers, 2000 steps
"""

import math

import numpy as np

from . import abi
from .problem import NLEVEL, Problem

CENTER7 = np.array([-0.02084, 0.1667, -0.7709, 0.0, 0.7709, -0.1667, 0.02084],
                   np.float64)


# ---------------------------------------------------------------------------
# grid and metrics
# ---------------------------------------------------------------------------

def grid_coords(ni, nj, nk, dh, surface=None, z_bottom=None):
    """Body-fitted grid (padded, shape (nz, ny, nx)), k upward.

    x, y uniform with spacing dh; each vertical grid line runs linearly from
    z_bottom to surface(x, y).  Ghost nodes continue the node spacing
    (above the surface: mirrored extrapolation, forward/gd_t.c:1448-1454).
    """
    nx, ny, nz = ni + 6, nj + 6, nk + 6
    x1 = (np.arange(nx) - 3) * dh
    y1 = (np.arange(ny) - 3) * dh
    X, Y = np.meshgrid(x1, y1, indexing="xy")           # (ny, nx)
    if surface is None:
        ztop = np.zeros_like(X)
    else:
        ztop = surface(X, Y)
    if z_bottom is None:
        z_bottom = -(nk - 1) * dh
    s = (np.arange(nz) - 3) / float(nk - 1)              # 0 at nk1, 1 at nk2
    Z = z_bottom + (ztop[None, :, :] - z_bottom) * s[:, None, None]
    Xg = np.broadcast_to(X[None], (nz, ny, nx))
    Yg = np.broadcast_to(Y[None], (nz, ny, nx))
    return Xg, Yg, Z


def _dcentre(a, axis):
    """Centred 7-point derivative in index space on the physical region."""
    out = np.zeros(a.shape, np.float64)
    sl = [slice(3, -3)] * 3
    for n, c in enumerate(CENTER7):
        if c == 0.0:
            continue
        src = list(sl)
        src[axis] = slice(n, a.shape[axis] - 6 + n)
        out[tuple(sl)] += c * a[tuple(src)]
    return out


def _mirror_ghosts(m):
    """Ghost values mirrored about the boundary (forward/gd_t.c:291-401)."""
    nz, ny, nx = m.shape
    for g in range(3):                       # x
        m[:, :, g] = m[:, :, 5 - g]
        m[:, :, nx - 1 - g] = m[:, :, nx - 6 + g]
    for g in range(3):                       # y
        m[:, g, :] = m[:, 5 - g, :]
        m[:, ny - 1 - g, :] = m[:, ny - 6 + g, :]
    for g in range(3):                       # z
        m[g, :, :] = m[5 - g, :, :]
        m[nz - 1 - g, :, :] = m[nz - 6 + g, :, :]
    return m


def metrics(X, Y, Z):
    """jac, xi_x..zeta_z (float32, flattened) from node coordinates."""
    d = {}
    xs = [np.asarray(X, np.float64), np.asarray(Y, np.float64),
          np.asarray(Z, np.float64)]
    # axis order of the arrays is (z, y, x): xi -> axis 2, eta -> 1, zeta -> 0
    v1 = [_dcentre(c, 2) for c in xs]      # x_xi, y_xi, z_xi
    v2 = [_dcentre(c, 1) for c in xs]      # x_et, ...
    v3 = [_dcentre(c, 0) for c in xs]      # x_zt, ...

    def cross(a, b):
        return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                a[0] * b[1] - a[1] * b[0]]

    g12 = cross(v1, v2)
    jac = g12[0] * v3[0] + g12[1] * v3[1] + g12[2] * v3[2]
    core = (slice(3, -3),) * 3
    safe = np.ones_like(jac)
    safe[core] = jac[core]
    g23 = cross(v2, v3)
    g31 = cross(v3, v1)
    out = {"jac": jac}
    for name, g in (("xi", g23), ("eta", g31), ("zeta", g12)):
        for c, ax in enumerate("xyz"):
            out["%s_%s" % (name, ax)] = g[c] / safe
    for k in out:
        a = out[k].astype(np.float32)
        d[k] = np.ascontiguousarray(_mirror_ghosts(a)).ravel()
    return d


# ---------------------------------------------------------------------------
# PML
# ---------------------------------------------------------------------------

def pml_face_box(p, d, s, nlay):
    box = [p.ni1, p.ni2, p.nj1, p.nj2, p.nk1, p.nk2]
    lo, hi = 2 * d, 2 * d + 1
    if s == 0:
        box[hi] = box[lo] + nlay
    else:
        box[lo] = box[hi] - nlay
    return np.array(box, np.int32)


def pml_coefs(nlay, L0, dh, vref, alpha_max, beta_max, side):
    """A, B, D of one face (forward/bdry_t.c:237-268, 333-366)."""
    npts = nlay + 1
    R = math.pow(10.0, -((math.log10(float(nlay)) - 1.0) / math.log10(2.0) + 4.0))
    R = float(np.float32(R))
    dmax = float(np.float32(-vref / (2.0 * L0) * math.log(R) * 3.0))
    A = np.zeros(npts, np.float32)
    B = np.zeros(npts, np.float32)
    D = np.zeros(npts, np.float32)
    for n in range(npts):
        L = float(np.float32(n * dh))
        i = npts - 1 - n if side == 0 else n
        dd = np.float32(dmax * (L / L0) ** 2)
        aa = np.float32(alpha_max * (1.0 - (L / L0)))
        bb = np.float32(1.0 + (beta_max - 1.0) * (L / L0) ** 2)
        dd = np.float32(dd / bb)
        A[i] = np.float32(aa + dd)
        D[i] = dd
        B[i] = np.float32(1.0 / bb)
    return A, B, D


def add_pml(p, X, Y, Z, nlay, faces, vref, alpha_max, beta_max=2.0):
    """Enable CFS-PML on `faces` (list of (dim, side)), coefficients from the
    mean grid spacing along the face normal (forward/bdry_t.c:371-506)."""
    xs = [np.asarray(X), np.asarray(Y), np.asarray(Z)]
    for d, s in faces:
        box = pml_face_box(p, d, s, nlay)
        sl = (slice(box[4], box[5] + 1), slice(box[2], box[3] + 1),
              slice(box[0], box[1] + 1))
        ax = 2 - d
        seg = [np.diff(c[sl].astype(np.float64), axis=ax) for c in xs]
        dh = float(np.float32(np.sqrt(seg[0] ** 2 + seg[1] ** 2 + seg[2] ** 2).mean()))
        L0 = float(np.float32(dh * nlay))
        A, B, D = pml_coefs(nlay, L0, dh, vref, alpha_max, beta_max, s)
        avol = int((box[1] - box[0] + 1) * (box[3] - box[2] + 1) * (box[5] - box[4] + 1))
        p.pml[d][s] = dict(box=box, A=A, B=B, D=D,
                           aux=np.zeros(NLEVEL * 9 * avol, np.float32))


# ---------------------------------------------------------------------------
# media
# ---------------------------------------------------------------------------

def set_iso_media(p, vp, vs, rho):
    vp, vs, rho = [np.broadcast_to(np.asarray(a, np.float32), (p.nz, p.ny, p.nx))
                   for a in (vp, vs, rho)]
    mu = (vs * vs * rho).astype(np.float32)
    lam = (vp * vp * rho - 2.0 * mu).astype(np.float32)
    p.medium_type = abi.CGFD_MEDIUM_ELASTIC_ISO
    p.media = {"slw": np.ascontiguousarray((1.0 / rho).astype(np.float32)).ravel(),
               "lambda": np.ascontiguousarray(lam).ravel(),
               "mu": np.ascontiguousarray(mu).ravel()}


def layered(Z, surface_z, layers):
    """Vp, Vs, rho by depth below the local surface.  layers: list of
    (depth_of_bottom_interface_m or None, vp, vs, rho) from top down."""
    depth = surface_z[None, :, :] - Z
    vp = np.empty(Z.shape, np.float32)
    vs = np.empty(Z.shape, np.float32)
    rho = np.empty(Z.shape, np.float32)
    prev = -np.inf
    for bot, a, b, c in layers:
        hi = np.inf if bot is None else bot
        m = (depth > prev) & (depth <= hi) if prev > -np.inf else depth <= hi
        vp[m], vs[m], rho[m] = a, b, c
        prev = hi
    return vp, vs, rho


# ---------------------------------------------------------------------------
# sources and receivers
# ---------------------------------------------------------------------------

def ricker(t, fc, t0):
    u = (t - t0) * 2.0 * math.pi * fc
    return (1.0 - u * u / 2.0) * np.exp(-u * u / 4.0)


def add_moment_source(p, i, j, k, M, fc, t0, stf_len=None, spatial="point"):
    """One moment-tensor source at padded index (i, j, k), Ricker wavelet.

    M = (Mxx, Myy, Mzz, Myz, Mxz, Mxy).  Table layout [is][it][istage]
    (forward/src_t.c:1050), sampled at t = it*dt + c_stage*dt."""
    dt = p.dt
    max_nt = p.nt_total if stf_len is None else int(stf_len / dt + 0.5)
    rk_t = np.array([0.0, 0.5, 0.5, 1.0], np.float32)
    it = np.arange(max_nt, dtype=np.float32)
    t = (it[:, None] * np.float32(dt) + rk_t[None, :] * np.float32(dt)).astype(np.float32)
    stf = ricker(t.astype(np.float64), fc, t0).astype(np.float32).ravel()
    tabs = {}
    for name, m in zip(("Mxx", "Myy", "Mzz", "Myz", "Mxz", "Mxy"), M):
        tabs[name] = (stf * np.float32(m)).astype(np.float32)
    gauss = spatial != "point"
    p.src = dict(n=1, max_nt=max_nt, max_stage=4, force=0, moment=1,
                 spatial=abi.CGFD_SRC_GAUSSIAN if gauss else abi.CGFD_SRC_POINT,
                 ext_half=3 if gauss else 0, ext_coef=1.5 if gauss else 0.0,
                 surface_strict=0, n_surface_force=0,
                 si=np.array([i], np.int32), sj=np.array([j], np.int32),
                 sk=np.array([k], np.int32),
                 si_inc=np.zeros(1, np.float32), sj_inc=np.zeros(1, np.float32),
                 sk_inc=np.zeros(1, np.float32),
                 it_begin=np.zeros(1, np.int32),
                 it_end=np.array([max_nt - 1], np.int32), **tabs)


def add_surface_receivers(p, ij_list):
    """Stations at the surface by grid index (flag_coord 0, depth 0)."""
    n = len(ij_list)
    dijk = np.zeros(3 * n, np.float32)
    idx = np.zeros(8 * n, np.int32)
    for r, (fi, fj) in enumerate(ij_list):
        i, j = int(math.floor(fi)), int(math.floor(fj))
        il, jl, kl = i + 3, j + 3, p.nk2
        di = 0.0 if il == p.ni2 else fi - i
        dj = 0.0 if jl == p.nj2 else fj - j
        dijk[3 * r:3 * r + 3] = (di, dj, 0.0)
        for c, (a, b, cc) in enumerate([(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0),
                                        (0, 0, 1), (1, 0, 1), (0, 1, 1), (1, 1, 1)]):
            idx[8 * r + c] = (il + a) + (jl + b) * p.nx + (kl + cc) * p.nx * p.ny
    p.recv = dict(n=n, max_nt=p.nt_total, ncmp=p.ncmp, dijk=dijk, indx1d=idx,
                  seismo=np.zeros(n * p.ncmp * p.nt_total, np.float32))


# ---------------------------------------------------------------------------
# configurations
# ---------------------------------------------------------------------------

def gaussian_roughness(nx, ny, dh, std, corr, seed):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((ny, nx))
    k1 = np.fft.fftfreq(nx, d=dh)
    k2 = np.fft.fftfreq(ny, d=dh)
    KX, KY = np.meshgrid(k1, k2, indexing="xy")
    filt = np.exp(-(np.pi * corr) ** 2 * (KX ** 2 + KY ** 2))
    r = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    r *= std / max(r.std(), 1e-30)
    return r


def dc_moment(strike, dip, rake, m0=1e16):
    """Double couple (Aki & Richards convention, x north, y east, z down),
    returned in the solver's frame (z up) as (Mxx, Myy, Mzz, Myz, Mxz, Mxy)."""
    s, d, r = np.radians([strike, dip, rake])
    mxx = -(np.sin(d) * np.cos(r) * np.sin(2 * s) + np.sin(2 * d) * np.sin(r) * np.sin(s) ** 2)
    mxy = np.sin(d) * np.cos(r) * np.cos(2 * s) + 0.5 * np.sin(2 * d) * np.sin(r) * np.sin(2 * s)
    mxz = -(np.cos(d) * np.cos(r) * np.cos(s) + np.cos(2 * d) * np.sin(r) * np.sin(s))
    myy = np.sin(d) * np.cos(r) * np.sin(2 * s) - np.sin(2 * d) * np.sin(r) * np.cos(s) ** 2
    myz = -(np.cos(d) * np.cos(r) * np.sin(s) - np.cos(2 * d) * np.sin(r) * np.cos(s))
    mzz = np.sin(2 * d) * np.sin(r)
    # z down -> z up flips the sign of the xz and yz components
    return tuple(m0 * v for v in (mxx, myy, mzz, -myz, -mxz, mxy))


def flat_model(ni=100, nj=100, nk=60, steps=500, dt=0.005, npml=10):
    """Flat free surface, homogeneous, explosive source (see module doc)."""
    dh = 100.0
    p = Problem(ni, nj, nk, dt, steps + 1)
    X, Y, Z = grid_coords(ni, nj, nk, dh)
    p.metric = metrics(X, Y, Z)
    set_iso_media(p, 6000.0, 3464.0, 2700.0)
    p.free_top = 1
    add_pml(p, X, Y, Z, npml, [(0, 0), (0, 1), (1, 0), (1, 1), (2, 0)],
            vref=6000.0, alpha_max=math.pi * 2.0)
    depth_cells = int(round(2000.0 / dh))
    add_moment_source(p, p.ni1 + ni // 2, p.nj1 + nj // 2, p.nk2 - depth_cells,
                      (1e16, 1e16, 1e16, 0.0, 0.0, 0.0), fc=2.0, t0=0.6)
    add_surface_receivers(p, [(10 + 4 * n, nj // 2) for n in range(20)])
    return p


def topo_model(ni=400, nj=400, nk=200, steps=2000, dt=None, npml=12, seed=2024,
               nrecv=400):
    """Curvilinear topography, three layers, double couple (module doc)."""
    dh = 100.0
    rng = np.random.default_rng(seed)
    Lx, Ly = (ni - 1) * dh, (nj - 1) * dh
    rough = gaussian_roughness(ni + 6, nj + 6, dh, 100.0, 1000.0, seed)

    def surface(X, Y):
        r2 = (X - Lx / 2) ** 2 + (Y - Ly / 2) ** 2
        return 2000.0 * np.exp(-r2 / 5000.0 ** 2) + rough

    z_bottom = -(nk - 1) * dh
    X, Y, Z = grid_coords(ni, nj, nk, dh, surface, z_bottom)
    ztop = Z[-4]
    vp, vs, rho = layered(Z, ztop, [(3000.0, 4000.0, 2310.0, 2400.0),
                                    (10000.0, 5500.0, 3175.0, 2650.0),
                                    (None, 6500.0, 3750.0, 2900.0)])
    if dt is None:
        # CFL-limited step of this grid, two significant digits
        hmin = float(np.diff(Z[3:-3, 3:-3, 3:-3], axis=0).min())
        dt = float("%.2g" % (1.3 * min(hmin, dh) / 6500.0 / math.sqrt(3) * 0.9))
    p = Problem(ni, nj, nk, dt, steps + 1)
    p.metric = metrics(X, Y, Z)
    set_iso_media(p, vp, vs, rho)
    p.free_top = 1
    add_pml(p, X, Y, Z, npml, [(0, 0), (0, 1), (1, 0), (1, 1), (2, 0)],
            vref=6500.0, alpha_max=math.pi * 1.5)
    strike, dip, rake = rng.uniform(0, 360), rng.uniform(10, 90), rng.uniform(-180, 180)
    depth = min(rng.uniform(4000.0, 8000.0), (nk - npml - 8) * dh)
    si, sj = p.ni1 + ni // 2 + int(rng.integers(-20, 20)), p.nj1 + nj // 2 + int(rng.integers(-20, 20))
    sk = p.nk2 - int(round(depth / dh))
    add_moment_source(p, si, sj, sk, dc_moment(strike, dip, rake), fc=1.5, t0=1.0)
    side = int(round(math.sqrt(nrecv)))
    coords = [(npml + 2 + (ni - 2 * npml - 4) * a / max(side - 1, 1),
               npml + 2 + (nj - 2 * npml - 4) * b / max(side - 1, 1))
              for a in range(side) for b in range(side)][:nrecv]
    add_surface_receivers(p, [(int(x), int(y)) for x, y in coords])
    return p
