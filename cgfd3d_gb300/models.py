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

def _abl_mask(i, vel, dt, nlay, dh):
    """bdry_ablexp_cal_mask (forward/bdry_t.c:822-839) in float arithmetic."""
    f32 = np.float32
    length = f32(nlay) * f32(dh)
    nstep = int(f32(f32(length / f32(vel)) / f32(dt)))
    total = f32(0.0)
    for n in range(nstep):
        x = f32(f32(f32(n) * f32(dt)) * f32(vel)) / length
        total = f32(total + x * x)
    alpha = f32(0.6 / float(total))
    r = f32(f32(i) / f32(nlay))
    return f32(np.exp(f32(-alpha * (r * r))))


def _abl_dh(X, Y, Z, box, axis):
    """Mean grid spacing along `axis` over a block (bdry_cal_abl_len_dh,
    forward/bdry_t.c:372-506): segment lengths in double, averaged."""
    i1, i2, j1, j2, k1, k2 = box
    sl = (slice(k1, k2 + 1), slice(j1, j2 + 1), slice(i1, i2 + 1))
    x, y, z = [np.asarray(A, np.float64)[sl] for A in (X, Y, Z)]
    ax = {0: 2, 1: 1, 2: 0}[axis]
    d = np.sqrt(np.diff(x, axis=ax) ** 2 + np.diff(y, axis=ax) ** 2 + np.diff(z, axis=ax) ** 2)
    return np.float32(d.sum() / d.size)


def add_ablexp(p, layers, vel=6000.0, coords=None, dh=None):
    """Exponential sponge on the faces in `layers` (x_left, x_right,
    y_front, y_back, z_bottom, z_top -> number of layers), as
    bdry_ablexp_set builds it (forward/bdry_t.c:513-820): six disjoint
    blocks (x layers over the whole j, k range; y layers between them;
    z layers inside both) and per-index masks, the outermost layer damped
    most.  The grid spacing per block is the mean along the face normal of
    the curvilinear grid `coords` = (X, Y, Z) (padded (nz, ny, nx)), or `dh`
    for a Cartesian grid.  vel: reference velocity (scalar or per face)."""
    names = ["x_left", "x_right", "y_front", "y_back", "z_bottom", "z_top"]
    nl = {n: int(layers.get(n, 0)) for n in names}
    v = {n: float(vel[n] if isinstance(vel, dict) else vel) for n in names}
    Ex, Ey, Ez = (np.ones(m, np.float32) for m in (p.nx, p.ny, p.nz))
    ix1, ix2 = p.ni1 + nl["x_left"], p.ni2 - nl["x_right"]
    jy1, jy2 = p.nj1 + nl["y_front"], p.nj2 - nl["y_back"]
    boxes = [(p.ni1, p.ni1 + nl["x_left"] - 1, p.nj1, p.nj2, p.nk1, p.nk2),
             (p.ni2 - nl["x_right"] + 1, p.ni2, p.nj1, p.nj2, p.nk1, p.nk2),
             (ix1, ix2, p.nj1, p.nj1 + nl["y_front"] - 1, p.nk1, p.nk2),
             (ix1, ix2, p.nj2 - nl["y_back"] + 1, p.nj2, p.nk1, p.nk2),
             (ix1, ix2, jy1, jy2, p.nk1, p.nk1 + nl["z_bottom"] - 1),
             (ix1, ix2, jy1, jy2, p.nk2 - nl["z_top"] + 1, p.nk2)]
    blk = np.zeros((6, 7), np.int32)
    for n, name in enumerate(names):
        b = boxes[n]
        blk[n, 1:] = b
        if b[1] < b[0] or b[3] < b[2] or b[5] < b[4] or nl[name] == 0:
            continue
        blk[n, 0] = 1
        axis = n // 2
        h = dh if coords is None else _abl_dh(*coords, b, axis)
        lo, hi = b[2 * axis], b[2 * axis + 1]
        cnt = hi - lo + 1
        E = (Ex, Ey, Ez)[axis]
        for a in range(lo, hi + 1):
            depth = cnt - (a - lo) if n % 2 == 0 else a - lo + 1
            E[a] = _abl_mask(depth, v[name], p.dt, cnt, h)
    p.ablexp = dict(Ex=Ex, Ey=Ey, Ez=Ez, blk=blk)
    return p


def add_dd_sources(p, ijk, vi=None, mij=None, max_nt=None):
    """Distributed (dd) sources at grid points: `ijk` (n, 3) local indices
    (ghosts included); vi (max_nt, 4, n, 3) force rates and/or mij
    (max_nt, 4, n, 6) moment rates (Mxx Myy Mzz Myz Mxz Mxy) per step and RK
    stage, as the reference's set-up leaves them in its dd files."""
    ijk = np.asarray(ijk, np.int32).reshape(-1, 3)
    tabs = [t for t in (vi, mij) if t is not None]
    if not tabs:
        raise ValueError("dd sources need vi or mij")
    nt = tabs[0].shape[0] if max_nt is None else int(max_nt)
    p.dd = dict(si=np.ascontiguousarray(ijk[:, 0]), sj=np.ascontiguousarray(ijk[:, 1]),
                sk=np.ascontiguousarray(ijk[:, 2]), max_nt=nt,
                vi=None if vi is None else np.ascontiguousarray(vi, np.float32).ravel(),
                mij=None if mij is None else np.ascontiguousarray(mij, np.float32).ravel())
    return p


def add_graves_qs(p, Qs, freq):
    """Graves Q attenuation of an elastic medium (visco_config graves_Qs):
    Qs per point (nx*ny*nz, or a scalar), reference frequency `freq`."""
    q = np.broadcast_to(np.asarray(Qs, np.float32), (p.vol,)).copy()
    p.graves_qs = dict(Qs=q, freq=float(freq))
    return p


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


# ---------------------------------------------------------------------------
# anisotropic and attenuating media on the topography (300 x 300 x 150)
# ---------------------------------------------------------------------------

def gaussian_field_3d(shape, dh, corr, seed):
    """Unit-variance Gaussian random field with Gaussian correlation of
    length `corr` (metres) on a grid of spacing dh, shape (nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape).astype(np.float32)
    ks = [np.fft.fftfreq(n, d=dh).astype(np.float32) for n in shape]
    filt = np.ones((1, 1, 1), np.float32)
    for ax, k in enumerate(ks):
        sh = [1, 1, 1]
        sh[ax] = k.size
        filt = filt * np.exp(-(np.pi * corr * k) ** 2 / 2.0).reshape(sh)
    f = np.fft.ifftn(np.fft.fftn(w) * filt).real.astype(np.float32)
    f -= f.mean()
    f /= max(float(f.std()), 1e-30)
    return f


def normal_cdf(x):
    from math import sqrt
    from scipy.special import erf
    return 0.5 * (1.0 + erf(np.asarray(x, np.float64) / sqrt(2.0)))


def thomsen_to_vti(vp, vs, rho, eps, delta, gamma):
    """Thomsen (1986) parameters -> c11, c13, c33, c55, c66 (the relations of
    the reference's converter, media/media_utility.hpp:424)."""
    vp, vs, rho = [np.asarray(a, np.float64) for a in (vp, vs, rho)]
    c33 = rho * vp * vp
    c55 = rho * vs * vs
    c11 = c33 * (1.0 + 2.0 * eps)
    c66 = c55 * (1.0 + 2.0 * gamma)
    c13 = np.sqrt(2.0 * delta * c33 * (c33 - c55) + (c33 - c55) ** 2) - c55
    return [np.ascontiguousarray(c.astype(np.float32)).ravel()
            for c in (c11, c13, c33, c55, c66)]


def bond_matrix(R):
    """6x6 Bond transformation of a stiffness in Voigt order (xx, yy, zz, yz,
    xz, xy) for the rotation R (..., 3, 3): C' = M C M^T (Auld)."""
    a = np.asarray(R, np.float64)
    M = np.empty(a.shape[:-2] + (6, 6))
    pairs = [(1, 2), (2, 0), (0, 1)]          # columns 4, 5, 6: yz, zx, xy
    for r in range(3):
        for c in range(3):
            M[..., r, c] = a[..., r, c] ** 2
        for n, (u, v) in enumerate(pairs):
            M[..., r, 3 + n] = 2.0 * a[..., r, u] * a[..., r, v]
    rows = [(1, 2), (2, 0), (0, 1)]           # rows 4, 5, 6
    for n, (u, v) in enumerate(rows):
        for c in range(3):
            M[..., 3 + n, c] = a[..., u, c] * a[..., v, c]
        for m, (s_, t) in enumerate(pairs):
            M[..., 3 + n, 3 + m] = a[..., u, s_] * a[..., v, t] + a[..., u, t] * a[..., v, s_]
    return M


def tti_stiffness(c11, c13, c33, c55, c66, tilt, azimuth):
    """The 21 constants of a tilted transversely isotropic medium: the VTI
    stiffness (c12 = c11 - 2 c66) with its symmetry axis rotated by `tilt`
    from the vertical towards azimuth `azimuth` (radians, per point or
    scalar).  Returns a dict c11..c66 of float32 arrays."""
    c11, c13, c33, c55, c66 = [np.asarray(v, np.float64) for v in (c11, c13, c33, c55, c66)]
    n = c11.size
    C = np.zeros((n, 6, 6))
    C[:, 0, 0] = C[:, 1, 1] = c11
    C[:, 2, 2] = c33
    C[:, 0, 1] = C[:, 1, 0] = c11 - 2.0 * c66
    C[:, 0, 2] = C[:, 2, 0] = C[:, 1, 2] = C[:, 2, 1] = c13
    C[:, 3, 3] = C[:, 4, 4] = c55
    C[:, 5, 5] = c66
    th = np.broadcast_to(np.asarray(tilt, np.float64), (n,))
    ph = np.broadcast_to(np.asarray(azimuth, np.float64), (n,))
    ct, st, cp, sp = np.cos(th), np.sin(th), np.cos(ph), np.sin(ph)
    R = np.zeros((n, 3, 3))                   # Rz(azimuth) @ Ry(tilt)
    R[:, 0, 0], R[:, 0, 1], R[:, 0, 2] = cp * ct, -sp, cp * st
    R[:, 1, 0], R[:, 1, 1], R[:, 1, 2] = sp * ct, cp, sp * st
    R[:, 2, 0], R[:, 2, 1], R[:, 2, 2] = -st, 0.0, ct
    M = bond_matrix(R)
    Cr = np.einsum("nij,njk,nlk->nil", M, C, M)
    out = {}
    for I in range(6):
        for J in range(I, 6):
            out["c%d%d" % (I + 1, J + 1)] = np.ascontiguousarray(Cr[:, I, J].astype(np.float32))
    return out


def gmb_coefficients(Qp, Qs, nmaxwell, fmin, fmax, fr):
    """GMB relaxation frequencies and weights for constant Qp, Qs, and the
    relaxed-to-unrelaxed modulus factors, restating the least-squares fit of
    forward/md_t.c:642-792 (2n-1 log-spaced frequencies between fmin and
    fmax, weights by the normal equations, moduli referred to fr).

    Returns wl (nmaxwell), YP, YS (nmaxwell), fac_p, fac_s with
    lam+2mu unrelaxed = (lam+2mu) fac_p and mu unrelaxed = mu fac_s."""
    kmax = 2 * nmaxwell - 1
    wr, wmin, wmax = 2 * math.pi * fr, 2 * math.pi * fmin, 2 * math.pi * fmax
    wk = wmin * (wmax / wmin) ** (np.arange(kmax) / float(kmax - 1))
    wl = wk[0::2][:nmaxwell]

    def fit(Q):
        q1 = 1.0 / round(Q)
        G = (wl[None, :] * wk[:, None] + wl[None, :] ** 2 * q1) / \
            (wl[None, :] ** 2 + wk[:, None] ** 2)
        Y = np.linalg.solve(G.T @ G, G.T @ np.full(kmax, q1))
        th1 = 1.0 - np.sum(Y / (1.0 + (wr / wl) ** 2))
        th2 = np.sum(Y * wr / wl / (1.0 + (wr / wl) ** 2))
        R = math.sqrt(th1 ** 2 + th2 ** 2)
        return Y, (R + th1) / (2.0 * R * R)

    YP, fac_p = fit(Qp)
    YS, fac_s = fit(Qs)
    return wl.astype(np.float32), YP, YS, fac_p, fac_s


def topo_media_model(kind, ni=300, nj=300, nk=150, steps=1500, dt=None,
                     npml=12, seed=2025, nrecv=400, nmaxwell=3):
    """The topography model with a VTI (kind "vti"), tilted TI (kind
    "aniso", all 21 constants) or GMB visco-elastic (kind "visco") medium.

    vti:   the three layers perturbed by 5 % with a seeded Gaussian random
           field of 2 km correlation; Thomsen epsilon, delta ~ U[0, 0.2] and
           gamma ~ U[0, 0.1] per point (independent seeded fields mapped
           through the normal CDF); converted to c11, c13, c33, c55, c66.
    aniso: the vti medium with its symmetry axis tilted 30 degrees +- 10
           (seeded Gaussian random field) towards azimuth 40 degrees.
    visco: the three layers, Qp = 200, Qs = 100, `nmaxwell` Maxwell bodies
           fitted over 0.5-5 Hz with reference frequency 1.58 Hz.
    """
    p = topo_model(ni=ni, nj=nj, nk=nk, steps=steps, dt=dt, npml=npml,
                   seed=seed, nrecv=0)
    rho = (1.0 / p.media["slw"].astype(np.float64))
    mu = p.media["mu"].astype(np.float64)
    lam = p.media["lambda"].astype(np.float64)
    vs = np.sqrt(mu / rho)
    vp = np.sqrt((lam + 2 * mu) / rho)
    shape = (p.nz, p.ny, p.nx)
    if kind in ("vti", "aniso"):
        pert = 1.0 + 0.05 * gaussian_field_3d(shape, 100.0, 2000.0, seed + 1).ravel()
        vp, vs, rho = vp * pert, vs * pert, rho * pert
        u = [normal_cdf(gaussian_field_3d(shape, 100.0, 2000.0, seed + s).ravel())
             for s in (2, 3, 4)]
        eps, delta, gamma = 0.2 * u[0], 0.2 * u[1], 0.1 * u[2]
        c11, c13, c33, c55, c66 = thomsen_to_vti(vp, vs, rho, eps, delta, gamma)
        p.medium_type = abi.CGFD_MEDIUM_ELASTIC_VTI
        p.media = {"slw": np.ascontiguousarray((1.0 / rho).astype(np.float32)),
                   "c11": c11, "c13": c13, "c33": c33, "c55": c55, "c66": c66}
        if kind == "aniso":
            tilt = np.radians(30.0 + 10.0 * gaussian_field_3d(shape, 100.0, 2000.0,
                                                              seed + 5).ravel())
            p.medium_type = abi.CGFD_MEDIUM_ELASTIC_ANISO
            p.media = dict(slw=p.media["slw"],
                           **tti_stiffness(c11, c13, c33, c55, c66, tilt, np.radians(40.0)))
    elif kind == "visco":
        wl, YP, YS, fac_p, fac_s = gmb_coefficients(200.0, 100.0, nmaxwell,
                                                    0.5, 5.0, 1.58)
        mu_u = mu * fac_s
        lam_u = (lam + 2 * mu) * fac_p - 2 * mu_u
        p.medium_type = abi.CGFD_MEDIUM_VISCOELASTIC_ISO
        p.media["lambda"] = lam_u.astype(np.float32)
        p.media["mu"] = mu_u.astype(np.float32)
        p.nmaxwell = nmaxwell
        p.wl = wl
        r = (2.0 * mu_u / lam_u)
        p.Ylam = [((1.0 + r) * YP[n] - r * YS[n]).astype(np.float32)
                  for n in range(nmaxwell)]
        p.Ymu = [np.full(p.vol, YS[n], np.float32) for n in range(nmaxwell)]
        # memory variables: 6 per Maxwell body after the 9 components
        ncmp = 9 + 6 * nmaxwell
        wav = np.zeros(NLEVEL * ncmp * p.vol, np.float32)
        p.ncmp = ncmp
        p.wav = wav
        for row in p.pml:
            for f in row:
                if f is not None:
                    n9 = f["aux"].size // (NLEVEL * 9)
                    f["aux"] = np.zeros(NLEVEL * ncmp * n9, np.float32)
        X, Y, Z = _coords_of(p, seed)
        p.coords = {"x3d": X, "y3d": Y, "z3d": Z}
    else:
        raise ValueError(kind)
    side = int(round(math.sqrt(nrecv)))
    if nrecv > 0:
        coords = [(npml + 2 + (ni - 2 * npml - 4) * a / max(side - 1, 1),
                   npml + 2 + (nj - 2 * npml - 4) * b / max(side - 1, 1))
                  for a in range(side) for b in range(side)][:nrecv]
        add_surface_receivers(p, [(int(x), int(y)) for x, y in coords])
    return p


def _coords_of(p, seed):
    """Grid coordinates of topo_model's grid (flattened float32)."""
    dh = 100.0
    ni, nj, nk = p.ni, p.nj, p.nk
    Lx, Ly = (ni - 1) * dh, (nj - 1) * dh
    rough = gaussian_roughness(ni + 6, nj + 6, dh, 100.0, 1000.0, seed)

    def surface(X, Y):
        r2 = (X - Lx / 2) ** 2 + (Y - Ly / 2) ** 2
        return 2000.0 * np.exp(-r2 / 5000.0 ** 2) + rough

    X, Y, Z = grid_coords(ni, nj, nk, dh, surface, -(nk - 1) * dh)
    return [np.ascontiguousarray(a, dtype=np.float32).ravel() for a in (X, Y, Z)]


# ---------------------------------------------------------------------------
# batched shots: windows of the topography model (config 3)
# ---------------------------------------------------------------------------

def _topo_base(ni, nj, nk, seed):
    """Grid, metrics and layered media of the topography model (padded
    (nz, ny, nx) arrays)."""
    dh = 100.0
    Lx, Ly = (ni - 1) * dh, (nj - 1) * dh
    rough = gaussian_roughness(ni + 6, nj + 6, dh, 100.0, 1000.0, seed)

    def surface(X, Y):
        r2 = (X - Lx / 2) ** 2 + (Y - Ly / 2) ** 2
        return 2000.0 * np.exp(-r2 / 5000.0 ** 2) + rough

    X, Y, Z = grid_coords(ni, nj, nk, dh, surface, -(nk - 1) * dh)
    met = {k: v.reshape(nk + 6, nj + 6, ni + 6) for k, v in metrics(X, Y, Z).items()}
    vp, vs, rho = layered(Z, Z[-4], [(3000.0, 4000.0, 2310.0, 2400.0),
                                     (10000.0, 5500.0, 3175.0, 2650.0),
                                     (None, 6500.0, 3750.0, 2900.0)])
    return X, Y, Z, met, vp, vs, rho


def moment_random(rng, m0=1e16):
    """Six i.i.d. N(0,1) components, Frobenius-normalised, times m0:
    (Mxx, Myy, Mzz, Myz, Mxz, Mxy)."""
    m = rng.standard_normal(6)
    fro = math.sqrt(m[0] ** 2 + m[1] ** 2 + m[2] ** 2 + 2 * (m[3] ** 2 + m[4] ** 2 + m[5] ** 2))
    return tuple(float(m0 * v / fro) for v in m)


def window_shots(nshot, base=(400, 400, 200), wmin=(128, 128, 96),
                 wmax=(256, 256, 160), steps=1000, dt=0.005, npml=12,
                 seed=2026, nrecv=64, base_model=None):
    """`nshot` shots, each on its own window of the topography model: window
    sizes uniform in [wmin, wmax] (seeded), placed inside the base model with
    the free surface at the top; per shot a source at depth 1-8 km (inside
    the window, at least PML + 3 cells from its sides), a random moment
    tensor (six i.i.d. N(0,1) components, Frobenius-normalised), Ricker
    2 Hz, and `nrecv` surface receivers on a regular grid.  Metrics and
    media are cropped from the base model (ghost layers are the base
    model's neighbouring values)."""
    rng = np.random.default_rng(seed)
    bni, bnj, bnk = base
    if base_model is None:
        base_model = _topo_base(bni, bnj, bnk, seed)
    X, Y, Z, met, vp, vs, rho = base_model
    shots = []
    for s in range(nshot):
        wi = int(rng.integers(wmin[0], wmax[0] + 1))
        wj = int(rng.integers(wmin[1], wmax[1] + 1))
        wk = int(rng.integers(wmin[2], wmax[2] + 1))
        wi, wj, wk = min(wi, bni), min(wj, bnj), min(wk, bnk)
        i0 = int(rng.integers(0, bni - wi + 1))
        j0 = int(rng.integers(0, bnj - wj + 1))
        k0 = bnk - wk                       # window top = base surface
        sl = (slice(k0, k0 + wk + 6), slice(j0, j0 + wj + 6), slice(i0, i0 + wi + 6))
        p = Problem(wi, wj, wk, dt, steps + 1)
        p.metric = {k: np.ascontiguousarray(v[sl]).ravel() for k, v in met.items()}
        set_iso_media(p, vp[sl], vs[sl], rho[sl])
        p.free_top = 1
        add_pml(p, X[sl], Y[sl], Z[sl], npml, [(0, 0), (0, 1), (1, 0), (1, 1), (2, 0)],
                vref=6500.0, alpha_max=math.pi * 2.0)
        margin = npml + 3
        depth = rng.uniform(1000.0, min(8000.0, (wk - margin - 2) * 100.0))
        si = p.ni1 + int(rng.integers(margin, wi - margin))
        sj = p.nj1 + int(rng.integers(margin, wj - margin))
        sk = p.nk2 - int(round(depth / 100.0))
        add_moment_source(p, si, sj, sk, moment_random(rng), fc=2.0, t0=0.6,
                          stf_len=min(steps + 1, 400) * dt)
        side = int(round(math.sqrt(nrecv)))
        coords = [(npml + 2 + (wi - 2 * npml - 4) * a / max(side - 1, 1),
                   npml + 2 + (wj - 2 * npml - 4) * b / max(side - 1, 1))
                  for a in range(side) for b in range(side)][:nrecv]
        add_surface_receivers(p, [(int(x), int(y)) for x, y in coords])
        p.window = dict(i0=i0, j0=j0, k0=k0)
        shots.append(p)
    return shots
