"""Python binding of the C oracle (oracle/cgfd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, never by the product package.
"""

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "libcgfd_oracle.so")

TIMG_ZERO = 0     # value the reference build reads beyond its local array
TIMG_MIRROR = 1   # the mirror the traction-image formula intends


def build(force=False):
    """Compile the oracle with gcc (x86-64 and aarch64 alike)."""
    src = os.path.join(HERE, "cgfd_oracle.c")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(src)):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    subprocess.run(["gcc", "-O3", "-ffp-contract=off", "-fPIC", "-shared",
                    "-I" + os.path.join(REPO, "include"), "-o", LIB, src,
                    "-lpthread", "-lm"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.oracle_allstep.restype = C.c_int
        _lib.oracle_allstep.argtypes = [C.c_void_p, C.c_int, C.c_int,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.oracle_allstep_pg.restype = C.c_int
        _lib.oracle_allstep_pg.argtypes = [C.c_void_p, C.c_int, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p]
        _lib.oracle_dvh2dvz_iso.restype = C.c_int
        _lib.oracle_dvh2dvz_iso.argtypes = [C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p]
        _lib.oracle_dvh2dvz_vti.restype = C.c_int
        _lib.oracle_dvh2dvz_vti.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.oracle_dvh2dvz_vis.restype = C.c_int
        _lib.oracle_dvh2dvz_vis.argtypes = [C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p]
    return _lib


def allstep(problem, timg_mode=TIMG_ZERO, nthreads=1, want_mats=False,
            want_pg=False):
    """Run the oracle on a cgfd3d_gb300.problem.Problem in place.

    Returns the free-surface matrices (want_mats) and/or the 15 peak-motion
    maps (want_pg) when asked for."""
    import numpy as np
    cs = problem.to_c()
    mats = None
    if problem.free_top:
        n2 = problem.nx * problem.ny * 9
        mats = [np.zeros(n2, np.float32) for _ in range(3)]
        ptrs = [m.ctypes.data for m in mats]
    else:
        ptrs = [None, None, None]
    pg = None
    if want_pg and problem.free_top:
        pg = np.zeros(15 * problem.nx * problem.ny, np.float32)
    rc = lib().oracle_allstep_pg(C.addressof(cs), timg_mode, nthreads, *ptrs,
                                 None if pg is None else pg.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle_allstep failed with code %d" % rc)
    if want_mats and want_pg:
        return mats, pg
    if want_pg:
        return pg
    return mats if want_mats else None


# ---------------------------------------------------------------------------
# double-precision build of the same time loop (cgfd_oracle_f64.c)
# ---------------------------------------------------------------------------

LIB64 = os.path.join(HERE, "_build", "libcgfd_oracle_f64.so")


def build64(force=False):
    """Compile the double-precision instantiation of the oracle."""
    srcs = [os.path.join(HERE, f) for f in ("cgfd_oracle_f64.c", "cgfd_oracle.c")]
    if (not force and os.path.exists(LIB64)
            and os.path.getmtime(LIB64) >= max(os.path.getmtime(s) for s in srcs)):
        return LIB64
    os.makedirs(os.path.dirname(LIB64), exist_ok=True)
    subprocess.run(["gcc", "-O3", "-ffp-contract=off", "-fPIC", "-shared",
                    "-I" + os.path.join(REPO, "include"), "-I" + HERE, "-o", LIB64,
                    srcs[0], "-lpthread", "-lm"], check=True)
    return LIB64


_lib64 = None
_wide = {}


def _widen(t):
    """The ctypes type of `t` with every float (and pointer to float) made
    double, as cgfd_oracle_f64.c sees the problem description."""
    if t is C.c_float:
        return C.c_double
    if isinstance(t, type) and issubclass(t, C._Pointer) and t._type_ is C.c_float:
        return C.POINTER(C.c_double)
    if isinstance(t, type) and issubclass(t, C.Array):
        return _widen(t._type_) * t._length_
    if isinstance(t, type) and issubclass(t, C.Structure):
        if t not in _wide:
            _wide[t] = type(t.__name__ + "64", (C.Structure,),
                            {"_fields_": [(n, _widen(ft)) for n, ft in t._fields_]})
        return _wide[t]
    return t


def _copy_wide(src, dst):
    for name, ft in type(src)._fields_:
        v = getattr(src, name)
        wt = dict(type(dst)._fields_)[name]
        if isinstance(ft, type) and issubclass(ft, C.Structure):
            _copy_wide(v, getattr(dst, name))
        elif isinstance(ft, type) and issubclass(ft, C.Array):
            _copy_array(v, getattr(dst, name), ft)
        elif isinstance(ft, type) and issubclass(ft, C._Pointer) and ft._type_ is C.c_float:
            setattr(dst, name, C.cast(v, wt))
        else:
            setattr(dst, name, v)


def _copy_array(src, dst, ft):
    et = ft._type_
    for n in range(ft._length_):
        if isinstance(et, type) and issubclass(et, C.Structure):
            _copy_wide(src[n], dst[n])
        elif isinstance(et, type) and issubclass(et, C.Array):
            _copy_array(src[n], dst[n], et)
        elif isinstance(et, type) and issubclass(et, C._Pointer) and et._type_ is C.c_float:
            dst[n] = C.cast(src[n], C.POINTER(C.c_double))
        else:
            dst[n] = src[n]


def _as_f64(obj):
    """Deep copy of a problem's containers with every float32 array as a
    float64 array (ints and scalars unchanged)."""
    import numpy as np
    if isinstance(obj, np.ndarray):
        return obj.astype(np.float64) if obj.dtype == np.float32 else obj
    if isinstance(obj, dict):
        return {k: _as_f64(v) for k, v in obj.items()}
    if isinstance(obj, list):
        return [_as_f64(v) for v in obj]
    return obj


def widen_problem(problem):
    """A copy of a cgfd3d_gb300.problem.Problem whose float32 arrays are
    float64 (the inputs as the FP32 runs read them, exactly)."""
    q = problem.copy()
    for k, v in list(q.__dict__.items()):
        q.__dict__[k] = _as_f64(v)
    return q


def allstep64(problem, timg_mode=TIMG_ZERO, nthreads=1):
    """Run the double-precision oracle on a copy of `problem` (float32
    inputs widened exactly to float64).  Returns the widened problem, whose
    wavefield, PML auxiliaries and seismograms then hold the FP64 results
    (problem.level(problem.final_level()) etc.)."""
    import numpy as np
    global _lib64
    if _lib64 is None:
        _lib64 = C.CDLL(build64())
        _lib64.oracle_allstep_pg.restype = C.c_int
        _lib64.oracle_allstep_pg.argtypes = [C.c_void_p, C.c_int, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p]
    q = widen_problem(problem)
    cs = q.to_c()                      # float-typed pointers to double data
    cw = _widen(type(cs))()
    _copy_wide(cs, cw)
    cw._keep = cs._keep
    mats = [np.zeros(q.nx * q.ny * 9, np.float64) for _ in range(3)] if q.free_top else None
    ptrs = [m.ctypes.data for m in mats] if mats else [None, None, None]
    rc = _lib64.oracle_allstep_pg(C.addressof(cw), timg_mode, nthreads, *ptrs, None)
    if rc != 0:
        raise RuntimeError("oracle_allstep (double) failed with code %d" % rc)
    return q


def surface_matrices(problem):
    """Free-surface matrices of the problem's medium, as the oracle computes
    them before the time loop: dict of matVx2Vz2, matVy2Vz2, matF2Vz2 and,
    for visco-elastic media, matD (each nx*ny*9)."""
    import numpy as np
    cs = problem.to_c()
    n2 = problem.nx * problem.ny * 9
    out = {k: np.zeros(n2, np.float32)
           for k in ("matVx2Vz2", "matVy2Vz2", "matF2Vz2")}
    ptr = {k: v.ctypes.data for k, v in out.items()}
    if problem.medium_type == 3:
        lib().oracle_dvh2dvz_vti(C.addressof(cs), ptr["matVx2Vz2"], ptr["matVy2Vz2"])
    elif problem.medium_type == 4:
        L = lib()
        L.oracle_dvh2dvz_aniso.argtypes = [C.c_void_p] * 3
        L.oracle_dvh2dvz_aniso(C.addressof(cs), ptr["matVx2Vz2"], ptr["matVy2Vz2"])
    elif problem.medium_type == 5:
        out["matD"] = np.zeros(n2, np.float32)
        lib().oracle_dvh2dvz_vis(C.addressof(cs), ptr["matVx2Vz2"],
                                 ptr["matVy2Vz2"], out["matD"].ctypes.data)
    else:
        lib().oracle_dvh2dvz_iso(C.addressof(cs), ptr["matVx2Vz2"],
                                 ptr["matVy2Vz2"], ptr["matF2Vz2"])
    return out


def metric_calc(nx, ny, nz, ni1, ni2, nj1, nj2, nk1, nk2, x3d, y3d, z3d):
    """Grid metrics as the reference computes them (jac, xi_x..zeta_z;
    10 x nx*ny*nz float32)."""
    import numpy as np
    L = lib()
    L.oracle_metric_calc.restype = C.c_int
    L.oracle_metric_calc.argtypes = [C.c_int] * 9 + [C.c_void_p] * 4
    x, y, z = [np.ascontiguousarray(a, np.float32).ravel() for a in (x3d, y3d, z3d)]
    out = np.zeros(10 * nx * ny * nz, np.float32)
    L.oracle_metric_calc(nx, ny, nz, ni1, ni2, nj1, nj2, nk1, nk2, x.ctypes.data,
                         y.ctypes.data, z.ctypes.data, out.ctypes.data)
    return out.reshape(10, -1)


def locate(x3d, y3d, z3d, points, is_depth=None):
    """Points located on a curvilinear grid (padded (nz, ny, nx) coordinates,
    3 ghost layers) as the reference locates stations and sources given by
    coordinates.  Returns found (n,), global physical indices (n, 3), shifts
    (n, 3) and the located z (n,) (depths converted)."""
    import numpy as np
    L = lib()
    L.oracle_locate.restype = C.c_int
    L.oracle_locate.argtypes = [C.c_int] * 3 + [C.c_void_p] * 3 + [C.c_int] + [C.c_void_p] * 8
    nz, ny, nx = np.shape(x3d)
    x, y, z = [np.ascontiguousarray(a, np.float32).ravel() for a in (x3d, y3d, z3d)]
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    n = len(pts)
    px, py, pz = [np.ascontiguousarray(pts[:, d]) for d in range(3)]
    dep = np.zeros(n, np.int32) if is_depth is None else np.ascontiguousarray(is_depth, np.int32)
    found = np.zeros(n, np.int32)
    idx = np.zeros((n, 3), np.int32)
    shift = np.zeros((n, 3), np.float32)
    zout = np.zeros(n, np.float32)
    L.oracle_locate(nx, ny, nz, x.ctypes.data, y.ctypes.data, z.ctypes.data, n,
                    px.ctypes.data, py.ctypes.data, pz.ctypes.data, dep.ctypes.data,
                    found.ctypes.data, idx.ctypes.data, shift.ctypes.data, zout.ctypes.data)
    return found, idx, shift, zout


LAYER_METHODS = {"loc": 0, "har": 1, "ari": 2}
LAYER_KINDS = {"one_component": 0, "elastic_isotropic": 21, "elastic_vti_prem": 22, "elastic_vti_thomsen": 23,
               "elastic_vti_cij": 24}


def layer(model, x3d, y3d, z3d, method="loc"):
    """A layered model (dict of cgfd3d_gb300.media.read_md3lay) discretised
    on a grid as the reference's media_layer2model_el_iso / _el_vti do with
    the equivalent-medium method "loc", "har" or "ari": (var,) for
    one-component models (media_layer2model_onecmp), (lambda, mu, rho) for
    elastic isotropic models, (c11, c33, c55, c66, c13, rho) for VTI ones;
    None where the reference would exit (point outside the interface mesh or,
    isotropic, vp <= sqrt(2) vs)."""
    import numpy as np
    L = lib()
    L.oracle_layer.restype = C.c_int
    L.oracle_layer.argtypes = ([C.c_int] * 5 + [C.c_float] * 4 + [C.c_void_p] +
                               [C.c_int] * 3 + [C.c_void_p] * 4)
    kind = LAYER_KINDS[model.get("media_type", "elastic_isotropic")]
    nz, ny, nx = np.shape(x3d)
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    rec = np.ascontiguousarray(model["rec"], np.float32)
    out = [np.zeros((nz, ny, nx), np.float32) for _ in range({0: 1, 21: 3}.get(kind, 6))]
    ptrs = (C.c_void_p * len(out))(*[o.ctypes.data for o in out])
    bad = L.oracle_layer(kind, LAYER_METHODS[method], model["NI"], model["NX"], model["NY"],
                         model["MINX"], model["MINY"], model["DX"], model["DY"],
                         rec.ctypes.data, nx, ny, nz, x.ctypes.data, y.ctypes.data,
                         z.ctypes.data, C.cast(ptrs, C.c_void_p))
    return None if bad else tuple(out)


def layer_el_iso(model, x3d, y3d, z3d, method="loc"):
    """lambda, mu, rho of an elastic isotropic layered model (see layer)."""
    return layer(model, x3d, y3d, z3d, method)


def layer_el_iso_loc(model, x3d, y3d, z3d):
    """layer_el_iso with the "loc" method."""
    return layer_el_iso(model, x3d, y3d, z3d, "loc")


def bin_model(m, x3d, y3d, z3d, vis=False):
    """A model given as binary volumes (dict: order, size, spacing, origin,
    ext and the file-order volumes rho_vol, vp_vol, vs_vol or qp_vol, qs_vol)
    interpolated on a grid as media_bin2model_el_iso (rho, lambda, mu) or
    media_bin2model_vis_iso (Qp, Qs) does; None where the reference exits."""
    import numpy as np
    L = lib()
    L.oracle_bin.restype = C.c_int
    L.oracle_bin.argtypes = [C.c_int] + [C.c_void_p] * 6 + [C.c_int] * 3 + [C.c_void_p] * 4
    nz, ny, nx = np.shape(x3d)
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    keys = ("qp_vol", "qs_vol") if vis else ("rho_vol", "vp_vol", "vs_vol")
    vols = [np.ascontiguousarray(m[k], np.float32) for k in keys]
    hdr = [np.ascontiguousarray(m[k], t) for k, t in
           (("order", np.int32), ("size", np.int32), ("spacing", np.float32),
            ("origin", np.float32), ("ext", np.float32))]
    out = [np.zeros((nz, ny, nx), np.float32) for _ in keys]
    vp_ = (C.c_void_p * len(vols))(*[v.ctypes.data for v in vols])
    op_ = (C.c_void_p * len(out))(*[o.ctypes.data for o in out])
    bad = L.oracle_bin(1 if vis else 0, *[h.ctypes.data for h in hdr], C.cast(vp_, C.c_void_p),
                       nx, ny, nz, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                       C.cast(op_, C.c_void_p))
    return None if bad else tuple(out)


def grid_el_iso(model, x3d, y3d, z3d, method="loc"):
    """An elastic isotropic 3-D grid model (dict of
    cgfd3d_gb300.media.read_md3grd) discretised on a grid as the reference's
    media_grid2model_el_iso does: (rho, lambda, mu); None where the reference
    would exit."""
    import numpy as np
    L = lib()
    L.oracle_grid_el_iso.restype = C.c_int
    L.oracle_grid_el_iso.argtypes = ([C.c_int] * 3 + [C.c_void_p] + [C.c_int] * 2 +
                                     [C.c_float] * 4 + [C.c_void_p] + [C.c_int] * 3 +
                                     [C.c_void_p] * 4)
    nz, ny, nx = np.shape(x3d)
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    rec = np.ascontiguousarray(model["rec"], np.float32)
    ngz = np.ascontiguousarray(model["ngz"], np.int32)
    out = [np.zeros((nz, ny, nx), np.float32) for _ in range(3)]
    ptrs = (C.c_void_p * 3)(*[o.ctypes.data for o in out])
    bad = L.oracle_grid_el_iso(LAYER_METHODS[method], model["NI"], model["NL"], ngz.ctypes.data,
                               model["NX"], model["NY"], model["MINX"], model["MINY"],
                               model["DX"], model["DY"], rec.ctypes.data, nx, ny, nz,
                               x.ctypes.data, y.ctypes.data, z.ctypes.data,
                               C.cast(ptrs, C.c_void_p))
    return None if bad else tuple(out)


def grid_el_vti_loc(model, x3d, y3d, z3d):
    """An elastic VTI 3-D grid model (dict of cgfd3d_gb300.media.read_md3grd)
    with "loc", as media_grid2model_el_vti: (c11, c33, c55, c66, c13, rho);
    None where the reference would exit."""
    import numpy as np
    L = lib()
    L.oracle_grid_el_vti_loc.restype = C.c_int
    L.oracle_grid_el_vti_loc.argtypes = ([C.c_int] * 3 + [C.c_void_p] + [C.c_int] * 2 +
                                         [C.c_float] * 4 + [C.c_void_p] + [C.c_int] * 3 +
                                         [C.c_void_p] * 4)
    nz, ny, nx = np.shape(x3d)
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    rec = np.ascontiguousarray(model["rec"], np.float32)
    ngz = np.ascontiguousarray(model["ngz"], np.int32)
    out = [np.zeros((nz, ny, nx), np.float32) for _ in range(6)]
    ptrs = (C.c_void_p * 6)(*[o.ctypes.data for o in out])
    bad = L.oracle_grid_el_vti_loc(LAYER_KINDS[model["media_type"]], model["NI"], model["NL"],
                                   ngz.ctypes.data, model["NX"], model["NY"], model["MINX"],
                                   model["MINY"], model["DX"], model["DY"], rec.ctypes.data,
                                   nx, ny, nz, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                   C.cast(ptrs, C.c_void_p))
    return None if bad else tuple(out)
