"""Media discretisation: layered and binary-volume models onto a grid.

``read_md3lay`` parses the reference's layered-model text format (.md3lay,
media/media_read_file.cpp:22-240) for elastic isotropic models;
``layer_el_iso`` discretises such a model on a curvilinear grid on the
device (``cgfd_media_layer_el_iso``) as the reference's
media_layer2model_el_iso does (media/media_layer2model.cpp:140-190, 422-560,
1334-1384, 1984-2190).  "loc": per grid point the interfaces' elevations
interpolated at (x, y), the layer below the point, each property's value
plus its gradient times depth-below-interface to its power, the mean of the
two layers for points on an interface, then lambda, mu, rho.  "har" / "ari":
points whose cell touches more than one layer are recomputed from 9^3
samples of the cell, averaged harmonically (kappa, mu) or arithmetically.
"""

import ctypes as C

import numpy as np

from . import _lib

# columns of a layer record: elevation, then (value, gradient, power) of each
# property of the media type, in the .md3lay file's order
# (media/media_read_file.cpp:150-400)
MD3LAY_PROPERTIES = {
    "one_component": ["var"],
    "elastic_isotropic": ["rho", "vp", "vs"],
    "elastic_vti_prem": ["rho", "vph", "vpv", "vsh", "vsv", "eta"],
    "elastic_vti_thomsen": ["rho", "vp0", "vs0", "epsilon", "delta", "gamma"],
    "elastic_vti_cij": ["rho", "c11", "c33", "c55", "c66", "c13"],
}
# the media-type numbers of the reference (media/media_utility.hpp:40-43),
# also those of cgfd_media_layer_el_vti's media_type argument
MEDIA_TYPE_CODES = {"one_component": 0, "elastic_isotropic": 21, "elastic_vti_prem": 22,
                    "elastic_vti_thomsen": 23, "elastic_vti_cij": 24}
MD3LAY_COLUMNS = ["elevation", "rho", "rho_grad", "rho_pow", "vp", "vp_grad", "vp_pow",
                  "vs", "vs_grad", "vs_pow"]


def read_md3lay(text):
    """A .md3lay model (text or path) of one component or an elastic
    isotropic or VTI medium
    as a dict: media_type, NI, NX, NY, MINX, MINY, DX, DY and rec
    (NI, NY, NX, 1 + 3 * properties) float32; lines starting with '#' and
    empty lines are skipped, as the reference's reader does."""
    if "\n" not in text:
        with open(text) as f:
            text = f.read()
    words = []
    for line in text.splitlines(True):
        if line.startswith("#") or line == "\n":
            continue
        words += line.split()
    if not words or words[0] not in MD3LAY_PROPERTIES:
        raise ValueError("layered models of %s are read" % ", ".join(MD3LAY_PROPERTIES))
    kind = words[0]
    nc = 1 + 3 * len(MD3LAY_PROPERTIES[kind])
    NI = int(words[1])
    NX, NY = int(words[2]), int(words[3])
    MINX, MINY, DX, DY = [np.float32(w) for w in words[4:8]]
    vals = np.array([np.float32(w) for w in words[8:8 + NI * NY * NX * nc]], np.float32)
    if vals.size != NI * NY * NX * nc or NI < 1 or NX < 2 or NY < 2:
        raise ValueError("incomplete layered model")
    return dict(media_type=kind, NI=NI, NX=NX, NY=NY, MINX=float(MINX), MINY=float(MINY),
                DX=float(DX), DY=float(DY), rec=vals.reshape(NI, NY, NX, nc))


def layer_el_iso(model, x3d, y3d, z3d, method="loc"):
    """lambda, mu, rho of an elastic isotropic model on the grid (arrays
    shaped like x3d), computed on the device with the equivalent-medium
    method "loc", "har" or "ari"."""
    if model.get("media_type", "elastic_isotropic") != "elastic_isotropic":
        raise ValueError("layer_el_iso takes elastic_isotropic models")
    shape = np.shape(x3d)
    nz, ny, nx = shape
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    rec = np.ascontiguousarray(model["rec"], np.float32)
    out = [np.empty(shape, np.float32) for _ in range(3)]
    _lib.check(_lib.lib().cgfd_media_layer_el_iso(
        int(model["NI"]), int(model["NX"]), int(model["NY"]), C.c_float(model["MINX"]),
        C.c_float(model["MINY"]), C.c_float(model["DX"]), C.c_float(model["DY"]),
        rec.ctypes.data, nx, ny, nz, x.ctypes.data, y.ctypes.data, z.ctypes.data,
        method.encode(), *[o.ctypes.data for o in out]))
    return tuple(out)


def layer_el_vti(model, x3d, y3d, z3d, method="loc"):
    """c11, c33, c55, c66, c13, rho of an elastic VTI model
    (elastic_vti_prem, _thomsen or _cij) on the grid, computed on the device
    (cgfd_media_layer_el_vti)."""
    kind = model.get("media_type")
    if kind not in ("elastic_vti_prem", "elastic_vti_thomsen", "elastic_vti_cij"):
        raise ValueError("layer_el_vti takes elastic_vti_* models")
    shape = np.shape(x3d)
    nz, ny, nx = shape
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    rec = np.ascontiguousarray(model["rec"], np.float32)
    out = [np.empty(shape, np.float32) for _ in range(6)]
    _lib.check(_lib.lib().cgfd_media_layer_el_vti(
        MEDIA_TYPE_CODES[kind], int(model["NI"]), int(model["NX"]), int(model["NY"]),
        C.c_float(model["MINX"]), C.c_float(model["MINY"]), C.c_float(model["DX"]),
        C.c_float(model["DY"]), rec.ctypes.data, nx, ny, nz, x.ctypes.data, y.ctypes.data,
        z.ctypes.data, method.encode(), *[o.ctypes.data for o in out]))
    return tuple(out)


def layer(model, x3d, y3d, z3d, method="loc"):
    """The model's medium on the grid: (lambda, mu, rho) for elastic
    isotropic models, (c11, c33, c55, c66, c13, rho) for VTI ones.
    One-component models (Qp, Qs) are read but not discretised on the
    device."""
    kind = model.get("media_type", "elastic_isotropic")
    if kind == "one_component":
        raise ValueError("one-component layered models are not discretised on the device")
    if kind == "elastic_isotropic":
        return layer_el_iso(model, x3d, y3d, z3d, method)
    return layer_el_vti(model, x3d, y3d, z3d, method)


class BinModel(C.Structure):
    """cgfd_bin_model_t: the layout of a model given as binary volumes, as
    the reference's par file gives it (bin_order, bin_size, bin_spacing,
    bin_origin)."""
    _fields_ = [("order", C.c_int * 3), ("size", C.c_int * 3), ("spacing", C.c_float * 3),
                ("origin", C.c_float * 3)]

    @classmethod
    def of(cls, order, size, spacing, origin):
        m = cls()
        for d in range(3):
            m.order[d], m.size[d] = int(order[d]), int(size[d])
            m.spacing[d], m.origin[d] = float(spacing[d]), float(origin[d])
        return m


def bin_model(layout, ext, vols, x3d, y3d, z3d, vis=False):
    """A model given as binary volumes on the grid, on the device: rho,
    lambda, mu from (rho, vp, vs) volumes, or Qp, Qs from (Qp, Qs) volumes
    when vis is set.  layout: BinModel; ext: the grid's xmin, xmax, ymin,
    ymax; vols: the volumes as stored in their files (flat or shaped)."""
    shape = np.shape(x3d)
    nz, ny, nx = shape
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    nfile = layout.size[0] * layout.size[1] * layout.size[2]
    v = [np.ascontiguousarray(a, np.float32).ravel() for a in vols]
    if len(v) != (2 if vis else 3) or any(a.size != nfile for a in v):
        raise ValueError("expected %d volumes of %d samples" % (2 if vis else 3, nfile))
    out = [np.empty(shape, np.float32) for _ in v]
    fn = _lib.lib().cgfd_media_bin_vis_iso if vis else _lib.lib().cgfd_media_bin_el_iso
    _lib.check(fn(C.byref(layout), *[C.c_float(float(e)) for e in ext],
                  *[a.ctypes.data for a in v], nx, ny, nz, x.ctypes.data, y.ctypes.data,
                  z.ctypes.data, *[o.ctypes.data for o in out]))
    return tuple(out)


class BinBox(C.Structure):
    """cgfd_bin_box_t: first sample and count per file dimension."""
    _fields_ = [("first", C.c_int * 3), ("count", C.c_int * 3)]


def bin_crop(layout, ext, z3d):
    """The box of the files a grid needs (cgfd_media_bin_crop): (first,
    count) per file dimension."""
    nz, ny, nx = np.shape(z3d)
    z = np.ascontiguousarray(z3d, np.float32)
    box = BinBox()
    _lib.check(_lib.lib().cgfd_media_bin_crop(C.byref(layout), *[C.c_float(float(e)) for e in ext],
                                              nx, ny, nz, z.ctypes.data, C.byref(box)))
    return tuple(box.first), tuple(box.count)


def bin_model_box(layout, ext, box, vols, x3d, y3d, z3d, vis=False):
    """bin_model on volumes holding only `box` = (first, count) of the files
    (file order, count[0] fastest), as a caller that read just that box
    passes them (cgfd_media_bin_el_iso_box / _vis_iso_box)."""
    shape = np.shape(x3d)
    nz, ny, nx = shape
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    b = BinBox()
    for d in range(3):
        b.first[d], b.count[d] = int(box[0][d]), int(box[1][d])
    n = b.count[0] * b.count[1] * b.count[2]
    v = [np.ascontiguousarray(a, np.float32).ravel() for a in vols]
    if len(v) != (2 if vis else 3) or any(a.size != n for a in v):
        raise ValueError("expected %d volumes of %d samples" % (2 if vis else 3, n))
    out = [np.empty(shape, np.float32) for _ in v]
    fn = _lib.lib().cgfd_media_bin_vis_iso_box if vis else _lib.lib().cgfd_media_bin_el_iso_box
    _lib.check(fn(C.byref(layout), C.byref(b), *[C.c_float(float(e)) for e in ext],
                  *[a.ctypes.data for a in v], nx, ny, nz, x.ctypes.data, y.ctypes.data,
                  z.ctypes.data, *[o.ctypes.data for o in out]))
    return tuple(out)


def read_md3grd(text, ext):
    """An elastic isotropic or VTI 3-D grid model (.md3grd text or path) as the
    reference's reader leaves it for a grid of extent ext = (xmin, xmax,
    ymin, ymax) (read_grid_file, media/media_read_file.cpp): the mesh
    cropped to columns floor((xmin - MINX) / DX) .. ceil((xmax - MINX) / DX)
    and the rows alike.  Returns a dict: media_type, NL, ngz (levels per
    layer), NI (levels), NX, NY, MINX, MINY, DX, DY and rec (NI, NY, NX, 4 or
    7) = elevation, then rho, vp, vs or the six VTI parameters.  The file has
    no comment lines (the reference's reader takes none)."""
    if "\n" not in text:
        with open(text) as f:
            text = f.read()
    words = text.split()
    ncol = {"elastic_isotropic": 4, "elastic_vti_prem": 7, "elastic_vti_thomsen": 7,
            "elastic_vti_cij": 7}
    if not words or words[0] not in ncol:
        raise ValueError("grid models of %s are read" % ", ".join(ncol))
    kind, nc = words[0], ncol[words[0]]
    NL = int(words[1])
    ngz = [int(w) for w in words[2:2 + NL]]
    NI = sum(ngz)
    pos = 2 + NL
    NX, NY = int(words[pos]), int(words[pos + 1])
    MINX, MINY, DX, DY = [np.float32(w) for w in words[pos + 2:pos + 6]]
    vals = np.array([np.float32(w) for w in words[pos + 6:pos + 6 + NI * NY * NX * nc]],
                    np.float32)
    if NL < 1 or min(ngz) < 1 or NX < 2 or NY < 2 or vals.size != NI * NY * NX * nc:
        raise ValueError("incomplete grid model")
    full = vals.reshape(NI, NY, NX, nc)
    xmin, xmax, ymin, ymax = [np.float32(e) for e in ext]
    q = lambda a, b, d: np.float32(np.float32(a - b) / d)
    ix0, iy0 = q(xmin, MINX, DX), q(ymin, MINY, DY)
    if ix0 < 0 or iy0 < 0:
        raise ValueError("the grid model does not cover the grid")
    ix0, iy0 = int(ix0), int(iy0)
    ix1, iy1 = int(np.ceil(q(xmax, MINX, DX))), int(np.ceil(q(ymax, MINY, DY)))
    if ix1 > NX - 1 or iy1 > NY - 1:
        raise ValueError("the grid model does not cover the grid")
    minx = np.float32(np.float32(ix0 * DX) + MINX)
    miny = np.float32(np.float32(iy0 * DY) + MINY)
    return dict(media_type=kind, NL=NL, ngz=ngz, NI=NI, NX=ix1 - ix0 + 1,
                NY=iy1 - iy0 + 1, MINX=float(minx), MINY=float(miny), DX=float(DX),
                DY=float(DY), rec=np.ascontiguousarray(full[:, iy0:iy1 + 1, ix0:ix1 + 1]))


def grid_el_iso(model, x3d, y3d, z3d, method="loc"):
    """rho, lambda, mu of an elastic isotropic 3-D grid model (dict of
    read_md3grd) on the grid, computed on the device
    (cgfd_media_grid_el_iso)."""
    shape = np.shape(x3d)
    nz, ny, nx = shape
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    rec = np.ascontiguousarray(model["rec"], np.float32)
    ngz = np.ascontiguousarray(model["ngz"], np.int32)
    out = [np.empty(shape, np.float32) for _ in range(3)]
    _lib.check(_lib.lib().cgfd_media_grid_el_iso(
        int(model["NI"]), int(model["NL"]), ngz.ctypes.data, int(model["NX"]), int(model["NY"]),
        C.c_float(model["MINX"]), C.c_float(model["MINY"]), C.c_float(model["DX"]),
        C.c_float(model["DY"]), rec.ctypes.data, nx, ny, nz, x.ctypes.data, y.ctypes.data,
        z.ctypes.data, method.encode(), *[o.ctypes.data for o in out]))
    return tuple(out)


def grid_el_vti(model, x3d, y3d, z3d, method="loc"):
    """c11, c33, c55, c66, c13, rho of an elastic VTI 3-D grid model (dict of
    read_md3grd) on the grid with "loc", computed on the device
    (cgfd_media_grid_el_vti)."""
    shape = np.shape(x3d)
    nz, ny, nx = shape
    x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
    rec = np.ascontiguousarray(model["rec"], np.float32)
    ngz = np.ascontiguousarray(model["ngz"], np.int32)
    out = [np.empty(shape, np.float32) for _ in range(6)]
    _lib.check(_lib.lib().cgfd_media_grid_el_vti(
        MEDIA_TYPE_CODES[model["media_type"]], int(model["NI"]), int(model["NL"]),
        ngz.ctypes.data, int(model["NX"]), int(model["NY"]), C.c_float(model["MINX"]),
        C.c_float(model["MINY"]), C.c_float(model["DX"]), C.c_float(model["DY"]),
        rec.ctypes.data, nx, ny, nz, x.ctypes.data, y.ctypes.data, z.ctypes.data,
        method.encode(), *[o.ctypes.data for o in out]))
    return tuple(out)
