"""Media discretisation: layered models onto a grid.

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

# columns of a layer record: elevation, then (value, gradient, power) of
# rho, vp, vs
MD3LAY_COLUMNS = ["elevation", "rho", "rho_grad", "rho_pow", "vp", "vp_grad", "vp_pow",
                  "vs", "vs_grad", "vs_pow"]


def read_md3lay(text):
    """An elastic isotropic .md3lay model (text or path) as a dict: NI, NX,
    NY, MINX, MINY, DX, DY and rec (NI, NY, NX, 10) float32; lines starting
    with '#' and empty lines are skipped, as the reference's reader does."""
    if "\n" not in text:
        with open(text) as f:
            text = f.read()
    words = []
    for line in text.splitlines(True):
        if line.startswith("#") or line == "\n":
            continue
        words += line.split()
    if not words or words[0] != "elastic_isotropic":
        raise ValueError("only elastic_isotropic layered models are read")
    NI = int(words[1])
    NX, NY = int(words[2]), int(words[3])
    MINX, MINY, DX, DY = [np.float32(w) for w in words[4:8]]
    vals = np.array([np.float32(w) for w in words[8:8 + NI * NY * NX * 10]], np.float32)
    if vals.size != NI * NY * NX * 10 or NI < 1 or NX < 2 or NY < 2:
        raise ValueError("incomplete layered model")
    return dict(NI=NI, NX=NX, NY=NY, MINX=float(MINX), MINY=float(MINY), DX=float(DX),
                DY=float(DY), rec=vals.reshape(NI, NY, NX, 10))


def layer_el_iso(model, x3d, y3d, z3d, method="loc"):
    """lambda, mu, rho of the model on the grid (arrays shaped like x3d),
    computed on the device with the equivalent-medium method "loc", "har"
    or "ari"."""
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
