"""Stations and sources given by coordinates, located on the device.

:class:`Locator` wraps ``cgfd_locator_*`` (include/cgfd3d_gpu.h): the
reference's search of a curvilinear grid for the cell holding a point and
of the point's shift in it (gd_curv_coord_to_glob_indx,
forward/gd_t.c:1917-1995, with gd_curv_depth_to_axis, :2179-2297, for points
given by depth), with the same results bit for bit.  :func:`stations` then
turns located stations into the receiver arrays of a problem as
io_recv_read_locate does (forward/io_funcs.c:233-414).
"""

import ctypes as C

import numpy as np

from . import _lib

GHOSTS = 3


class Locator:
    """A grid (padded (nz, ny, nx) coordinates) resident on the device."""

    def __init__(self, x3d, y3d, z3d):
        self.shape = np.shape(x3d)
        if len(self.shape) != 3 or np.shape(y3d) != self.shape or np.shape(z3d) != self.shape:
            raise ValueError("x3d, y3d, z3d must be (nz, ny, nx) arrays of one shape")
        nz, ny, nx = self.shape
        x, y, z = [np.ascontiguousarray(a, np.float32) for a in (x3d, y3d, z3d)]
        self._h = C.c_void_p()
        _lib.check(_lib.lib().cgfd_locator_create(nx, ny, nz, x.ctypes.data, y.ctypes.data,
                                                   z.ctypes.data, C.byref(self._h)))

    def locate(self, points, is_depth=None):
        """points (n, 3) of x, y, z (z a depth below the surface where
        is_depth is set).  Returns found (n,), global physical indices
        (n, 3), shifts (n, 3) and the located z (n,)."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        n = len(pts)
        px, py, pz = [np.ascontiguousarray(pts[:, d]) for d in range(3)]
        dep = None if is_depth is None else np.ascontiguousarray(is_depth, np.int32)
        if dep is not None and dep.shape != (n,):
            raise ValueError("is_depth must hold one flag per point")
        found = np.zeros(n, np.int32)
        idx = np.zeros((n, 3), np.int32)
        shift = np.zeros((n, 3), np.float32)
        zout = np.zeros(n, np.float32)
        _lib.check(_lib.lib().cgfd_locator_locate(
            self._h, n, px.ctypes.data, py.ctypes.data, pz.ctypes.data,
            None if dep is None else dep.ctypes.data, found.ctypes.data, idx.ctypes.data,
            shift.ctypes.data, zout.ctypes.data))
        return found, idx, shift, zout

    def close(self):
        if self._h:
            _lib.lib().cgfd_locator_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def stations(shape, index, shift):
    """Receiver arrays from located stations, as io_recv_read_locate builds
    them for stations given by coordinates (forward/io_funcs.c:311-402): a
    negative shift moves to the cell below (shift + 1, index - 1); stations
    outside the physical points are dropped; the shift is zeroed at the last
    physical index of each axis; eight interpolation corners.  shape: the
    padded (nz, ny, nx).  Returns (kept station numbers, dijk (3 per
    station), indx1d (8 per station))."""
    nz, ny, nx = shape
    ni, nj, nk = nx - 2 * GHOSTS, ny - 2 * GHOSTS, nz - 2 * GHOSTS
    keep, dijk, idx = [], [], []
    for r in range(len(index)):
        g = [int(v) for v in index[r]]
        s = [np.float32(v) for v in shift[r]]
        for d in range(3):
            if s[d] < 0.0:
                s[d] = np.float32(1.0 + np.float64(s[d]))
                g[d] -= 1
        if not (0 <= g[0] <= ni - 1 and 0 <= g[1] <= nj - 1 and 0 <= g[2] <= nk - 1):
            continue
        il, jl, kl = g[0] + GHOSTS, g[1] + GHOSTS, g[2] + GHOSTS
        if il == ni - 1 + GHOSTS:
            s[0] = np.float32(0.0)
        if jl == nj - 1 + GHOSTS:
            s[1] = np.float32(0.0)
        if kl == nk - 1 + GHOSTS:
            s[2] = np.float32(0.0)
        keep.append(r)
        dijk += s
        for c in range(8):
            a, b, e = c & 1, (c >> 1) & 1, c >> 2
            idx.append((il + a) + (jl + b) * nx + (kl + e) * nx * ny)
    return keep, np.array(dijk, np.float32), np.array(idx, np.int32)
