"""Output of the time loop: slices and snapshots of the wavefield.

Slices and snapshots are boxes of the state packed on the device
(:meth:`cgfd3d_gb300.solver.Solver.pack_boxes`, ``cgfd_solver_pack_boxes``),
so an output step copies only the points the writers read instead of the
whole wavefield.  The helpers below build the boxes that the reference's
writers read and say at which steps a snapshot is due:

* ``io_slice_nc_put`` (forward/io_funcs.c:992-1111): every step, components
  0..ncmp-1 (0..8 for GMB visco-elastic media, whose memory variables are not
  written), an x slice over (k, j) of the physical points, a y slice over
  (k, i), a z slice over (j, i);
* ``io_snap_nc_put`` (forward/io_funcs.c:1114-1268): a box with strides,
  written when ``it >= it1`` and ``(it - it1) % dit == 0`` and
  ``(it - it1) / dit <= (nt_total - it1) / dit`` (C integer division).
"""

from . import abi


def _visco(problem):
    return int(problem.medium_type) == abi.CGFD_MEDIUM_VISCOELASTIC_ISO


def slice_components(problem):
    """Last component index a slice holds (io_funcs.c:1018-1020)."""
    return 8 if _visco(problem) else int(problem.ncmp) - 1


def slice_boxes(problem, x=(), y=(), z=()):
    """Boxes of x slices at padded indices ``x``, y slices at ``y`` and z
    slices at ``z``, in that order, as io_slice_nc_put reads them."""
    p = problem
    c2 = slice_components(p)
    ni, nj, nk = p.ni2 - p.ni1 + 1, p.nj2 - p.nj1 + 1, p.nk2 - p.nk1 + 1
    out = []
    for i in x:
        out.append(abi.Box(0, c2, int(i), 1, 1, p.nj1, nj, 1, p.nk1, nk, 1))
    for j in y:
        out.append(abi.Box(0, c2, p.ni1, ni, 1, int(j), 1, 1, p.nk1, nk, 1))
    for k in z:
        out.append(abi.Box(0, c2, p.ni1, ni, 1, p.nj1, nj, 1, int(k), 1, 1))
    return out


def snapshot_box(i1, ni, di, j1, nj, dj, k1, nk, dk, c1=0, c2=8):
    """Box of one snapshot (iosnap_t fields i1, ni, di, ...), components
    c1..c2 (velocity 0..2, stress 3..8; strain is converted from stress)."""
    return abi.Box(c1, c2, i1, ni, di, j1, nj, dj, k1, nk, dk)


def _cdiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def _cmod(a, b):
    return a - b * _cdiv(a, b)


def snapshot_due(it, nt_total, it1, dit):
    """Whether io_snap_nc_put writes a snapshot (it1, dit) at step it."""
    return (it >= it1 and _cdiv(it - it1, dit) <= _cdiv(nt_total - it1, dit)
            and _cmod(it - it1, dit) == 0)
