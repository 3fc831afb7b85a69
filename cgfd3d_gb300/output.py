"""Output of the time loop: slices and snapshots of the wavefield, SAC
seismograms of stations and receiver lines.

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

import numpy as np

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


# ---------------------------------------------------------------------------
# SAC seismograms
# ---------------------------------------------------------------------------
#
# SAC binary files (the Seismic Analysis Code's published format): a header
# of 70 floats, 40 ints and 23 character fields (192 bytes), then npts
# floats, in the byte order of the writing host.  The reference fills it as
# lib/sacLib.c:8-389 does: every field "undefined" (-12345, "-12345  "),
# then delta, b = 0, e = delta*(npts-1), nvhdr 6, npts, iftype ITIME (1),
# leven 1, the event and station fields, cmpaz = cmpinc = 0, and kstnm /
# kcmpnm copied from an 8-byte "-12345" (two trailing NULs, not spaces).

_SAC_NFLOAT, _SAC_NINT = 70, 40
_SAC_F = {"delta": 0, "b": 5, "e": 6, "stla": 31, "stlo": 32, "stel": 33, "stdp": 34,
          "evla": 35, "evlo": 36, "evel": 37, "evdp": 38, "cmpaz": 57, "cmpinc": 58}
_SAC_I = {"nvhdr": 6, "npts": 9, "iftype": 15, "leven": 35}
# character fields in order: kstnm, kevnm (16 bytes), then 21 of 8 bytes
_SAC_K_WIDTHS = [8, 16] + [8] * 21
_SAC_KCMPNM = 19          # index of kcmpnm among the character fields
_SAC_LE = np.dtype("<f4"), np.dtype("<i4")


def sac_bytes(trace, delta, stla, stlo, stel, stdp, evla=0.0, evlo=0.0, evel=0.0,
              evdp=0.0):
    """The bytes of one SAC file as sacExport1C1R writes it (little-endian,
    the byte order of x86-64 and aarch64 hosts)."""
    tr = np.ascontiguousarray(trace, dtype=np.float32).ravel()
    npts = tr.size
    f = np.full(_SAC_NFLOAT, -12345.0, np.float32)
    i = np.full(_SAC_NINT, -12345, np.int32)
    d = np.float32(delta)
    f[_SAC_F["delta"]] = d
    f[_SAC_F["b"]] = 0.0
    f[_SAC_F["e"]] = d * np.float32(npts - 1)
    for k, v in (("stla", stla), ("stlo", stlo), ("stel", stel), ("stdp", stdp),
                 ("evla", evla), ("evlo", evlo), ("evel", evel), ("evdp", evdp),
                 ("cmpaz", 0.0), ("cmpinc", 0.0)):
        f[_SAC_F[k]] = np.float32(v)
    i[_SAC_I["nvhdr"]] = 6
    i[_SAC_I["npts"]] = npts
    i[_SAC_I["iftype"]] = 1
    i[_SAC_I["leven"]] = 1
    chars = []
    for n, w in enumerate(_SAC_K_WIDTHS):
        if n in (0, _SAC_KCMPNM):
            chars.append(b"-12345\0\0")
        else:
            chars.append(b"-12345  ".ljust(w, b"\0"))
    return (f.astype(_SAC_LE[0]).tobytes() + i.astype(_SAC_LE[1]).tobytes() +
            b"".join(chars) + tr.astype(_SAC_LE[0]).tobytes())


CMP_NAMES = ["Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz", "Tyz", "Txz", "Txy"]


def _write(path, data):
    with open(path, "wb") as fh:
        fh.write(data)


def write_station_sac(out_dir, evtnm, names, xyz, seismo, dt, cmp_names=CMP_NAMES,
                      visco=False):
    """One SAC file per station and component, "<dir>/<evt>.<name>.<cmp>.sac",
    as io_recv_output_sac writes them (forward/io_funcs.c:1648-1692): the
    station's x, y, z in stla, stlo, stel and dt in both stdp and delta (the
    reference's argument order); GMB media write the first 9 components.
    seismo: (nstation, ncmp, nt).  Returns the paths."""
    seismo = np.asarray(seismo, np.float32)
    ncmp = 9 if visco else seismo.shape[1]
    paths = []
    for r, name in enumerate(names):
        x, y, z = xyz[r]
        for c in range(ncmp):
            path = "%s/%s.%s.%s.sac" % (out_dir, evtnm, name, cmp_names[c])
            _write(path, sac_bytes(seismo[r, c], dt, x, y, z, dt))
            paths.append(path)
    return paths


def station_strain_iso(lam, mu, stress):
    """Strain from the six stress traces of an isotropic station
    (forward/io_funcs.c:1719-1745), float arithmetic as the reference
    rounds it: E1, E2, E3 evaluated in double and stored as float.
    stress: (6, nt) in the order Txx, Tyy, Tzz, Tyz, Txz, Txy."""
    lam, mu = np.float32(lam), np.float32(mu)
    ld, md = np.float64(lam), np.float64(mu)
    e1 = np.float32(np.float64(lam + mu) / (md * (3.0 * ld + 2.0 * md)))
    e2 = np.float32(-ld / (2.0 * md * (3.0 * ld + 2.0 * md)))
    e3 = np.float32(1.0 / md)
    t = np.asarray(stress, np.float32)
    e0 = e2 * ((t[0] + t[1]) + t[2])
    d = e2 - e1
    out = np.empty_like(t)
    for n in range(3):
        out[n] = e0 - d * t[n]
    half = 0.5 * np.float64(e3)
    for n in range(3, 6):
        out[n] = (half * t[n].astype(np.float64)).astype(np.float32)
    return out


def write_station_strain_sac(out_dir, evtnm, names, xyz, seismo, lam, mu, dt):
    """Exx, Eyy, Ezz, Eyz, Exz, Exy SAC files of each station of an isotropic
    (or GMB visco-elastic) medium, as io_recv_output_sac_el_iso_strain writes
    them (forward/io_funcs.c:1698-1778); lam, mu: the media at each station's
    first interpolation point.  Returns the paths."""
    seismo = np.asarray(seismo, np.float32)
    paths = []
    for r, name in enumerate(names):
        x, y, z = xyz[r]
        e = station_strain_iso(lam[r], mu[r], seismo[r, 3:9])
        for n, cmp in enumerate(("Exx", "Eyy", "Ezz", "Eyz", "Exz", "Exy")):
            path = "%s/%s.%s.%s.sac" % (out_dir, evtnm, name, cmp)
            _write(path, sac_bytes(e[n], dt, x, y, z, dt))
            paths.append(path)
    return paths


def write_line_sac(out_dir, evtnm, line_name, seq, xyz, seismo, dt, cmp_names=CMP_NAMES):
    """SAC files of a receiver line, "<dir>/<evt>.<line>.no<seq>.<cmp>.sac",
    as io_line_output_sac writes them (forward/io_funcs.c:1823-1862).
    seismo: (nreceiver, ncmp, nt).  Returns the paths."""
    seismo = np.asarray(seismo, np.float32)
    paths = []
    for r in range(seismo.shape[0]):
        x, y, z = xyz[r]
        for c in range(seismo.shape[1]):
            path = "%s/%s.%s.no%d.%s.sac" % (out_dir, evtnm, line_name, seq[r], cmp_names[c])
            _write(path, sac_bytes(seismo[r, c], dt, x, y, z, dt))
            paths.append(path)
    return paths
