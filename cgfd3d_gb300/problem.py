"""Host-side problem description in the reference's array layout.

A :class:`Problem` holds numpy arrays for everything the time loop of
CGFD3D's ``drv_rk_curv_col_allstep`` (forward/drv_rk_curv_col.c:27-556)
reads and writes, and turns them into the flat C struct of
include/cgfd3d_gpu.h (``to_c()``).  The arrays keep the reference layout:
padded volumes (ni+6, nj+6, nk+6) flattened as i + j*nx + k*nx*ny, wavefield
levels x components x volume (forward/wav_t.c:40-136), PML auxiliary
variables level x component x face box (forward/bdry_t.c:290-327).
"""

import ctypes as C
import json

import numpy as np

from . import abi

NCMP_EL = 9
NLEVEL = 4
COMPONENTS = ["Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz", "Tyz", "Txz", "Txy"]


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a, ctype=C.c_float):
    if a is None:
        return C.POINTER(ctype)()
    return a.ctypes.data_as(C.POINTER(ctype))


class Problem:
    """Numpy-backed problem; attribute names follow the reference structs."""

    def __init__(self, ni, nj, nk, dt, nt_total, t0=0.0, ncmp=NCMP_EL):
        self.ni, self.nj, self.nk = int(ni), int(nj), int(nk)
        self.nx, self.ny, self.nz = self.ni + 6, self.nj + 6, self.nk + 6
        self.ni1, self.ni2 = 3, 3 + self.ni - 1
        self.nj1, self.nj2 = 3, 3 + self.nj - 1
        self.nk1, self.nk2 = 3, 3 + self.nk - 1
        self.dt, self.t0, self.nt_total = float(dt), float(t0), int(nt_total)
        self.ncmp, self.nlevel = int(ncmp), NLEVEL
        self.metric = {}
        self.coords = {}          # x3d, y3d, z3d (visco free surface only)
        self.medium_type = abi.CGFD_MEDIUM_ELASTIC_ISO
        self.media = {}
        self.nmaxwell = 0
        self.wl = None
        self.Ylam, self.Ymu = [], []
        self.free_top = 0
        self.graves_qs = None     # dict(Qs=volume, freq=Hz): Graves Q attenuation
        self.ablexp = None        # dict(Ex, Ey, Ez, blk (6, 7)): exponential sponge
        self.dd = None            # dict(si, sj, sk, max_nt, vi, mij): dd sources
        self.pml = [[None, None] for _ in range(3)]
        self.src = None
        self.recv = None
        self.line = None
        self.wav = np.zeros(self.nlevel * self.ncmp * self.vol, np.float32)

    # -- sizes ---------------------------------------------------------------
    @property
    def vol(self):
        return self.nx * self.ny * self.nz

    @property
    def grid_dims(self):
        return (self.ni, self.nj, self.nk, self.nx, self.ny, self.nz,
                self.ni1, self.ni2, self.nj1, self.nj2, self.nk1, self.nk2)

    @property
    def n_phys(self):
        return self.ni * self.nj * self.nk

    def final_level(self):
        """Level holding the state after nt_total steps (pre/end swap)."""
        return 3 if self.nt_total % 2 == 1 else 0

    def level(self, lev):
        n = self.ncmp * self.vol
        return self.wav[lev * n:(lev + 1) * n]

    def component(self, lev, c):
        v = self.vol
        return self.level(lev)[c * v:(c + 1) * v].reshape(self.nz, self.ny, self.nx)

    def pml_final(self, d, s):
        f = self.pml[d][s]
        n = f["aux"].size // NLEVEL
        lev = self.final_level()
        return f["aux"][lev * n:(lev + 1) * n]

    # -- conversion ------------------------------------------------------------
    def to_c(self):
        """Build the C struct; the returned object keeps the arrays alive."""
        s = abi.Problem()
        for name, val in zip(["ni", "nj", "nk", "nx", "ny", "nz", "ni1", "ni2",
                              "nj1", "nj2", "nk1", "nk2"], self.grid_dims):
            setattr(s, name, val)
        keep = []

        def P(a, ctype=C.c_float):
            if a is None:
                return C.POINTER(ctype)()
            keep.append(a)
            return _ptr(a, ctype)

        for n in abi.METRIC_NAMES:
            setattr(s, n, P(self.metric.get(n)))
        s.medium_type = self.medium_type
        s.slw = P(self.media.get("slw"))
        s.lambda_ = P(self.media.get("lambda"))
        s.mu = P(self.media.get("mu"))
        for n in abi.ANISO_NAMES:
            setattr(s, n, P(self.media.get(n)))
        s.nmaxwell = self.nmaxwell
        s.wl = P(self.wl)
        for m in range(len(self.Ylam)):
            s.Ylam[m] = P(self.Ylam[m])
            s.Ymu[m] = P(self.Ymu[m])
        s.free_top = int(self.free_top)
        for d in range(3):
            for side in range(2):
                f = self.pml[d][side]
                face = s.pml[d][side]
                if f is None:
                    face.enabled = 0
                    continue
                face.enabled = 1
                (face.ni1, face.ni2, face.nj1, face.nj2, face.nk1,
                 face.nk2) = [int(v) for v in f["box"]]
                face.A, face.B, face.D = P(f["A"]), P(f["B"]), P(f["D"])
                face.aux = P(f["aux"])
        src = self.src
        if src is not None and src["n"] > 0:
            s.src_n = src["n"]
            s.src_max_nt = src["max_nt"]
            s.src_max_stage = src["max_stage"]
            s.src_force = src["force"]
            s.src_moment = src["moment"]
            s.src_spatial = src["spatial"]
            s.src_ext_half = src["ext_half"]
            s.src_ext_coef = src["ext_coef"]
            s.src_surface_strict = src.get("surface_strict", 0)
            s.src_n_surface_force = src.get("n_surface_force", 0)
            for n in ("si", "sj", "sk", "it_begin", "it_end"):
                setattr(s, "src_" + n, P(src[n], C.c_int))
            for n in ("si_inc", "sj_inc", "sk_inc"):
                setattr(s, "src_" + n, P(src[n]))
            for n in ("Fx", "Fy", "Fz", "Mxx", "Myy", "Mzz", "Mxz", "Myz", "Mxy"):
                setattr(s, n, P(src.get(n)))
            if src.get("n_surface_force", 0) > 0:
                s.src_force_rate_indx = P(src["force_rate_indx"], C.c_int)
                for n in ("Fx_rate", "Fy_rate", "Fz_rate"):
                    setattr(s, n, P(src[n]))
        r = self.recv
        if r is not None and r["n"] > 0:
            s.recv_n, s.recv_max_nt, s.recv_ncmp = r["n"], r["max_nt"], r["ncmp"]
            s.recv_dijk = P(r["dijk"])
            s.recv_indx1d = P(r["indx1d"], C.c_int)
            s.recv_seismo = P(r["seismo"])
        ln = self.line
        if ln is not None and ln["n"] > 0:
            s.line_n, s.line_max_nt = ln["n"], ln["max_nt"]
            s.line_iptr = P(ln["iptr"], C.c_int)
            s.line_seismo = P(ln["seismo"])
        s.ncmp, s.nlevel = self.ncmp, self.nlevel
        s.wav = P(self.wav)
        s.dt, s.t0, s.nt_total = self.dt, self.t0, self.nt_total
        for n in ("x3d", "y3d", "z3d"):
            setattr(s, n, P(self.coords.get(n)))
        if self.graves_qs is not None:
            s.graves_qs = 1
            s.qs_freq = float(self.graves_qs["freq"])
            s.Qs = P(self.graves_qs["Qs"])
        if self.dd is not None:
            d = self.dd
            s.dd_n, s.dd_max_nt = len(d["si"]), int(d["max_nt"])
            s.dd_si, s.dd_sj, s.dd_sk = [P(d[k], C.c_int) for k in ("si", "sj", "sk")]
            s.dd_vi, s.dd_mij = P(d.get("vi")), P(d.get("mij"))
        if self.ablexp is not None:
            s.ablexp = 1
            s.ablexp_Ex, s.ablexp_Ey, s.ablexp_Ez = [P(self.ablexp[k]) for k in ("Ex", "Ey", "Ez")]
            blk = np.asarray(self.ablexp["blk"], np.int32).reshape(6, 7)
            for n in range(6):
                for m in range(7):
                    s.ablexp_blk[n][m] = int(blk[n, m])
        s._keep = keep
        return s

    def copy(self):
        """Deep copy of every mutable array (inputs shared)."""
        q = Problem.__new__(Problem)
        q.__dict__.update(self.__dict__)
        q.wav = self.wav.copy()
        q.pml = [[None if f is None else dict(f, aux=f["aux"].copy())
                  for f in row] for row in self.pml]
        if self.recv is not None:
            q.recv = dict(self.recv, seismo=self.recv["seismo"].copy())
        if self.line is not None:
            q.line = dict(self.line, seismo=self.line["seismo"].copy())
        return q


def from_golden(path_or_npz):
    """Problem with the inputs of a golden fixture (tests/golden/*.npz).

    Returns (problem, expected) where expected holds the reference outputs.
    """
    d = np.load(path_or_npz) if isinstance(path_or_npz, str) else path_or_npz
    g = d["gd.dims"]
    nt_total = int(d["nt_total"][0])
    p = Problem(g[0], g[1], g[2], float(d["dt"][0]), nt_total,
                float(d["t0"][0]), int(d["wav.ncmp"][0]))
    assert tuple(int(v) for v in g) == p.grid_dims
    for n in abi.METRIC_NAMES:
        p.metric[n] = _f32(d["metric." + n])
    for n in ("x3d", "y3d", "z3d"):
        if "gd." + n in d:
            p.coords[n] = _f32(d["gd." + n])
    p.medium_type = int(d["md.medium_type"][0])
    p.media["slw"] = _f32(d["md.slw"])
    for n in ["lambda", "mu"] + abi.ANISO_NAMES:
        if "md." + n in d:
            p.media[n] = _f32(d["md." + n])
    if "md.nmaxwell" in d:
        p.nmaxwell = int(d["md.nmaxwell"][0])
        p.wl = _f32(d["md.wl"])
        p.Ylam = [_f32(d["md.Ylam.%d" % m]) for m in range(p.nmaxwell)]
        p.Ymu = [_f32(d["md.Ymu.%d" % m]) for m in range(p.nmaxwell)]
    free = d["bdry.is_sides_free"].reshape(3, 2)
    p.free_top = int(free[2, 1])
    if "md.Qs" in d:
        p.graves_qs = dict(Qs=_f32(d["md.Qs"]), freq=float(d["md.visco_Qs_freq"][0]))
    if "src.dd_total_number" in d and int(d["src.dd_is_valid"][0]) == 1:
        nd = int(d["src.dd_total_number"][0])
        p.dd = dict(si=_i32(d["src.dd_si"]), sj=_i32(d["src.dd_sj"]), sk=_i32(d["src.dd_sk"]),
                    max_nt=int(d["src.dd_max_nt"][0]),
                    vi=_f32(d["src.dd_vi"]) if "src.dd_vi" in d else None,
                    mij=_f32(d["src.dd_mij"]) if "src.dd_mij" in d else None)
        assert len(p.dd["si"]) == nd
    if "bdry.ablexp_Ex" in d:
        p.ablexp = dict(Ex=_f32(d["bdry.ablexp_Ex"]), Ey=_f32(d["bdry.ablexp_Ey"]),
                        Ez=_f32(d["bdry.ablexp_Ez"]), blk=_i32(d["bdry.ablexp_blk"]))
    pml = d["bdry.is_sides_pml"].reshape(3, 2)
    # the final state whole, or (fixtures of the full-size configurations)
    # only some planes of it, keyed by name ("k62", "j53", ...)
    expected = {}
    if "out.wav.final" in d:
        expected["wav"] = d["out.wav.final"]
    planes = {k[len("out.wav.plane."):]: d[k] for k in d.files
              if k.startswith("out.wav.plane.")}
    if planes:
        expected["planes"] = planes
    for dd in range(3):
        for s in range(2):
            if pml[dd, s] != 1:
                continue
            key = "pml.%d.%d." % (dd, s)
            aux0 = _f32(d[key + "aux0"])      # level 0 (pre) only
            aux = np.zeros(NLEVEL * aux0.size, np.float32)
            aux[:aux0.size] = aux0
            p.pml[dd][s] = dict(box=_i32(d[key + "box"]), A=_f32(d[key + "A"]),
                                B=_f32(d[key + "B"]), D=_f32(d[key + "D"]),
                                aux=aux)
            if "out.pml.%d.%d.final" % (dd, s) in d:
                expected["pml.%d.%d" % (dd, s)] = d["out.pml.%d.%d.final" % (dd, s)]
    ns = int(d["src.total_number"][0])
    if ns > 0:
        src = dict(n=ns, max_nt=int(d["src.max_nt"][0]),
                   max_stage=int(d["src.max_stage"][0]),
                   force=int(d["src.force_actived"][0]),
                   moment=int(d["src.moment_actived"][0]),
                   spatial=int(d["src.itype_spatial_ext"][0]),
                   ext_half=int(d["src.ext_half_npoint"][0]),
                   ext_coef=float(d["src.ext_func_coef"][0]),
                   surface_strict=int(d["src.is_surface_force_strict"][0]),
                   n_surface_force=int(d["src.total_number_surface_force"][0]))
        for n in ("si", "sj", "sk", "it_begin", "it_end"):
            src[n] = _i32(d["src." + n])
        for n in ("si_inc", "sj_inc", "sk_inc"):
            src[n] = _f32(d["src." + n])
        for n in ("Fx", "Fy", "Fz", "Mxx", "Myy", "Mzz", "Mxz", "Myz", "Mxy"):
            if "src." + n in d:
                src[n] = _f32(d["src." + n])
        if src["n_surface_force"] > 0:
            src["force_rate_indx"] = _i32(d["src.force_rate_indx"])
            for n in ("Fx_rate", "Fy_rate", "Fz_rate"):
                src[n] = _f32(d["src." + n])
        p.src = src
    nr = int(d["recv.total_number"][0])
    if nr > 0:
        max_nt, ncmp = int(d["recv.max_nt"][0]), int(d["recv.ncmp"][0])
        p.recv = dict(
            n=nr, max_nt=max_nt, ncmp=ncmp,
            dijk=_f32(np.concatenate([d["recv.%d.dijk" % r] for r in range(nr)])),
            indx1d=_i32(np.concatenate([d["recv.%d.indx1d" % r] for r in range(nr)])),
            seismo=np.zeros(nr * ncmp * max_nt, np.float32))
        expected["recv"] = np.concatenate(
            [d["out.recv.%d.seismo" % r] for r in range(nr)])
    nl = int(d["line.num_of_lines"][0])
    if nl > 0:
        iptr = np.concatenate([d["line.%d.iptr" % l] for l in range(nl)])
        max_nt = int(d["line.max_nt"][0])
        p.line = dict(n=int(iptr.size), max_nt=max_nt, iptr=_i32(iptr),
                      seismo=np.zeros(iptr.size * p.ncmp * max_nt, np.float32))
        expected["line"] = np.concatenate(
            [d["out.line.%d.seismo" % l] for l in range(nl)])
    lev0 = _f32(d["wav.level0"])
    p.wav[:lev0.size] = lev0
    if "out.matVx2Vz2" in d:
        expected["matVx2Vz2"] = d["out.matVx2Vz2"]
        expected["matVy2Vz2"] = d["out.matVy2Vz2"]
        expected["matF2Vz2"] = d["out.matF2Vz2"]
    if "out.matD" in d:
        expected["matD"] = d["out.matD"]
    if "case.json" in d:
        expected["case"] = json.loads(bytes(d["case.json"]).decode())
    return p, expected
