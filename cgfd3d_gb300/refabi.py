"""ctypes mirrors of the CGFD3D structs read by the drop-in entry point.

Field for field the declarations of include/cgfd3d_ref_abi.h (which restate
forward/fd_t.h, gd_t.h, md_t.h, src_t.h, bdry_t.h, wav_t.h, io_funcs.h and the
leading fields of mympi_t.h).  ``build_reference_structs`` fills them from a
:class:`cgfd3d_gb300.problem.Problem` so that ``drv_rk_curv_col_allstep`` can
be called exactly as the reference's ``main`` calls it
(forward/main_curv_col_el_3d.c:849-858).
"""

import ctypes as C

import numpy as np

from . import abi

PF = C.POINTER(C.c_float)
PPF = C.POINTER(PF)
PI = C.POINTER(C.c_int)
PPI = C.POINTER(PI)
PSZ = C.POINTER(C.c_size_t)
PCH = C.POINTER(C.c_char_p)
T = 4  # GD_TILE_N*


class FdOp(C.Structure):
    _fields_ = [("total_len", C.c_int), ("half_len", C.c_int),
                ("left_len", C.c_int), ("right_len", C.c_int),
                ("indx", PI), ("shift", PI), ("coef", PF)]


class Fd(C.Structure):
    _fields_ = ([("CFL", C.c_float), ("num_rk_stages", C.c_int),
                 ("rk_a", PF), ("rk_b", PF), ("rk_rhs_time", PF),
                 ("fdc_len", C.c_int), ("fdc_half_len", C.c_int),
                 ("fdc_nghosts", C.c_int), ("fdc_indx", PI), ("fdc_coef", PF)]
                + [(n, C.c_int) for n in (
                    "fdx_nghosts", "fdy_nghosts", "fdz_nghosts",
                    "fdx_max_len", "fdy_max_len", "fdz_max_len",
                    "fdx_max_half_len", "fdy_max_half_len", "fdz_max_half_len",
                    "num_of_pairs", "num_of_fdx_op", "num_of_fdy_op", "num_of_fdz_op")]
                + [("pair_fdx_op", C.c_void_p), ("pair_fdy_op", C.c_void_p),
                   ("pair_fdz_op", C.c_void_p)])


class Gd(C.Structure):
    _fields_ = ([("type", C.c_int)]
                + [(n, C.c_int) for n in (
                    "ni", "nj", "nk", "nx", "ny", "nz", "ni1", "ni2", "nj1", "nj2",
                    "nk1", "nk2", "npoint_ghosts", "fdx_nghosts", "fdy_nghosts",
                    "fdz_nghosts", "gni1", "gnj1", "gnk1", "gni2", "gnj2", "gnk2",
                    "ni1_to_glob_phys0", "nj1_to_glob_phys0", "nk1_to_glob_phys0",
                    "ni2_to_glob_phys0", "nj2_to_glob_phys0", "nk2_to_glob_phys0",
                    "n1", "n2", "n3", "n4", "ncmp")]
                + [(n, PF) for n in ("v4d", "x3d", "y3d", "z3d", "x1d", "y1d", "z1d")]
                + [(n, C.c_float) for n in (
                    "dx", "dy", "dz", "x0_glob", "y0_glob", "z0_glob", "xmin", "xmax",
                    "ymin", "ymax", "zmin", "zmax", "xmin_phy", "xmax_phy", "ymin_phy",
                    "ymax_phy", "zmin_phy", "zmax_phy")]
                + [(n, PF) for n in ("cell_xmin", "cell_xmax", "cell_ymin",
                                     "cell_ymax", "cell_zmin", "cell_zmax")]
                + [(n, C.c_int * T) for n in ("tile_istart", "tile_iend", "tile_jstart",
                                              "tile_jend", "tile_kstart", "tile_kend")]
                + [(n, ((C.c_float * T) * T) * T) for n in (
                    "tile_xmin", "tile_xmax", "tile_ymin", "tile_ymax", "tile_zmin",
                    "tile_zmax")]
                + [(n, C.c_size_t) for n in ("siz_iy", "siz_iz", "siz_icmp",
                                             "siz_line", "siz_slice", "siz_volume")]
                + [("cmp_pos", PSZ), ("cmp_name", PCH), ("index_name", PCH)])


class Metric(C.Structure):
    _fields_ = ([(n, C.c_int) for n in ("n1", "n2", "n3", "n4", "nx", "ny", "nz", "ncmp")]
                + [(n, PF) for n in ("v4d", "jac", "xi_x", "xi_y", "xi_z", "eta_x",
                                     "eta_y", "eta_z", "zeta_x", "zeta_y", "zeta_z")]
                + [(n, C.c_size_t) for n in ("siz_iy", "siz_iz", "siz_icmp")]
                + [("cmp_pos", PSZ), ("cmp_name", PCH)])


_CIJ = ["c11", "c12", "c13", "c14", "c15", "c16", "c22", "c23", "c24", "c25", "c26",
        "c33", "c34", "c35", "c36", "c44", "c45", "c46", "c55", "c56", "c66"]


class Md(C.Structure):
    _fields_ = ([(n, C.c_int) for n in ("n1", "n2", "n3", "n4", "nx", "ny", "nz", "ncmp")]
                + [("v4d", PF)]
                + [(n, C.c_size_t) for n in ("siz_iy", "siz_iz", "siz_icmp")]
                + [("cmp_pos", PSZ), ("cmp_name", PCH), ("medium_type", C.c_int),
                   ("rho", PF), ("kappa", PF), ("lambda_", PF), ("mu", PF),
                   ("nmaxwell", C.c_int), ("visco_GMB_freq", C.c_float),
                   ("visco_GMB_fmin", C.c_float), ("visco_GMB_fmax", C.c_float),
                   ("Qs", PF), ("Qp", PF), ("Ylam", PPF), ("Ymu", PPF), ("wl", PF)]
                + [(n, PF) for n in _CIJ]
                + [("visco_type", C.c_int), ("visco_Qs_freq", C.c_float)])


class Src(C.Structure):
    _fields_ = ([(n, C.c_int) for n in ("total_number", "max_nt", "max_stage", "it",
                                        "istage")]
                + [("evtnm", C.c_char * 1024)]
                + [(n, PI) for n in ("si", "sj", "sk")]
                + [(n, PF) for n in ("si_inc", "sj_inc", "sk_inc")]
                + [(n, PI) for n in ("it_begin", "it_end")]
                + [(n, C.c_int) for n in (
                    "is_surface_force_strict", "total_number_surface_force",
                    "idx_next_surface_force", "itype_spatial_ext", "ext_half_npoint",
                    "ext_length_npoint", "ext_size_npoint")]
                + [("ext_func_coef", C.c_float), ("force_actived", C.c_int),
                   ("moment_actived", C.c_int)]
                + [(n, PF) for n in ("Fx", "Fy", "Fz", "Mxx", "Myy", "Mzz", "Mxz",
                                     "Myz", "Mxy")]
                + [("force_rate_indx", PI)]
                + [(n, PF) for n in ("Fx_rate", "Fy_rate", "Fz_rate", "TxSrc", "TySrc",
                                     "TzSrc", "VxSrc", "VySrc", "VzSrc")]
                + [(n, C.c_int) for n in (
                    "dd_is_valid", "dd_is_add_at_point", "dd_smo_hlen", "dd_vi_actived",
                    "dd_mij_actived", "dd_total_number", "dd_max_nt", "dd_nt_per_read",
                    "dd_nt_this_read", "dd_it_here")]
                + [(n, PI) for n in ("dd_si", "dd_sj", "dd_sk")]
                + [("dd_indx", PSZ)]
                + [(n, PF) for n in ("dd_si_inc", "dd_sj_inc", "dd_sk_inc")]
                + [("fp_vi", C.c_void_p), ("fp_mij", C.c_void_p), ("dd_vi", PF),
                   ("dd_mij", PF)])


_POS = ["Vx_pos", "Vy_pos", "Vz_pos", "Txx_pos", "Tyy_pos", "Tzz_pos", "Tyz_pos",
        "Txz_pos", "Txy_pos"]


class AuxVar(C.Structure):
    _fields_ = ([("var", PF)]
                + [(n, C.c_int) for n in ("nx", "ny", "nz", "ncmp", "nlevel")]
                + [(n, C.c_size_t) for n in ("siz_iy", "siz_iz", "siz_icmp", "siz_ilevel")]
                + [("cmp_pos", PSZ), ("cmp_name", PCH), ("level_pos", PSZ)]
                + [(n, C.c_size_t) for n in _POS]
                + [(n, PF) for n in ("cur", "pre", "rhs", "end", "tmp")])


class BdryBlock(C.Structure):
    _fields_ = [(n, C.c_int) for n in (
        "enable", "nx1", "nx2", "ny1", "ny2", "nz1", "nz2", "nx", "ny", "nz",
        "ni1", "ni2", "nj1", "nj2", "nk1", "nk2", "ni", "nj", "nk")]


I32 = (C.c_int * 2) * 3
PF32 = (PF * 2) * 3


class Bdry(C.Structure):
    _fields_ = ([(n, I32) for n in ("is_sides_pml", "is_sides_free", "is_sides_mpml",
                                    "is_sides_ablexp")]
                + [(n, C.c_int) for n in ("is_enable_pml", "is_enable_free",
                                          "is_enable_mpml", "is_enable_ablexp",
                                          "nx", "ny", "nz")]
                + [(n, I32) for n in ("num_of_layers", "ni1", "ni2", "nj1", "nj2",
                                      "nk1", "nk2")]
                + [(n, PF32) for n in ("A", "B", "D", "Am", "Bm", "Dm")]
                + [("auxvar", (AuxVar * 2) * 3), ("bdry_blk", BdryBlock * 6)]
                + [(n, PF) for n in (
                    "ablexp_Ex", "ablexp_Ey", "ablexp_Ez", "matVx2Vz2", "matVy2Vz2",
                    "matD", "matF2Vz2", "matVx2Vz1", "matVy2Vz1", "matVy2Vx1",
                    "matVz2Vx1", "matVy2Vx2", "matVz2Vx2", "matVx2Vy1", "matVz2Vy1",
                    "matVx2Vy2", "matVz2Vy2")])


class Wav(C.Structure):
    _fields_ = ([("v5d", PF)]
                + [(n, C.c_int) for n in ("n1", "n2", "n3", "n4", "n5", "nx", "ny", "nz",
                                          "ncmp", "nlevel", "nmaxwell", "visco_type")]
                + [(n, C.c_size_t) for n in ("siz_iy", "siz_iz", "siz_icmp", "siz_ilevel")]
                + [("cmp_pos", PSZ), ("cmp_name", PCH), ("level_pos", PSZ)]
                + [(n, C.c_size_t) for n in _POS]
                + [(n.replace("_pos", "_seq"), C.c_size_t) for n in _POS]
                + [(n, PSZ) for n in ("Jxx_pos", "Jyy_pos", "Jzz_pos", "Jxy_pos",
                                      "Jxz_pos", "Jyz_pos", "Jxx_seq", "Jyy_seq",
                                      "Jzz_seq", "Jxy_seq", "Jxz_seq", "Jyz_seq")])


class RecvOne(C.Structure):
    _fields_ = ([(n, C.c_float) for n in ("x", "y", "z", "di", "dj", "dk")]
                + [(n, C.c_int) for n in ("i", "j", "k")]
                + [("indx1d", C.c_int * 8), ("seismo", PF), ("name", C.c_char * 1024)])


class Recv(C.Structure):
    _fields_ = [("total_number", C.c_int), ("max_nt", C.c_int), ("ncmp", C.c_int),
                ("recvone", C.POINTER(RecvOne))]


class Line(C.Structure):
    _fields_ = [("num_of_lines", C.c_int), ("max_nt", C.c_int), ("ncmp", C.c_int),
                ("line_nr", PI), ("line_seq", PI), ("recv_seq", PPI),
                ("recv_iptr", PPI), ("recv_x", PPF), ("recv_y", PPF), ("recv_z", PPF),
                ("recv_seismo", PPF), ("line_name", PCH)]


class Slice(C.Structure):
    _fields_ = [("siz_max_wrk", C.c_size_t),
                ("num_of_slice_x", C.c_int), ("slice_x_indx", PI), ("slice_x_fname", PCH),
                ("num_of_slice_y", C.c_int), ("slice_y_indx", PI), ("slice_y_fname", PCH),
                ("num_of_slice_z", C.c_int), ("slice_z_indx", PI), ("slice_z_fname", PCH)]


class Snap(C.Structure):
    _fields_ = ([("siz_max_wrk", C.c_size_t), ("num_of_snap", C.c_int)]
                + [(n, PI) for n in ("i1", "j1", "k1", "ni", "nj", "nk", "di", "dj", "dk",
                                     "it1", "dit", "out_vel", "out_stress", "out_strain",
                                     "i1_to_glob", "j1_to_glob", "k1_to_glob")]
                + [("fname", PCH)])


class Mympi(C.Structure):
    _fields_ = [("nprocx", C.c_int), ("nprocy", C.c_int), ("myid", C.c_int)]


STRUCTS = {"fd_t": Fd, "gd_t": Gd, "gdcurv_metric_t": Metric, "md_t": Md,
           "src_t": Src, "bdrypml_auxvar_t": AuxVar, "bdry_block_t": BdryBlock,
           "bdry_t": Bdry, "wav_t": Wav, "iorecv_one_t": RecvOne, "iorecv_t": Recv,
           "ioline_t": Line, "ioslice_t": Slice, "iosnap_t": Snap, "fd_op_t": FdOp}


def _fp(a):
    return a.ctypes.data_as(PF)


def build_reference_structs(p):
    """Reference structs over the arrays of Problem `p` (shared memory: the
    drop-in writes the final state into p.wav, p.pml aux, and the receiver
    buffers returned in the keep dict)."""
    keep = {}
    fd = Fd()
    fd.num_rk_stages = 4
    fd.num_of_pairs = 8
    rk_a = np.array([0.5, 0.5, 1.0], np.float32)
    rk_b = np.array([1 / 6, 1 / 3, 1 / 3, 1 / 6], np.float32)
    keep["rk"] = (rk_a, rk_b)
    fd.rk_a, fd.rk_b = _fp(rk_a), _fp(rk_b)
    gd = Gd()
    for n, v in zip(["ni", "nj", "nk", "nx", "ny", "nz", "ni1", "ni2", "nj1", "nj2",
                     "nk1", "nk2"], p.grid_dims):
        setattr(gd, n, v)
    gd.type = 3
    gd.siz_iy = gd.siz_line = p.nx
    gd.siz_iz = gd.siz_slice = p.nx * p.ny
    gd.siz_icmp = gd.siz_volume = p.vol
    for n in ("x3d", "y3d", "z3d"):
        if n in p.coords:
            setattr(gd, n, _fp(p.coords[n]))
    met = Metric()
    for n, v in p.metric.items():
        setattr(met, n, _fp(v))
    md = Md()
    md.medium_type = p.medium_type
    md.rho = _fp(p.media["slw"])
    if "lambda" in p.media:
        md.lambda_ = _fp(p.media["lambda"])
        md.mu = _fp(p.media["mu"])
    for n in abi.ANISO_NAMES:
        if n in p.media:
            setattr(md, n, _fp(p.media[n]))
    if p.nmaxwell > 0:
        md.nmaxwell = p.nmaxwell
        md.visco_type = 2                     # CONST_VISCO_GMB
        md.wl = _fp(p.wl)
        yl = (PF * p.nmaxwell)(*[_fp(a) for a in p.Ylam])
        ym = (PF * p.nmaxwell)(*[_fp(a) for a in p.Ymu])
        keep["Y"] = (yl, ym)
        md.Ylam = C.cast(yl, PPF)
        md.Ymu = C.cast(ym, PPF)
    if p.graves_qs is not None:
        md.visco_type = 1                     # CONST_VISCO_GRAVES_QS
        md.visco_Qs_freq = float(p.graves_qs["freq"])
        md.Qs = _fp(p.graves_qs["Qs"])
    src = Src()
    s = p.src
    if s is not None and s["n"] > 0:
        src.total_number, src.max_nt, src.max_stage = s["n"], s["max_nt"], s["max_stage"]
        src.force_actived, src.moment_actived = s["force"], s["moment"]
        src.itype_spatial_ext, src.ext_half_npoint = s["spatial"], s["ext_half"]
        src.ext_func_coef = s["ext_coef"]
        src.is_surface_force_strict = s.get("surface_strict", 0)
        src.total_number_surface_force = s.get("n_surface_force", 0)
        for n in ("si", "sj", "sk", "it_begin", "it_end"):
            setattr(src, n, s[n].ctypes.data_as(PI))
        for n in ("si_inc", "sj_inc", "sk_inc", "Fx", "Fy", "Fz", "Mxx", "Myy", "Mzz",
                  "Mxz", "Myz", "Mxy", "Fx_rate", "Fy_rate", "Fz_rate"):
            if s.get(n) is not None:
                setattr(src, n, _fp(s[n]))
        if s.get("force_rate_indx") is not None:
            src.force_rate_indx = s["force_rate_indx"].ctypes.data_as(PI)
    if p.dd is not None:
        # distributed sources: the reference hands its time loop files of
        # per-step tables (forward/src_t.c:1640-1835); write them and open
        # them with the C library, as the reference's set-up leaves them
        import tempfile
        libc = C.CDLL(None)
        libc.fopen.restype = C.c_void_p
        libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
        d = p.dd
        src.dd_is_valid, src.dd_is_add_at_point = 1, 1
        src.dd_total_number, src.dd_max_nt = len(d["si"]), int(d["max_nt"])
        src.max_stage = 4
        for n in ("si", "sj", "sk"):
            setattr(src, "dd_" + n, d[n].ctypes.data_as(PI))
        for key, act, fp in (("vi", "dd_vi_actived", "fp_vi"), ("mij", "dd_mij_actived", "fp_mij")):
            if d.get(key) is None:
                continue
            tmp = tempfile.NamedTemporaryFile(suffix=".bin", delete=False)
            tmp.write(np.ascontiguousarray(d[key], np.float32).tobytes())
            tmp.close()
            keep.setdefault("dd_files", []).append(tmp.name)
            setattr(src, act, 1)
            setattr(src, fp, libc.fopen(tmp.name.encode(), b"rb"))
    bd = Bdry()
    bd.is_sides_free[2][1] = int(p.free_top)
    bd.is_enable_free = int(p.free_top)
    n2 = p.nx * p.ny * 9
    mats = [np.zeros(n2, np.float32) for _ in range(4)]
    keep["mats"] = mats
    bd.matVx2Vz2, bd.matVy2Vz2, bd.matF2Vz2, bd.matD = [_fp(m) for m in mats]
    for d in range(3):
        for sd in range(2):
            f = p.pml[d][sd]
            if f is None:
                continue
            bd.is_enable_pml = 1
            bd.is_sides_pml[d][sd] = 1
            b = [int(v) for v in f["box"]]
            bd.ni1[d][sd], bd.ni2[d][sd], bd.nj1[d][sd] = b[0], b[1], b[2]
            bd.nj2[d][sd], bd.nk1[d][sd], bd.nk2[d][sd] = b[3], b[4], b[5]
            bd.A[d][sd], bd.B[d][sd], bd.D[d][sd] = _fp(f["A"]), _fp(f["B"]), _fp(f["D"])
            bd.auxvar[d][sd].var = _fp(f["aux"])
    if p.ablexp is not None:
        bd.is_enable_ablexp = 1
        bd.ablexp_Ex, bd.ablexp_Ey, bd.ablexp_Ez = [_fp(p.ablexp[k]) for k in ("Ex", "Ey", "Ez")]
        blk = np.asarray(p.ablexp["blk"]).reshape(6, 7)
        for n in range(6):
            b = bd.bdry_blk[n]
            b.enable, b.ni1, b.ni2, b.nj1, b.nj2, b.nk1, b.nk2 = [int(v) for v in blk[n]]
    wav = Wav()
    wav.v5d = _fp(p.wav)
    wav.ncmp, wav.nlevel = p.ncmp, p.nlevel
    wav.nx, wav.ny, wav.nz = p.nx, p.ny, p.nz
    rc = Recv()
    r = p.recv
    if r is not None and r["n"] > 0:
        ones = (RecvOne * r["n"])()
        bufs = [np.zeros(r["ncmp"] * r["max_nt"], np.float32) for _ in range(r["n"])]
        for k in range(r["n"]):
            ones[k].di, ones[k].dj, ones[k].dk = [float(v) for v in r["dijk"][3 * k:3 * k + 3]]
            for c in range(8):
                ones[k].indx1d[c] = int(r["indx1d"][8 * k + c])
            ones[k].seismo = _fp(bufs[k])
        rc.total_number, rc.max_nt, rc.ncmp = r["n"], r["max_nt"], r["ncmp"]
        rc.recvone = ones
        keep["recv"] = (ones, bufs)
    ln = Line()
    l = p.line
    if l is not None and l["n"] > 0:
        nr = np.array([l["n"]], np.int32)
        iptr = l["iptr"].astype(np.int32)
        seis = np.zeros(l["n"] * p.ncmp * l["max_nt"], np.float32)
        pp_i = (PI * 1)(iptr.ctypes.data_as(PI))
        pp_s = (PF * 1)(_fp(seis))
        ln.num_of_lines, ln.max_nt, ln.ncmp = 1, l["max_nt"], p.ncmp
        ln.line_nr = nr.ctypes.data_as(PI)
        ln.recv_iptr = C.cast(pp_i, PPI)
        ln.recv_seismo = C.cast(pp_s, PPF)
        keep["line"] = (nr, iptr, seis, pp_i, pp_s)
    sl, sn, mp = Slice(), Snap(), Mympi()
    structs = dict(fd=fd, gd=gd, metric=met, md=md, src=src, bdry=bd, wav=wav,
                   mympi=mp, iorecv=rc, ioline=ln, ioslice=sl, iosnap=sn)
    return structs, keep
