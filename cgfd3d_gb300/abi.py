"""ctypes mirror of include/cgfd3d_gpu.h (the flat C ABI).

The layout of every structure here must match the C header field by field;
tests/test_abi.py checks sizes and offsets against a compiled probe.
"""

import ctypes as C

CGFD_ABI_VERSION = 6
CGFD_MEDIUM_ELASTIC_ISO = 2
CGFD_MEDIUM_ELASTIC_VTI = 3
CGFD_MEDIUM_ELASTIC_ANISO = 4
ANISO_NAMES = ["c11", "c12", "c13", "c14", "c15", "c16", "c22", "c23", "c24", "c25",
               "c26", "c33", "c34", "c35", "c36", "c44", "c45", "c46", "c55", "c56", "c66"]
ANISO_EXTRA = [n for n in ANISO_NAMES if n not in ("c11", "c13", "c33", "c55", "c66")]
CGFD_MEDIUM_VISCOELASTIC_ISO = 5
CGFD_MAX_MAXWELL = 8
CGFD_SRC_POINT = 1
CGFD_SRC_GAUSSIAN = 2

CGFD_OK = 0
CGFD_EINVAL = 1
CGFD_ECUDA = 2
CGFD_ENOMEM = 3
CGFD_ENONFINITE = 4

PF = C.POINTER(C.c_float)
PI = C.POINTER(C.c_int)


class PmlFace(C.Structure):
    _fields_ = [
        ("enabled", C.c_int),
        ("ni1", C.c_int), ("ni2", C.c_int), ("nj1", C.c_int),
        ("nj2", C.c_int), ("nk1", C.c_int), ("nk2", C.c_int),
        ("A", PF), ("B", PF), ("D", PF),
        ("aux", PF),
    ]


_GRID = ["ni", "nj", "nk", "nx", "ny", "nz", "ni1", "ni2", "nj1", "nj2",
         "nk1", "nk2"]
METRIC_NAMES = ["jac", "xi_x", "xi_y", "xi_z", "eta_x", "eta_y", "eta_z",
                "zeta_x", "zeta_y", "zeta_z"]


class Problem(C.Structure):
    _fields_ = (
        [(n, C.c_int) for n in _GRID]
        + [(n, PF) for n in METRIC_NAMES]
        + [("medium_type", C.c_int),
           ("slw", PF), ("lambda_", PF), ("mu", PF),
           ("c11", PF), ("c13", PF), ("c33", PF), ("c55", PF), ("c66", PF),
           ("nmaxwell", C.c_int),
           ("wl", PF),
           ("Ylam", PF * CGFD_MAX_MAXWELL), ("Ymu", PF * CGFD_MAX_MAXWELL),
           ("free_top", C.c_int),
           ("pml", (PmlFace * 2) * 3),
           ("src_n", C.c_int), ("src_max_nt", C.c_int), ("src_max_stage", C.c_int),
           ("src_force", C.c_int), ("src_moment", C.c_int),
           ("src_spatial", C.c_int), ("src_ext_half", C.c_int),
           ("src_ext_coef", C.c_float),
           ("src_surface_strict", C.c_int), ("src_n_surface_force", C.c_int),
           ("src_si", PI), ("src_sj", PI), ("src_sk", PI),
           ("src_it_begin", PI), ("src_it_end", PI),
           ("src_si_inc", PF), ("src_sj_inc", PF), ("src_sk_inc", PF),
           ("Fx", PF), ("Fy", PF), ("Fz", PF),
           ("Mxx", PF), ("Myy", PF), ("Mzz", PF), ("Mxz", PF), ("Myz", PF),
           ("Mxy", PF),
           ("recv_n", C.c_int), ("recv_max_nt", C.c_int), ("recv_ncmp", C.c_int),
           ("recv_dijk", PF), ("recv_indx1d", PI), ("recv_seismo", PF),
           ("line_n", C.c_int), ("line_max_nt", C.c_int),
           ("line_iptr", PI), ("line_seismo", PF),
           ("ncmp", C.c_int), ("nlevel", C.c_int),
           ("wav", PF),
           ("dt", C.c_float), ("t0", C.c_float),
           ("nt_total", C.c_int),
           ("x3d", PF), ("y3d", PF), ("z3d", PF),
           ("src_force_rate_indx", PI),
           ("Fx_rate", PF), ("Fy_rate", PF), ("Fz_rate", PF),
           ("graves_qs", C.c_int), ("qs_freq", C.c_float), ("Qs", PF),
           ("ablexp", C.c_int),
           ("ablexp_Ex", PF), ("ablexp_Ey", PF), ("ablexp_Ez", PF),
           ("ablexp_blk", (C.c_int * 7) * 6)]
        + [(n, PF) for n in ANISO_EXTRA]
        + [("dd_n", C.c_int), ("dd_max_nt", C.c_int),
           ("dd_si", PI), ("dd_sj", PI), ("dd_sk", PI), ("dd_vi", PF), ("dd_mij", PF)]
    )


class Box(C.Structure):
    """cgfd_box_t: components c1..c2, points (i1 + a*di, j1 + b*dj, k1 + c*dk)
    in padded-array indices."""
    _fields_ = [(n, C.c_int) for n in
                ("c1", "c2", "i1", "ni", "di", "j1", "nj", "dj", "k1", "nk", "dk")]


def field_offsets(struct):
    return {name: getattr(struct, name).offset for name, _ in struct._fields_}
