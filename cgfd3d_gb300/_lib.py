"""Loader of the in-tree CUDA library (cgfd3d_gb300/_build/libcgfd3d_gpu.so).

The library is the only compute path: there is no CPU fallback, so a missing
or unloadable library raises instead of degrading.
"""

import ctypes as C
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcgfd3d_gpu.so")

_lib = None


class CgfdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("cgfd error %d: %s" % (code, msg))
        self.code = code


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "CUDA library %s is missing: run `python -c \"import "
            "__graft_entry__ as g; g.build()\"` (needs nvcc)" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    L.cgfd_last_error.restype = C.c_char_p
    L.cgfd_abi_version.restype = C.c_int
    L.cgfd_solver_create.argtypes = [vp, C.POINTER(vp)]
    L.cgfd_solver_run.argtypes = [vp, C.c_int]
    L.cgfd_solver_fetch.argtypes = [vp]
    L.cgfd_solver_step.argtypes = [vp]
    L.cgfd_solver_check_finite.argtypes = [vp]
    L.cgfd_solver_kernel_times.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_int)]
    L.cgfd_solver_set_timing.argtypes = [vp, C.c_int]
    L.cgfd_solver_set_wait_test.argtypes = [vp, C.c_int, C.c_int]
    L.cgfd_solver_transfer_bytes.argtypes = [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    L.cgfd_solver_fetch_pg.argtypes = [vp, vp]
    L.cgfd_solver_fetch_state.argtypes = [vp, vp]
    L.cgfd_box_floats.argtypes = [vp, C.c_int]
    L.cgfd_box_floats.restype = C.c_size_t
    L.cgfd_solver_pack_boxes.argtypes = [vp, vp, C.c_int, vp]
    L.cgfd_solver_fetch_boxes.argtypes = [vp, vp, C.c_int, vp]
    L.cgfd_solver_run_async.argtypes = [vp, C.c_int]
    L.cgfd_solver_pack_boxes_async.argtypes = [vp, vp, C.c_int, C.c_int]
    L.cgfd_solver_collect_boxes.argtypes = [vp, C.c_int, vp, vp]
    L.cgfd_solver_fetch_surface_matrices.argtypes = [vp, vp, vp, vp]
    L.cgfd_solver_fetch_surface_rotation.argtypes = [vp, vp]
    L.cgfd_solver_destroy.argtypes = [vp]
    L.cgfd_solver_destroy.restype = None
    L.cgfd_allstep.argtypes = [vp]
    L.cgfd_device_bytes.argtypes = [vp]
    L.cgfd_device_bytes.restype = C.c_size_t
    L.cgfd_metric_calc.argtypes = [C.c_int] * 9 + [vp] * 4
    L.cgfd_locator_create.argtypes = [C.c_int] * 3 + [vp] * 3 + [C.POINTER(vp)]
    L.cgfd_locator_locate.argtypes = [vp, C.c_int] + [vp] * 8
    L.cgfd_locator_destroy.argtypes = [vp]
    L.cgfd_media_layer_el_iso.argtypes = ([C.c_int] * 3 + [C.c_float] * 4 + [vp] +
                                          [C.c_int] * 3 + [vp] * 3 + [C.c_char_p] + [vp] * 3)
    L.cgfd_media_layer_pow_ok.argtypes = [C.c_int, vp, C.c_size_t]
    L.cgfd_media_grid_el_vti.argtypes = ([C.c_int] * 3 + [vp] + [C.c_int] * 2 + [C.c_float] * 4 +
                                         [vp] + [C.c_int] * 3 + [vp] * 3 + [C.c_char_p] +
                                         [vp] * 6)
    L.cgfd_media_grid_el_iso.argtypes = ([C.c_int] * 2 + [vp] + [C.c_int] * 2 + [C.c_float] * 4 +
                                         [vp] + [C.c_int] * 3 + [vp] * 3 + [C.c_char_p] +
                                         [vp] * 3)
    L.cgfd_media_layer_el_vti.argtypes = ([C.c_int] * 4 + [C.c_float] * 4 + [vp] +
                                          [C.c_int] * 3 + [vp] * 3 + [C.c_char_p] + [vp] * 6)
    L.cgfd_media_bin_el_iso.argtypes = ([vp] + [C.c_float] * 4 + [vp] * 3 + [C.c_int] * 3 +
                                        [vp] * 6)
    L.cgfd_media_bin_vis_iso.argtypes = ([vp] + [C.c_float] * 4 + [vp] * 2 + [C.c_int] * 3 +
                                         [vp] * 5)
    L.cgfd_media_bin_crop.argtypes = [vp] + [C.c_float] * 4 + [C.c_int] * 3 + [vp, vp]
    L.cgfd_media_bin_el_iso_box.argtypes = ([vp, vp] + [C.c_float] * 4 + [vp] * 3 +
                                            [C.c_int] * 3 + [vp] * 6)
    L.cgfd_media_bin_vis_iso_box.argtypes = ([vp, vp] + [C.c_float] * 4 + [vp] * 2 +
                                             [C.c_int] * 3 + [vp] * 5)
    L.cgfd_locator_destroy.restype = None
    L.cgfd_batch_create.argtypes = [vp, C.c_int, C.c_int, C.POINTER(vp)]
    L.cgfd_batch_run.argtypes = [vp, C.c_int]
    L.cgfd_batch_fetch_seismograms.argtypes = [vp]
    L.cgfd_solver_fetch_seismograms.argtypes = [vp]
    L.cgfd_batch_times.argtypes = [vp, C.POINTER(C.c_float), C.POINTER(C.c_int)]
    L.cgfd_batch_fetch.argtypes = [vp]
    L.cgfd_batch_reset.argtypes = [vp]
    L.cgfd_batch_set_kchunk.argtypes = [vp, C.c_int]
    L.cgfd_batch_autotune.argtypes = [vp, C.POINTER(C.c_int), C.c_int, C.c_int,
                                      C.POINTER(C.c_float), C.POINTER(C.c_int)]
    L.cgfd_batch_set_schedule.argtypes = [vp, C.c_int]
    L.cgfd_batch_schedule.argtypes = [vp]
    L.cgfd_batch_autotune_schedule.argtypes = [vp, C.POINTER(C.c_int), C.c_int, C.c_int,
                                               C.POINTER(C.c_float), C.POINTER(C.c_int),
                                               C.POINTER(C.c_int)]
    L.cgfd_batch_shot.argtypes = [vp, C.c_int]
    L.cgfd_batch_shot.restype = vp
    L.cgfd_batch_destroy.argtypes = [vp]
    L.cgfd_batch_destroy.restype = None
    L.cgfd_check_finite_noalloc.argtypes = [C.c_void_p, C.c_size_t, C.POINTER(C.c_int)]
    L.cgfd_check_finite_noalloc.restype = C.c_int
    if L.cgfd_abi_version() != abi.CGFD_ABI_VERSION:
        raise ImportError("libcgfd3d_gpu ABI version mismatch")
    _lib = L
    return L


DROPIN_PATH = os.path.join(HERE, "_build", "libcgfd3d_dropin.so")
_dropin = None


def dropin():
    """The drop-in library exporting drv_rk_curv_col_allstep."""
    global _dropin
    if _dropin is None:
        lib()
        if not os.path.exists(DROPIN_PATH):
            raise ImportError("drop-in library %s is missing: run build()" % DROPIN_PATH)
        D = C.CDLL(DROPIN_PATH)
        D.drv_rk_curv_col_allstep.restype = None
        D.drv_rk_curv_col_allstep.argtypes = [C.c_void_p] * 12 + [
            C.c_float, C.c_int, C.c_float, C.c_char_p, C.c_char_p, C.c_int,
            C.c_int, C.c_int]
        _dropin = D
    return _dropin


def check(rc):
    if rc != 0:
        raise CgfdError(rc, lib().cgfd_last_error().decode())
    return rc
