"""The reference solver links with its time loop and its media
discretisation (layered and binary-volume models) replaced by the GPU
library.

Where the reference tree is present, oracle/Makefile builds the reference's
main with the drop-in adapter compiled against the reference's own headers in
place of forward/drv_rk_curv_col.o, linked to libcgfd3d_gpu.  The binary must
link, define drv_rk_curv_col_allstep from the adapter and import the
library's entry points.
"""

import os
import subprocess

import pytest

from helpers import ref_tree

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = ref_tree() or ""


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "forward")),
                    reason="reference tree not present")
def test_reference_main_links_against_gpu_library():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "-j8",
                    "REF=" + REF, "_ref/cgfd3d_gpu_dropin"], check=True,
                   capture_output=True)
    exe = os.path.join(REPO, "oracle", "_ref", "cgfd3d_gpu_dropin")
    syms = subprocess.run(["nm", exe], check=True, capture_output=True,
                          text=True).stdout
    assert " T drv_rk_curv_col_allstep" in syms
    assert " U cgfd_solver_create" in syms
    assert " T sv_curv_col_el_iso_onestage" in syms  # the rest of the reference
    # the layered-media discretisation: main's call is wrapped by the adapter
    for fn in ("media_layer2model_el_iso", "media_layer2model_el_vti", "media_layer2model_el_aniso",
               "media_grid2model_el_iso", "media_grid2model_el_vti", "media_grid2model_el_aniso",
               "media_bin2model_el_iso",
               "media_bin2model_vis_iso"):
        assert " T __wrap_" + fn in syms
    for fn in ("cgfd_media_layer_el_iso", "cgfd_media_layer_el_vti", "cgfd_media_grid_el_iso",
               "cgfd_media_grid_el_vti",
               "cgfd_media_bin_el_iso", "cgfd_media_bin_vis_iso"):
        assert " U " + fn in syms
