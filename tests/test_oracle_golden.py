"""The C oracle against the reference's own outputs (golden fixtures).

The fixtures under tests/golden/ were produced by the CGFD3D reference CPU
build (oracle/Makefile, tests/golden/make_golden.py).  The oracle restates the
reference's float arithmetic in the same order, so the comparison is exact.
"""

import os

import numpy as np
import pytest

import oracle
from cgfd3d_gb300 import problem as P
from conftest import GOLDEN, GOLDEN_CASES


@pytest.mark.parametrize("case", GOLDEN_CASES)
@pytest.mark.parametrize("nthreads", [1, 3])
def test_oracle_matches_reference_bitwise(case, nthreads):
    p, exp = P.from_golden(os.path.join(GOLDEN, case + ".npz"))
    mats = oracle.allstep(p, oracle.TIMG_ZERO, nthreads, want_mats=True)
    np.testing.assert_array_equal(p.level(p.final_level()), exp["wav"])
    for key, val in exp.items():
        if key.startswith("pml."):
            d, s = int(key[4]), int(key[6])
            np.testing.assert_array_equal(p.pml_final(d, s), val)
    if "recv" in exp:
        np.testing.assert_array_equal(p.recv["seismo"], exp["recv"])
    if "line" in exp:
        np.testing.assert_array_equal(p.line["seismo"], exp["line"])
    if mats is not None:
        for m, n in zip(mats, ["matVx2Vz2", "matVy2Vz2", "matF2Vz2"]):
            np.testing.assert_array_equal(m, exp[n])


def test_mirror_variant_differs_from_reference():
    """The intended traction mirror is NOT what the reference computes."""
    p, exp = P.from_golden(os.path.join(GOLDEN, "iso_flat_explosion.npz"))
    oracle.allstep(p, oracle.TIMG_MIRROR, 2)
    got = p.level(p.final_level())
    assert np.abs(got - exp["wav"]).max() > 1e-3 * np.abs(exp["wav"]).max()


def test_planted_error_is_detected():
    """A one-ulp change of one input coefficient changes the result."""
    p, exp = P.from_golden(os.path.join(GOLDEN, "iso_box_pml6.npz"))
    q = (p.ni1 + p.ni // 2) + (p.nj1 + p.nj // 2) * p.nx + \
        (p.nk1 + p.nk // 2) * p.nx * p.ny
    p.media["mu"] = p.media["mu"].copy()
    p.media["mu"][q] = np.nextafter(p.media["mu"][q], np.float32(np.inf))
    oracle.allstep(p, oracle.TIMG_ZERO, 1)
    assert not np.array_equal(p.level(p.final_level()), exp["wav"])


@pytest.mark.parametrize("case", [c for c in GOLDEN_CASES
                                  if c.startswith(("vti", "visco", "iso_topo"))])
def test_surface_matrices_match_reference(case):
    """Free-surface conversion matrices (and the visco rotation matrix)."""
    p, exp = P.from_golden(os.path.join(GOLDEN, case + ".npz"))
    got = oracle.surface_matrices(p)
    for k, v in got.items():
        np.testing.assert_array_equal(v, exp[k], err_msg=k)


def test_visco_attenuation_is_exercised():
    """Zeroing the relaxation frequencies changes the visco result, so the
    fixture checks the memory-variable terms."""
    p, exp = P.from_golden(os.path.join(GOLDEN, "visco_topo_noise.npz"))
    p.wl = np.zeros_like(p.wl)
    oracle.allstep(p, oracle.TIMG_ZERO, 2)
    got = p.level(p.final_level())
    assert np.abs(got - exp["wav"]).max() > 1e-6 * np.abs(exp["wav"]).max()


def test_vti_differs_from_iso_formulas():
    """A planted error in one VTI constant (c13 scaled by 1.0001) is
    detected by the fixture."""
    p, exp = P.from_golden(os.path.join(GOLDEN, "vti_topo_noise.npz"))
    p.media["c13"] = p.media["c13"] * np.float32(1.0001)
    oracle.allstep(p, oracle.TIMG_ZERO, 2)
    assert not np.array_equal(p.level(p.final_level()), exp["wav"])


def test_surface_force_layers_are_exercised():
    """Without its surface layers (traction image, vlow) the point force at
    the flat surface would inject nothing: dropping them changes the run."""
    p, exp = P.from_golden(os.path.join(GOLDEN, "iso_surface_point_force.npz"))
    p.src = dict(p.src, Fz_rate=np.zeros_like(p.src["Fz_rate"]),
                 Fz=np.zeros_like(p.src["Fz"]))
    oracle.allstep(p, oracle.TIMG_ZERO, 2)
    assert not np.array_equal(p.level(p.final_level()), exp["wav"])
    assert np.abs(exp["wav"]).max() > 0


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_metric_calc_matches_reference(case):
    """The restated metric calculation (forward/gd_t.c:190-402) gives the
    reference's metrics, ghosts included, bit for bit."""
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    g = [int(v) for v in d["gd.dims"]]
    nx, ny, nz = g[3], g[4], g[5]
    got = oracle.metric_calc(nx, ny, nz, *g[6:12], d["gd.x3d"], d["gd.y3d"], d["gd.z3d"])
    names = ["jac", "xi_x", "xi_y", "xi_z", "eta_x", "eta_y", "eta_z",
             "zeta_x", "zeta_y", "zeta_z"]
    for c, n in enumerate(names):
        np.testing.assert_array_equal(got[c], d["metric." + n], err_msg=n)
