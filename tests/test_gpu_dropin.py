"""The drop-in entry point, called the way the reference's main calls it.

drv_rk_curv_col_allstep(fd, gd, metric, md, src, bdry, wav, mympi, iorecv,
ioline, ioslice, iosnap, dt, nt_total, t0, ...) receives the reference's own
structs (restated layouts, checked against the reference headers by
test_ref_abi.py), runs the time loop on the GPU and must leave in them what
the reference leaves: the final wavefield and PML state in level 0/3, the
free-surface matrices in bdry, and the seismograms in iorecv/ioline.  The
expected values are the reference's own outputs (golden fixtures).
"""

import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, GOLDEN_CASES
from helpers import assert_parity

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_dropin_matches_reference(case):
    from cgfd3d_gb300 import problem, refabi, solver
    p, exp = problem.from_golden(os.path.join(GOLDEN, case + ".npz"))
    st, keep = refabi.build_reference_structs(p)
    solver.drv_rk_curv_col_allstep_structs(st, p.dt, p.nt_total, p.t0,
                                           qc_check_nan_num_of_step=4)
    assert_parity(p.level(p.final_level()), exp["wav"], case + " wavefield")
    for key, val in exp.items():
        if key.startswith("pml."):
            d, s = int(key[4]), int(key[6])
            assert_parity(p.pml_final(d, s), val, case + " " + key)
    if "recv" in exp:
        got = np.concatenate(keep["recv"][1])
        assert_parity(got, exp["recv"], case + " receivers")
    if "line" in exp:
        assert_parity(keep["line"][2], exp["line"], case + " lines")
    if "matVx2Vz2" in exp:
        names = ["matVx2Vz2", "matVy2Vz2", "matF2Vz2"]
        if p.nmaxwell > 0:
            names.append("matD")
        for m, n in zip(keep["mats"], names):
            # the free-surface matrices are computed once: tighter bound
            np.testing.assert_allclose(m, exp[n], rtol=2e-5,
                                       atol=2e-6 * np.abs(exp[n]).max())


def test_peak_motion_maps_match_oracle():
    from cgfd3d_gb300 import problem, solver
    p, _ = problem.from_golden(os.path.join(GOLDEN, "iso_flat_explosion.npz"))
    q = p.copy()
    with solver.Solver(p) as s:
        s.run(p.nt_total)
        pg = s.fetch_pg().ravel()
    ref = oracle.allstep(q, oracle.TIMG_ZERO, 4, want_pg=True)
    for m in range(15):
        n = p.nx * p.ny
        assert_parity(pg[m * n:(m + 1) * n], ref[m * n:(m + 1) * n], "PG map %d" % m)
