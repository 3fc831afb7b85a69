"""Grid metrics computed on the device (cgfd_metric_calc and the solver's
coordinates-only path) against the reference's own metrics.

The reference computes jac, xi_*, eta_*, zeta_* from the node coordinates
with a centred 7-point operator and cross products and mirrors the ghost
layers (forward/gd_t.c:190-402); the golden fixtures hold its coordinates
and its metrics.  Device float arithmetic (fused multiply-adds) differs in
rounding only: every component within 2e-5 of its peak, relative L2 1e-5.
"""

import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES
from helpers import assert_parity

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_device_metrics_match_reference(case):
    from cgfd3d_gb300 import abi, solver
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    got = solver.metric_calc(d["gd.dims"], d["gd.x3d"], d["gd.y3d"], d["gd.z3d"])
    for n in abi.METRIC_NAMES:
        ref = d["metric." + n]
        # scale: the peak of the whole metric vector (xi, eta or zeta), since
        # some components are analytically zero on Cartesian grids and hold
        # rounding residue only
        group = [m for m in abi.METRIC_NAMES if m.split("_")[0] == n.split("_")[0]]
        peak = max(float(np.abs(d["metric." + m]).max()) for m in group)
        np.testing.assert_allclose(got[n], ref, rtol=0, atol=2e-5 * peak, err_msg=n)


def test_solver_from_coordinates_equals_given_metrics():
    """A problem given only its grid coordinates (metrics computed in the
    solver) runs like the same problem given the reference's metrics."""
    from cgfd3d_gb300 import problem, solver
    p, exp = problem.from_golden(os.path.join(GOLDEN, "iso_topo_noise.npz"))
    q = p.copy()
    q.metric = {}
    solver.drv_rk_curv_col_allstep(q)
    lev = q.final_level()
    assert_parity(q.level(lev), exp["wav"], "metrics from coordinates")
    if "recv" in exp:
        assert_parity(q.recv["seismo"], exp["recv"], "receivers")
