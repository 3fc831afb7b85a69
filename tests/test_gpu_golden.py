"""GPU parity against the reference's own outputs and against the oracle.

Calls the CUDA library through its C ABI (ctypes) on the golden fixtures and
compares every output with tolerances rel-L2 <= 1e-5 and
max-abs <= 1e-4 * peak (float32 arithmetic with fused multiply-adds on the
GPU versus the reference's separate multiply and add).
"""

import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES
from helpers import assert_parity

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gpu_matches_reference(case):
    from cgfd3d_gb300 import problem, solver
    p, exp = problem.from_golden(os.path.join(GOLDEN, case + ".npz"))
    solver.drv_rk_curv_col_allstep(p)
    assert_parity(p.level(p.final_level()), exp["wav"], case + " wavefield")
    for key, val in exp.items():
        if key.startswith("pml."):
            d, s = int(key[4]), int(key[6])
            assert_parity(p.pml_final(d, s), val, case + " " + key)
    if "recv" in exp:
        assert_parity(p.recv["seismo"], exp["recv"], case + " receivers")
    if "line" in exp:
        assert_parity(p.line["seismo"], exp["line"], case + " lines")


def test_gpu_stepwise_equals_oneshot():
    """run(3)+run(rest) through a resident solver equals the one-shot call."""
    from cgfd3d_gb300 import problem, solver
    p1, _ = problem.from_golden(os.path.join(GOLDEN, "iso_topo_noise.npz"))
    p2 = p1.copy()
    solver.drv_rk_curv_col_allstep(p1)
    with solver.Solver(p2) as s:
        s.run(3)
        s.run(p2.nt_total - 3)
        s.fetch()
    np.testing.assert_array_equal(p1.level(p1.final_level()),
                                  p2.level(p2.final_level()))
