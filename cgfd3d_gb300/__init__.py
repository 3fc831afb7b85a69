"""GB300-native time stepping for CGFD3D (collocated curvilinear grid,
MacCormack DRP operators, RK4, traction-image free surface, ADE CFS-PML).

    from cgfd3d_gb300 import problem, solver
    p, _ = problem.from_golden("tests/golden/iso_topo_noise.npz")
    solver.drv_rk_curv_col_allstep(p)
"""

from . import abi, problem  # noqa: F401

__all__ = ["abi", "problem", "solver", "models"]
