"""A stage-kernel wait that runs out, on the GPU, without a fault.

The stage kernel bounds every mbarrier wait.  Here the first CTA of each
stage launch leaves out the bulk copy of one wavefield plane (the test hook
of cgfd_solver_set_wait_test), so its consumers wait on a barrier that
nothing completes.  With a short poll limit the wait runs out, the CTA
stops (the producer drains the copies it did issue), and the run must
return the device error within a second -- not after one half-second
timeout per remaining wait.  A fresh solver on the same device then runs
normally and meets the parity bar against the oracle.
"""

import os
import time

import pytest

import oracle
from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _model():
    from cgfd3d_gb300 import models
    return models.topo_model(ni=96, nj=80, nk=48, steps=4, dt=0.005, nrecv=9)


def test_wait_runs_out_and_reports():
    from cgfd3d_gb300 import _lib, solver
    p = _model()
    with solver.Solver(p) as s:
        s.set_wait_test(1 << 13, skip_plane=7)
        t0 = time.perf_counter()
        with pytest.raises(_lib.CgfdError) as ei:
            s.run(2)
        dt = time.perf_counter() - t0
    assert "device wait timed out" in str(ei.value)
    assert dt < 1.0, dt


def test_device_usable_after_timeout():
    from cgfd3d_gb300 import _lib, solver
    p = _model()
    with solver.Solver(p.copy()) as s:
        s.set_wait_test(1 << 13, skip_plane=5)
        with pytest.raises(_lib.CgfdError):
            s.run(1)
    q, r = p.copy(), p.copy()
    solver.drv_rk_curv_col_allstep(q)
    oracle.allstep(r, oracle.TIMG_ZERO, os.cpu_count() or 4)
    lev = q.final_level()
    assert_parity(q.level(lev), r.level(lev), "after a timed-out run")


def test_short_limit_alone_does_not_fire():
    """A short poll limit with every copy issued completes normally."""
    from cgfd3d_gb300 import solver
    p = _model()
    with solver.Solver(p) as s:
        s.set_wait_test(1 << 16, skip_plane=-1)
        s.run(p.nt_total)
