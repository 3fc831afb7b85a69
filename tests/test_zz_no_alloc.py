"""The finiteness check that allocates nothing, against the solver's check.

cgfd_check_finite_noalloc() serves callers that cannot call cudaMalloc (their
device memory belongs to another framework's pool or sits under a hard cap,
or the check runs between launches of a time loop where an allocation would
synchronise the device).  It keeps its scratch in a file-scope device array
shared by every call.  This test feeds it the same wavefield the solver's own
cgfd_solver_check_finite() examines and requires the same verdict on two
calls in a row, in both orders, so that a result left in the shared scratch
by the previous call can never leak into the next one.  The file sorts last
so that a run stopping at the first failure has run every other test.
"""

import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _solver_verdict(problem):
    from cgfd3d_gb300 import _lib, solver
    with solver.Solver(problem) as s:
        try:
            s.check_finite()
            return 0
        except _lib.CgfdError as e:
            assert e.code == 4, e
            return 1


def _noalloc_verdict(level0):
    import torch
    from cgfd3d_gb300 import _lib
    dev = torch.from_numpy(level0).to("cuda")
    torch.cuda.synchronize()
    out = C.c_int(-1)
    _lib.check(_lib.lib().cgfd_check_finite_noalloc(
        C.c_void_p(dev.data_ptr()), dev.numel(), C.byref(out)))
    return out.value


def _pair():
    from cgfd3d_gb300 import problem
    good, _ = problem.from_golden(os.path.join(GOLDEN, "iso_box_pml6.npz"))
    bad = good.copy()
    lev = bad.level(0).reshape(bad.ncmp, bad.nz, bad.ny, bad.nx)
    lev[5, bad.nk1 + 2, bad.nj1 + 3, bad.ni1 + 4] = np.nan
    return good, bad


def test_noalloc_matches_solver_check_two_calls():
    good, bad = _pair()
    for order in ((bad, good), (good, bad)):
        for prob in order:
            assert _noalloc_verdict(prob.level(0)) == _solver_verdict(prob)
    assert _noalloc_verdict(bad.level(0)) == 1
    assert _noalloc_verdict(good.level(0)) == 0


def test_noalloc_rejects_oversize_input():
    import torch
    from cgfd3d_gb300 import _lib
    dev = torch.zeros(16, device="cuda")
    out = C.c_int(-1)
    rc = _lib.lib().cgfd_check_finite_noalloc(
        C.c_void_p(dev.data_ptr()), 65536 * 256 * 64 + 1, C.byref(out))
    assert rc == 1
    assert b"exceed the maximum" in _lib.lib().cgfd_last_error()
