"""Distributed (dd) sources at grid points on the device against the
oracle's restatement of sv_curv_col_el_rhs_srcdd: points in the interior, in
the PML, at the free surface and several in one column, together with an
ordinary moment source; the tables stop before the last steps."""

import os
import sys

import numpy as np
import pytest

from helpers import assert_parity

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def _problem(kind, seed):
    from cgfd3d_gb300 import models
    if kind == "iso":
        p = models.topo_model(ni=60, nj=52, nk=40, steps=12, dt=0.005, nrecv=9)
    else:
        p = models.topo_media_model(kind, ni=60, nj=52, nk=40, steps=12, dt=0.005, nrecv=9)
    rng = np.random.default_rng(seed)
    n = 40
    ijk = np.stack([rng.integers(p.ni1, p.ni2 + 1, n), rng.integers(p.nj1, p.nj2 + 1, n),
                    rng.integers(p.nk1, p.nk2 + 1, n)], 1)
    ijk[:5, 2] = p.nk2                        # at the free surface
    ijk[5:9, 0], ijk[5:9, 1] = 30, 26         # one column, several planes
    ijk[9:12, 0] = p.ni1 + 1                  # in the x PML
    max_nt = 9
    vi = (rng.standard_normal((max_nt, 4, n, 3)) * 1e12).astype(np.float32)
    mij = (rng.standard_normal((max_nt, 4, n, 6)) * 1e14).astype(np.float32)
    models.add_dd_sources(p, ijk, vi=vi, mij=mij)
    return p


@pytest.mark.parametrize("kind", ["iso", "vti"])
def test_dd_sources_match_oracle(kind):
    from cgfd3d_gb300 import solver
    p = _problem(kind, 3)
    q = p.copy()
    solver.drv_rk_curv_col_allstep(p)
    oracle.allstep(q, oracle.TIMG_ZERO, os.cpu_count() or 4)
    lev = p.final_level()
    assert_parity(p.level(lev), q.level(lev), kind + " wavefield with dd sources")
    assert_parity(p.recv["seismo"], q.recv["seismo"], kind + " receivers")
    assert np.abs(q.level(lev)).max() > 0


def test_dd_sources_change_the_result_and_stop():
    """The dd tables matter, and nothing of them is used past max_nt."""
    from cgfd3d_gb300 import solver
    p = _problem("iso", 4)
    base = p.copy()
    base.dd = None
    late = p.copy()
    late.dd = dict(p.dd, vi=p.dd["vi"].copy(), mij=p.dd["mij"].copy())
    solver.drv_rk_curv_col_allstep(p)
    solver.drv_rk_curv_col_allstep(base)
    lev = p.final_level()
    assert np.abs(p.level(lev) - base.level(lev)).max() > 0
    # values beyond max_nt rows do not exist; rows at it >= max_nt are never read:
    # a table two steps longer whose extra rows are huge gives the same result
    # when max_nt stays 9
    n = len(p.dd["si"])
    vi = np.concatenate([late.dd["vi"].reshape(9, 4, n, 3),
                         np.full((2, 4, n, 3), 1e30, np.float32)])
    mij = np.concatenate([late.dd["mij"].reshape(9, 4, n, 6),
                          np.full((2, 4, n, 6), 1e30, np.float32)])
    late.dd = dict(late.dd, vi=vi.ravel(), mij=mij.ravel(), max_nt=9)
    solver.drv_rk_curv_col_allstep(late)
    np.testing.assert_array_equal(late.level(lev), p.level(lev))
