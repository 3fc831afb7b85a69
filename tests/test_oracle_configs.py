"""The oracle pinned to the reference at the flat configuration's stated
size and step count (CPU only).

The reference's own CPU build ran the flat configuration -- 100 x 100 x 60,
CFS-PML 10, explosive source 2 km deep, 20 line receivers and 20 stations,
number_of_time_steps 500, i.e. 501 executed steps -- and its outputs are the
fixture tests/golden/configs/c0_flat_explosion_501.npz.  The C oracle must
reproduce them bit for bit after all 501 steps: line and station
seismograms and the four kept planes of the final state.  The
double-precision oracle must stay within the single-precision rounding
error of it (checked loosely; the GPU test reports the figures).
"""

import os

import numpy as np

import oracle
from helpers import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))
C0_FIXTURE = os.path.join(HERE, "golden", "configs", "c0_flat_explosion_501.npz")


def test_oracle_bit_identical_after_501_steps():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden", "configs"))
    from make_config_golden import planes_of
    from cgfd3d_gb300 import problem
    p, exp = problem.from_golden(C0_FIXTURE)
    assert p.nt_total == 501
    oracle.allstep(p, oracle.TIMG_ZERO, os.cpu_count() or 4)
    lev = p.final_level()
    got = planes_of(p.level(lev), p.ncmp, p.nx, p.ny, p.nz)
    assert sorted(got) == sorted(exp["planes"])
    for k in got:
        assert np.array_equal(got[k], exp["planes"][k]), k
    assert np.array_equal(p.line["seismo"], exp["line"])
    assert np.array_equal(p.recv["seismo"], exp["recv"])


def test_double_oracle_tracks_single_on_a_golden_case():
    """The double-precision build runs the same scheme: on a golden case its
    result differs from the single-precision one by rounding only."""
    from cgfd3d_gb300 import problem
    p, exp = problem.from_golden(os.path.join(HERE, "golden", "iso_topo_noise.npz"))
    w = oracle.allstep64(p, oracle.TIMG_ZERO, 4)
    lev = p.final_level()
    assert w.level(lev).dtype == np.float64
    r = rel_l2(exp["wav"], w.level(lev))
    assert 0.0 < r < 1e-5, r
    assert rel_l2(exp["recv"], w.recv["seismo"]) < 1e-5
