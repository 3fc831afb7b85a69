"""Point location (stations and sources given by coordinates): the C
oracle's restatement against the reference's own answers (no GPU)."""

import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIX = os.path.join(REPO, "tests", "golden", "locate", "locate_topo.npz")


def _oracle():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    return oracle


def test_oracle_locate_matches_reference_bitwise():
    z = np.load(FIX)
    found, idx, shift, zl = _oracle().locate(z["x3d"], z["y3d"], z["z3d"], z["points"],
                                             z["is_depth"])
    np.testing.assert_array_equal(found, z["found"])
    np.testing.assert_array_equal(idx, z["index"])
    np.testing.assert_array_equal(shift.view(np.int32), z["shift"].view(np.int32))
    np.testing.assert_array_equal(zl.view(np.int32), z["z_axis"].view(np.int32))


def test_fixture_covers_the_cases():
    """Inside cells, nodes and faces (shift 0 or 0.5), depth conversions,
    and points outside the physical cells."""
    z = np.load(FIX)
    assert (z["found"] == 0).sum() >= 5 and (z["found"] == 1).sum() >= 50
    assert ((z["shift"] == 0).all(1) & (z["found"] == 1)).sum() >= 8
    assert (z["shift"] == 0.5).any()
    assert (z["is_depth"] == 1).sum() >= 6


def test_station_arrays():
    """Shifts below zero move to the cell below; the last physical index
    zeroes the shift; eight corners in (i, j, k) order."""
    from cgfd3d_gb300 import locate
    shape = (16, 14, 12)                       # nz, ny, nx: ni=6, nj=8, nk=10
    keep, dijk, idx = locate.stations(shape, np.array([[2, 3, 9], [0, 0, 0], [5, 2, 4]]),
                                      np.array([[-0.25, 0.5, 0.0], [-0.1, 0.2, 0.3],
                                                [0.4, 0.1, 0.2]], np.float32))
    assert keep == [0, 2]                     # station 1 moves to i=-1: dropped
    np.testing.assert_array_equal(dijk[:3], np.float32([0.75, 0.5, 0.0]))
    assert dijk[3] == 0.0                     # i = ni-1 -> shift zeroed
    nx, ny = 12, 14
    assert idx[0] == (1 + 3) + (3 + 3) * nx + (9 + 3) * nx * ny
    assert idx[7] == idx[0] + 1 + nx + nx * ny
