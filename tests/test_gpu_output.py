"""Slice and snapshot output packed on the device (cgfd_solver_pack_boxes,
cgfd_solver_fetch_boxes) against whole-state copies and the reference.

A box copy moves values without arithmetic, so every packed value must equal
the same point of the whole-state copy bit for bit; against the reference's
final wavefield the slices meet the parity tolerance of the time loop.
"""

import os

import numpy as np
import pytest

from conftest import GOLDEN
from helpers import assert_parity

pytestmark = pytest.mark.gpu


def _golden(name):
    from cgfd3d_gb300 import problem
    return problem.from_golden(os.path.join(GOLDEN, name + ".npz"))


def _expect(state, b):
    """The box b cut from a whole state (ncmp, nz, ny, nx) in packed order."""
    c = slice(b.c1, b.c2 + 1)
    k = slice(b.k1, b.k1 + (b.nk - 1) * b.dk + 1, b.dk)
    j = slice(b.j1, b.j1 + (b.nj - 1) * b.dj + 1, b.dj)
    i = slice(b.i1, b.i1 + (b.ni - 1) * b.di + 1, b.di)
    return state[c, k, j, i]


@pytest.mark.parametrize("case", ["iso_topo_noise", "visco_topo_noise"])
def test_boxes_equal_whole_state(case):
    from cgfd3d_gb300 import output, solver
    p, _ = _golden(case)
    with solver.Solver(p) as s:
        s.run(5)
        state = s.fetch_state()
        boxes = output.slice_boxes(p, x=[p.ni1, (p.ni1 + p.ni2) // 2],
                                   y=[p.nj2], z=[p.nk2, p.nk2 - 4])
        boxes.append(output.snapshot_box(p.ni1, (p.ni2 - p.ni1) // 3 + 1, 3,
                                         p.nj1 + 1, (p.nj2 - p.nj1) // 2, 2,
                                         p.nk1, (p.nk2 - p.nk1) // 4 + 1, 4))
        boxes.append(output.snapshot_box(0, p.nx, 1, 0, p.ny, 1, 0, p.nz, 1,
                                         c1=0, c2=p.ncmp - 1))   # ghosts too
        packed = s.pack_boxes(boxes)
        for b, got in zip(boxes, packed):
            np.testing.assert_array_equal(got, _expect(state, b))
        w = np.full(state.shape, np.nan, np.float32)
        s.fetch_boxes(boxes[:-1], w)
        mask = np.zeros(state.shape, bool)
        for b in boxes[:-1]:
            _expect(mask, b)[...] = True
        np.testing.assert_array_equal(w[mask], state[mask])
        assert np.isnan(w[~mask]).all()       # nothing outside the boxes
    if case.startswith("visco"):
        assert boxes[0].c2 == 8                # memory variables not sliced


def test_slices_match_reference_final_state():
    """The slices of the last step meet the time loop's parity bar against
    the reference's final wavefield."""
    from cgfd3d_gb300 import output, solver
    p, exp = _golden("iso_topo_noise")
    ref = exp["wav"].reshape(p.ncmp, p.nz, p.ny, p.nx)
    with solver.Solver(p) as s:
        s.run(p.nt_total)
        boxes = output.slice_boxes(p, x=[(p.ni1 + p.ni2) // 2], y=[(p.nj1 + p.nj2) // 2],
                                   z=[p.nk2])
        for b, got in zip(boxes, s.pack_boxes(boxes)):
            assert_parity(got, _expect(ref, b), "slice %r" % ((b.i1, b.j1, b.k1),))


def test_bad_boxes_rejected():
    from cgfd3d_gb300 import _lib, abi, solver
    p, _ = _golden("iso_topo_noise")
    with solver.Solver(p) as s:
        for bad in [abi.Box(0, 9, 0, 1, 1, 0, 1, 1, 0, 1, 1),       # component 9 of 9
                    abi.Box(0, 0, p.nx - 1, 2, 1, 0, 1, 1, 0, 1, 1),  # past x end
                    abi.Box(0, 0, 0, 1, 1, 0, 1, 1, p.nz - 3, 2, 3),  # stride past z end
                    abi.Box(0, 0, -1, 1, 1, 0, 1, 1, 0, 1, 1)]:
            with pytest.raises(_lib.CgfdError):
                s.pack_boxes([bad])
        with pytest.raises(ValueError):
            s.pack_boxes([abi.Box(0, 0, 0, 1, 0, 0, 1, 1, 0, 1, 1)])  # stride 0
        s.run(1)        # the solver still steps after the rejections
        s.check_finite()


def test_overlapped_output_equals_blocking():
    """Steps queued with run_async and slices packed into alternating slots
    hand out the same values as blocking step-by-step output."""
    from cgfd3d_gb300 import output, solver
    p, _ = _golden("iso_topo_noise")
    q = p.copy()
    boxes = output.slice_boxes(p, x=[p.ni1 + 2], y=[p.nj2 - 1], z=[p.nk2])
    want = []
    with solver.Solver(q) as s:
        for _ in range(6):
            s.run(1)
            want.append(s.pack_boxes(boxes))
    got = []
    w = np.zeros((p.ncmp, p.nz, p.ny, p.nx), np.float32)
    with solver.Solver(p) as s:
        for it in range(6):
            s.run_async(1)
            s.pack_boxes_async(boxes, it % 2)
            if it > 0:
                got.append(s.collect_boxes((it - 1) % 2))
        got.append(s.collect_boxes(1))
        s.pack_boxes_async(boxes, 0)
        s.collect_boxes(0, w)                 # scatter form of the last step
        s.run(0)
    for a, b in zip(got, want):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
    for b, v in zip(boxes, want[-1]):
        np.testing.assert_array_equal(_expect(w, b), v)


def test_output_slot_misuse_rejected():
    from cgfd3d_gb300 import _lib, output, solver
    p, _ = _golden("iso_topo_noise")
    boxes = output.slice_boxes(p, z=[p.nk2])
    with solver.Solver(p) as s:
        s.pack_boxes_async(boxes, 0)
        with pytest.raises(_lib.CgfdError):
            s.pack_boxes_async(boxes, 0)      # slot 0 not collected yet
        s.collect_boxes(0)
        with pytest.raises(_lib.CgfdError):
            s.pack_boxes_async(boxes, 2)      # two slots
        with pytest.raises(ValueError):
            s.collect_boxes(1)                # nothing packed there
