"""Set-up helpers of the Python API against the reference's own set-up
(no GPU): the exponential sponge's blocks and masks."""

import os

import numpy as np
import pytest

from conftest import GOLDEN


@pytest.mark.parametrize("case", ["iso_flat_ablexp", "vti_topo_ablexp_graves"])
def test_ablexp_masks_match_reference(case):
    """Blocks identical; masks within one float ulp (the reference's expf and
    numpy's exp may round the last bit differently)."""
    from cgfd3d_gb300 import models, problem
    p, exp = problem.from_golden(os.path.join(GOLDEN, case + ".npz"))
    c = exp["case"]
    q = p.copy()
    coords = None
    if c["topo"]:
        coords = [p.coords[k].reshape(p.nz, p.ny, p.nx) for k in ("x3d", "y3d", "z3d")]
    models.add_ablexp(q, c["ablexp"], 6000.0, coords=coords,
                      dh=None if c["topo"] else c["dh"])
    np.testing.assert_array_equal(q.ablexp["blk"].ravel(), p.ablexp["blk"].ravel())
    for k in ("Ex", "Ey", "Ez"):
        np.testing.assert_allclose(q.ablexp[k], p.ablexp[k], rtol=2.5e-7, atol=0)
        assert (q.ablexp[k] < 1).sum() == (p.ablexp[k] < 1).sum()


def test_graves_qs_helper():
    from cgfd3d_gb300 import models
    p = models.flat_model(ni=20, nj=18, nk=16, steps=2)
    models.add_graves_qs(p, 30.0, 1.5)
    assert p.graves_qs["Qs"].shape == (p.vol,) and p.graves_qs["freq"] == 1.5
    assert p.to_c().graves_qs == 1
