"""Layered-media discretisation ("loc" method) against the reference's own
media_layer2model_el_iso: the oracle bit for bit (CPU), the device within
float rounding (GPU)."""

import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIX = os.path.join(REPO, "tests", "golden", "media", "layer_el_iso.npz")


def _fixture():
    from cgfd3d_gb300 import media
    z = np.load(FIX)
    return z, media.read_md3lay(bytes(z["md3lay"]).decode())


def test_md3lay_parser():
    z, m = _fixture()
    assert m["NI"] == 4 and m["rec"].shape == (4, m["NY"], m["NX"], 10)
    assert np.all(m["rec"][2, :, :, 0] == -800.0)       # the flat interface


def test_oracle_matches_reference_bitwise():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, m = _fixture()
    got = oracle.layer_el_iso_loc(m, z["x3d"], z["y3d"], z["z3d"])
    for g, w in zip(got, (z["lam"], z["mu"], z["rho"])):
        np.testing.assert_array_equal(g.view(np.int32), w.view(np.int32))
    # points on the flat interface take the mean of the two layers
    on = np.isclose(z["z3d"], -800.0)
    assert on.sum() > 100


def test_oracle_refuses_points_outside_the_mesh():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    z, m = _fixture()
    x = z["x3d"].copy()
    x[0, 0, 0] = m["MINX"] - 10.0
    assert oracle.layer_el_iso_loc(m, x, z["y3d"], z["z3d"]) is None


@pytest.mark.gpu
def test_device_matches_reference():
    from cgfd3d_gb300 import _lib, media
    z, m = _fixture()
    got = media.layer_el_iso(m, z["x3d"], z["y3d"], z["z3d"])
    for g, w in zip(got, (z["lam"], z["mu"], z["rho"])):
        np.testing.assert_allclose(g, w, rtol=2e-6, atol=0)
    x = z["x3d"].copy()
    x[0, 0, 0] = m["MINX"] - 10.0
    with pytest.raises(_lib.CgfdError):
        media.layer_el_iso(m, x, z["y3d"], z["z3d"])
