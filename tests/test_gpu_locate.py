"""Point location on the device (cgfd_locator_*) against the reference's
answers and the oracle: indices and shifts must be identical, bit for bit."""

import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FIX = os.path.join(REPO, "tests", "golden", "locate", "locate_topo.npz")

pytestmark = pytest.mark.gpu


def _oracle():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    return oracle


def _same(got, want):
    for g, w in zip(got, want):
        np.testing.assert_array_equal(np.asarray(g).view(np.int32), np.asarray(w).view(np.int32))


def test_locator_matches_reference():
    from cgfd3d_gb300 import locate
    z = np.load(FIX)
    with locate.Locator(z["x3d"], z["y3d"], z["z3d"]) as L:
        got = L.locate(z["points"], z["is_depth"])
    _same(got, (z["found"], z["index"], z["shift"], z["z_axis"]))


def _grid(ni, nj, nk, seed):
    from types import SimpleNamespace
    from cgfd3d_gb300 import models
    X, Y, Z = models._coords_of(SimpleNamespace(ni=ni, nj=nj, nk=nk), seed)
    return [np.asarray(a, np.float32).reshape(nk + 6, nj + 6, ni + 6) for a in (X, Y, Z)]


@pytest.mark.parametrize("dims", [(70, 50, 40), (3, 9, 5)])
def test_locator_matches_oracle(dims):
    """Random points over a topography grid (and a grid narrower than the
    4x4x4 tiling, whose empty tiles must never match), some by depth."""
    from cgfd3d_gb300 import locate
    ni, nj, nk = dims
    X, Y, Z = _grid(ni, nj, nk, 5)
    rng = np.random.default_rng(1)
    n = 40
    pts = np.stack([rng.uniform(X.min(), X.max(), n), rng.uniform(Y.min(), Y.max(), n),
                    rng.uniform(Z.min(), Z.max(), n)], 1).astype(np.float32)
    dep = (rng.random(n) < 0.3).astype(np.int32)
    pts[dep == 1, 2] = rng.uniform(0, 2000, int(dep.sum()))
    # grid nodes and cell-face centres of physical cells
    for q in range(8):
        i, j, k = rng.integers(3, 3 + ni), rng.integers(3, 3 + nj), rng.integers(3, 3 + nk)
        pts[q] = (X[k, j, i], Y[k, j, i], Z[k, j, i])
        dep[q] = 0
    want = _oracle().locate(X, Y, Z, pts, dep)
    with locate.Locator(X, Y, Z) as L:
        got = L.locate(pts, dep)
    assert want[0].sum() >= 8
    _same(got, want)


def test_locator_edge_cases():
    from cgfd3d_gb300 import _lib, locate
    z = np.load(FIX)
    with locate.Locator(z["x3d"], z["y3d"], z["z3d"]) as L:
        f, i, s, zl = L.locate(np.zeros((0, 3), np.float32))
        assert len(f) == 0
        f, i, s, zl = L.locate(np.float32([[1e9, 0, 0], [0, 0, -1e9]]))
        assert (f == 0).all() and (i == -1000).all() and (s == 0).all()
    with pytest.raises(_lib.CgfdError):
        locate.Locator(np.zeros((6, 6, 6)), np.zeros((6, 6, 6)), np.zeros((6, 6, 6)))
