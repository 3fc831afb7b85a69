"""The float64 restatement of the seismogram surrogate (the checker of the
device's gradients) against finite differences, and the network-free
baseline on exactly linear data (CPU only)."""

import numpy as np

import surrogate_ref as sr


def _params(rng, nrec):
    enc, dec = sr.layers(nrec)
    n = sum(o * i + o for o, i in enc + dec)
    p = np.zeros(n)
    off = 0
    for (o, i) in enc + dec:
        p[off:off + o * i] = rng.standard_normal(o * i) * np.sqrt(2.0 / i)
        p[off + o * i:off + o * i + o] = 0.01 * rng.standard_normal(o)
        off += o * i + o
    return p


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    nrec = 1
    params = _params(rng, nrec)
    B, nt = 2, 1000
    pos = rng.uniform(-1, 1, (B, 3))
    M = rng.standard_normal((B, 6))
    U = rng.standard_normal((B, nt, 3 * nrec))
    _, g = sr.loss_and_grad(params, pos, M, U, nrec, 1.0)
    enc, dec = sr.layers(nrec)
    off = 0
    for (o, i) in enc + dec:
        for idx in (off + int(rng.integers(o * i)), off + o * i + int(rng.integers(o))):
            h = 1e-6 * max(1.0, abs(params[idx]))
            p1, p2 = params.copy(), params.copy()
            p1[idx] += h
            p2[idx] -= h
            fd = (sr.loss_and_grad(p1, pos, M, U, nrec, 1.0)[0] -
                  sr.loss_and_grad(p2, pos, M, U, nrec, 1.0)[0]) / (2 * h)
            assert abs(g[idx] - fd) <= 1e-4 * abs(fd) + 1e-9, (idx, g[idx], fd)
        off += o * i + o


def test_im2col_adjoint():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((2, 7, 3))
    Y = rng.standard_normal((2, 14, sr.KS, 3))
    lhs = (sr.im2col_up(X) * Y).sum()
    rhs = (X * sr.col2im_up(Y, 7)).sum()
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, -3.14159265, 1e-3])
    r = sr.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == 1.0 + 2.0 ** -7              # rounds up
    assert abs(r[3] + 3.140625) < 1e-12
    assert abs(r[4] - 1e-3) < 1e-3 * 2.0 ** -8


def test_knn_green_recovers_linear_data():
    """With seismograms exactly linear in M and Green's functions constant
    over the neighbourhood, the k-nearest least-squares baseline is exact."""
    from cgfd3d_gb300 import surrogate
    rng = np.random.default_rng(2)
    G = rng.standard_normal((6, 50, 9))
    pos = rng.uniform(-1, 1, (40, 3))
    M = rng.standard_normal((40, 6))
    U = np.einsum("nk,ktr->ntr", M, G).astype(np.float32)
    q = rng.uniform(-1, 1, (5, 3))
    Mq = rng.standard_normal((5, 6)).astype(np.float32)
    pred = surrogate.knn_green(pos, M.astype(np.float32), U, q, Mq, k=12)
    true = np.einsum("nk,ktr->ntr", Mq, G)
    assert surrogate.misfit(pred, true).max() < 1e-5


def test_c_layout_matches_the_python_layout():
    """The C object's parameter count (cgfd_sg_net_nparam) is the training
    layout's, for several receiver counts; impossible layouts are refused."""
    from cgfd3d_gb300 import surrogate as SG
    for nrec, nt in ((64, 1000), (4, 1000), (16, 100), (1, 1024)):
        assert SG.nparam(nrec, nt) == SG.Layout(nrec, nt).nparam
    assert SG.nparam(64, 1025) == -1 and SG.nparam(0, 10) == -1
