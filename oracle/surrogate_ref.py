"""Float64 restatement of the seismogram surrogate's forward pass and
gradients (cgfd3d_gb300/surrogate.py, cgfd_sg.cu, cgfd_sg_gemm.cu).

TEST INFRASTRUCTURE ONLY: tests/ compare the device's bf16/fp32 forward
pass and parameter gradients with this numpy code -- exact, and with the
device's bf16 roundings emulated (emulate=True) -- and the product never
imports it.  The reference has no counterpart of the surrogate (it runs
the solver for every shot), so this restatement is checked on its own
against finite differences (tests/test_surrogate_ref.py).

The same network as the device: Fourier features of the position, three
GELU layers of 768 and one of 4096 (= 32 steps x 128 channels), five
decoder layers of nearest 2x upsampling plus a 5-tap convolution over time
(the last one linear, 6 x R channels), and the exact contraction of the six
Green's-function sets with the moment tensor.  Parameters are one flat
vector in the device's order (per layer W [out x in], then bias [out]).
"""

import numpy as np

NFEAT, NFREQ = 128, 20
HIDDEN, T0, C0, KS, UP, NDEC, NMT = 768, 32, 128, 5, 2, 5, 6


def bf16_round(a):
    """float64 values rounded to bfloat16 (round to nearest even)."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layers(nrec):
    R = 3 * nrec
    enc = [(HIDDEN, NFEAT), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (T0 * C0, HIDDEN)]
    dec = [(C0, KS * C0)] * (NDEC - 1) + [(NMT * R, KS * C0)]
    return enc, dec


def split(params, nrec):
    """Per-layer (W, b) views of the flat parameter vector."""
    enc, dec = layers(nrec)
    out, off = [], 0
    for (o, i) in enc + dec:
        W = params[off:off + o * i].reshape(o, i)
        b = params[off + o * i:off + o * i + o]
        out.append((W, b))
        off += o * i + o
    return out


def features(pos):
    B = len(pos)
    x = np.zeros((B, NFEAT))
    x[:, :3] = pos
    for d in range(3):
        for f in range(1, NFREQ + 1):
            a = np.pi * f * pos[:, d]
            c = 3 + d * 2 * NFREQ + 2 * (f - 1)
            x[:, c] = np.sin(a)
            x[:, c + 1] = np.cos(a)
    return x


def gelu(x):
    u = 0.7978845608028654 * (x + 0.044715 * x ** 3)
    return 0.5 * x * (1.0 + np.tanh(u))


def gelu_grad(x):
    c, a = 0.7978845608028654, 0.044715
    t = np.tanh(c * (x + a * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * c * (1.0 + 3.0 * a * x * x)


def im2col_up(X, up=UP, ks=KS):
    """X [B, Tin, C] -> A [B, Tin up, ks, C]"""
    B, Tin, C = X.shape
    Tout, h = Tin * up, ks // 2
    A = np.zeros((B, Tout, ks, C))
    for j in range(ks):
        tt = np.arange(Tout) + j - h
        ok = (tt >= 0) & (tt < Tout)
        A[:, ok, j, :] = X[:, tt[ok] // up, :]
    return A


def col2im_up(dA, Tin, up=UP, ks=KS):
    """Adjoint of im2col_up: dA [B, Tout, ks, C] -> dX [B, Tin, C]"""
    B, Tout, _, C = dA.shape
    h = ks // 2
    dX = np.zeros((B, Tin, C))
    for j in range(ks):
        tt = np.arange(Tout) + j - h
        ok = np.nonzero((tt >= 0) & (tt < Tout))[0]
        np.add.at(dX, (slice(None), tt[ok] // up), dA[:, ok, j, :])
    return dX


def forward(params, pos, M, nrec, nt, scale, keep=False, emulate=False):
    """Seismograms u [B, nt, 3 nrec]; with keep, also the activations.  With
    emulate, every value the device stores in bf16 (activations,
    pre-activations, the Green's functions) is rounded to bf16 here too;
    products and sums stay float64."""
    rd = bf16_round if emulate else (lambda v: v)
    P = split(np.asarray(params, np.float64), nrec)
    enc, dec = layers(nrec)
    B = len(pos)
    x = bf16_round(features(np.asarray(pos, np.float64)))
    acts = {"x0": x}
    h = x
    for n in range(len(enc)):
        W, b = P[n]
        z = h @ W.T + b
        acts["z%d" % n], acts["in%d" % n] = rd(z), h
        h = rd(gelu(z))
    X = h.reshape(B, T0, C0)
    ne = len(enc)
    for l in range(len(dec)):
        W, b = P[ne + l]
        A = im2col_up(X)
        Bt, Tout = A.shape[0], A.shape[1]
        z = A.reshape(Bt * Tout, -1) @ W.T + b
        acts["A%d" % l], acts["zd%d" % l] = A, rd(z)
        X = rd(z).reshape(B, Tout, -1) if l == len(dec) - 1 else rd(gelu(z)).reshape(B, Tout, -1)
    R = 3 * nrec
    G = X.reshape(B, -1, NMT, R)
    u = scale * np.einsum("bk,btkr->btr", np.asarray(M, np.float64), G[:, :nt])
    if keep:
        acts["G"] = G
        return u, acts
    return u


def loss_and_grad(params, pos, M, U, nrec, scale, emulate=False):
    """Mean squared relative misfit (1/B) sum_b |u_b - U_b|^2 / |U_b|^2 and
    its gradient with respect to the flat parameter vector.  With emulate,
    the gradients are rounded to bf16 where the device stores them (dG, the
    input gradients of every product, every dZ), as forward does for the
    activations."""
    rd = bf16_round if emulate else (lambda v: v)
    params = np.asarray(params, np.float64)
    P = split(params, nrec)
    enc, dec = layers(nrec)
    ne = len(enc)
    B, nt, R = U.shape
    u, a = forward(params, pos, M, nrec, nt, scale, keep=True, emulate=emulate)
    norm = (np.asarray(U, np.float64) ** 2).reshape(B, -1).sum(1)
    d = u - U
    loss = float(((d ** 2).reshape(B, -1).sum(1) / norm).mean())
    du = 2.0 * d / (B * norm[:, None, None])
    G = a["G"]
    dG = np.zeros_like(G)
    dG[:, :nt] = scale * np.einsum("bk,btr->btkr", np.asarray(M, np.float64), du)
    grads = [None] * (ne + len(dec))
    dz = rd(dG).reshape(B * G.shape[1], -1)
    for l in range(len(dec) - 1, -1, -1):
        W, _ = P[ne + l]
        A = a["A%d" % l]
        Bt, Tout, ks, C = A.shape
        A2 = A.reshape(Bt * Tout, -1)
        grads[ne + l] = (dz.T @ A2, dz.sum(0))
        dA = rd(dz @ W).reshape(Bt, Tout, ks, C)
        dX = col2im_up(dA, Tout // UP)
        zprev = a["zd%d" % (l - 1)].reshape(B, Tout // UP, -1) if l > 0 else \
            a["z%d" % (ne - 1)].reshape(B, T0, C0)
        dz = rd(dX * gelu_grad(zprev)).reshape(-1, dX.shape[-1])
    dz = dz.reshape(B, -1)
    for n in range(ne - 1, -1, -1):
        W, _ = P[n]
        grads[n] = (dz.T @ a["in%d" % n], dz.sum(0))
        if n == 0:
            break
        dz = rd(rd(dz @ W) * gelu_grad(a["z%d" % (n - 1)]))
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
