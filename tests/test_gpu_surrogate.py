"""The seismogram surrogate on the device: the tcgen05 matrix product
against torch, the forward pass and every parameter gradient against the
float64 restatement (oracle/surrogate_ref.py), and training on a teacher
network's outputs.

Tolerances: the device rounds weights, activations and their gradients to
bf16 (8 significant bits) and accumulates in fp32.  Against float64 a
forward pass agrees to about 1 % (relative L2).  The gradients of a batch
whose residual is mostly noise are far more sensitive: storing the
gradients in bf16 moves them by up to ~13 % (cosine 0.99) from exact
float64 in the first layer, which the restatement shows by rounding where
the device rounds (emulate=True).  So the device's gradients are held to
that emulation within 3 % (cosine 0.999) per layer, and to exact float64
within the emulation's own error.
"""

import numpy as np
import pytest

import surrogate_ref as sr

pytestmark = pytest.mark.gpu


def _sglib():
    from cgfd3d_gb300 import surrogate
    return surrogate._lib_sg()


@pytest.mark.parametrize("M,N,K", [(256, 384, 640), (200, 136, 72), (8, 1152, 640),
                                   (1024, 128, 1024),
                                   # at least two output tiles per SM: the
                                   # persistent form (not for the split-K mode),
                                   # 128 x 256 tiles (N > 128; a last tile of
                                   # 128 or fewer columns) and 256 x 128 tiles
                                   (32768, 1152, 640), (40000, 200, 136),
                                   (80000, 120, 72)])
def test_gemm_modes_match_torch(M, N, K):
    import ctypes as C
    import torch
    from cgfd3d_gb300 import _lib
    L = _sglib()
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    bias = torch.randn(N, generator=g).cuda()
    ref = A.float() @ B.float().T
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    # fp32 store
    C32 = torch.zeros(M, N, device="cuda")
    _lib.check(L.cgfd_sg_gemm(P(A), K, P(B), K, P(C32), N, M, N, K, 1.0, None, 0, 1, None, 1,
                              P(err), s))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.allclose(C32, ref, rtol=1e-4, atol=1e-3), (C32 - ref).abs().max().item()
    # bf16 with bias, GELU and the pre-activation copy
    ldc = (N + 7) // 8 * 8
    H = torch.zeros(M, ldc, dtype=torch.bfloat16, device="cuda")
    Z = torch.zeros(M, ldc, dtype=torch.bfloat16, device="cuda")
    _lib.check(L.cgfd_sg_gemm(P(A), K, P(B), K, P(H), ldc, M, N, K, 1.0, P(bias), 1, 0, P(Z),
                              1, P(err), s))
    torch.cuda.synchronize()
    z = ref + bias
    h = torch.nn.functional.gelu(z, approximate="tanh")
    assert torch.allclose(Z[:, :N].float(), z, rtol=1e-2, atol=1e-2)
    assert torch.allclose(H[:, :N].float(), h, rtol=1e-2, atol=1e-2)
    # fp32 accumulation split along K (added onto existing values)
    Cacc = torch.ones(M, N, device="cuda")
    _lib.check(L.cgfd_sg_gemm(P(A), K, P(B), K, P(Cacc), N, M, N, K, 1.0, None, 0, 2, None, 3,
                              P(err), s))
    torch.cuda.synchronize()
    assert torch.allclose(Cacc, ref + 1.0, rtol=1e-4, atol=1e-3)
    assert int(err.item()) == 0


def _flat_params_f64(net):
    import torch
    return net.w16.float().cpu().numpy().astype(np.float64)


def test_forward_and_gradients_match_float64():
    import torch
    from cgfd3d_gb300 import surrogate
    nrec, nt, B = 4, 1000, 8
    net = surrogate.Surrogate(nrec=nrec, nt=nt, seed=3, scale=1.0)
    rng = np.random.default_rng(5)
    pos = rng.uniform(-1, 1, (B, 3)).astype(np.float32)
    M = rng.standard_normal((B, 6)).astype(np.float32)
    params = _flat_params_f64(net)
    u_ref = sr.forward(params, pos, M, nrec, nt, 1.0)
    U = (u_ref * (1.0 + 0.3 * rng.standard_normal(u_ref.shape))).astype(np.float32)
    tp = torch.from_numpy(pos).cuda()
    tM = torch.from_numpy(M).cuda()
    u = net.predict(tp, tM).cpu().numpy().astype(np.float64)
    rel = np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)
    assert rel < 2e-2, rel
    tU = torch.from_numpy(U).cuda()
    norm = (tU.double() ** 2).reshape(B, -1).sum(1).float()
    loss_b = net.gradients(tp, tM, tU, norm)
    g = net.grad.cpu().numpy().astype(np.float64)
    loss_ref, g_ref = sr.loss_and_grad(params, pos, M, U, nrec, 1.0)
    _, g_emu = sr.loss_and_grad(params, pos, M, U, nrec, 1.0, emulate=True)
    loss = float((loss_b / norm).mean().item())
    assert abs(loss - loss_ref) < 2e-2 * loss_ref, (loss, loss_ref)
    assert net.device_error() == 0

    def cmp(x, y):
        cos = float(x @ y / (np.linalg.norm(x) * np.linalg.norm(y) + 1e-300))
        return cos, float(np.linalg.norm(x - y) / (np.linalg.norm(y) + 1e-300))

    for n, (a, b) in enumerate(net.lay.offsets):
        o = net.lay.layers[n][0]
        for name, sl in (("W", slice(a, b)), ("b", slice(b, b + o))):
            # the device against the restatement that rounds where it rounds:
            # agreement up to the rare rounding flips fp32 sums cause
            cos_e, rl_e = cmp(g[sl], g_emu[sl])
            assert cos_e > 0.999 and rl_e < 3e-2, (n, name, "emulated", cos_e, rl_e)
            # against exact float64: the error bf16 storage is designed to
            # give (the emulation's own), no more
            cos, rl = cmp(g[sl], g_ref[sl])
            _, rl_design = cmp(g_emu[sl], g_ref[sl])
            assert cos > 0.98 and rl <= 1.25 * rl_design + 2e-2, (n, name, cos, rl, rl_design)


def test_training_fits_a_teacher():
    """A student network trained by the device kernels fits the outputs of a
    fixed teacher network of the same shape: the misfit falls well below
    its starting value."""
    import torch
    from cgfd3d_gb300 import surrogate
    nrec, nt, B = 4, 1000, 64
    teacher = surrogate.Surrogate(nrec=nrec, nt=nt, seed=11, scale=1.0)
    student = surrogate.Surrogate(nrec=nrec, nt=nt, seed=12, scale=1.0, lr=3e-4)
    rng = np.random.default_rng(7)
    pos = torch.from_numpy(rng.uniform(-1, 1, (B, 3)).astype(np.float32)).cuda()
    M = torch.from_numpy(rng.standard_normal((B, 6)).astype(np.float32)).cuda()
    U = teacher.predict(pos, M).contiguous()
    norm = (U.double() ** 2).reshape(B, -1).sum(1).float()
    first = None
    for it in range(300):
        loss_b = student.gradients(pos, M, U, norm)
        student.apply()
        val = float((loss_b / norm).mean().item())
        first = val if first is None else first
    assert student.device_error() == 0
    assert np.isfinite(val) and val < 0.2 * first, (first, val)


def test_pipeline_on_solver_shots():
    """Shots of the batched solver on a small crop of the topography model
    feed the network: their seismograms equal single-shot runs of the same
    problems, training lowers the misfit, and held-out predictions are
    finite."""
    import torch
    from cgfd3d_gb300 import models, solver, surrogate as SG
    from helpers import assert_parity
    base = models._topo_base(96, 96, 64, 7)
    crop = (64, 64, 48)
    model = SG.crop_model(base, crop)
    ijd, M = SG.draw_sources(12, crop, seed=3)
    steps, nrec = 100, 16
    U, secs = SG.solve_shots(model, ijd, M, steps=steps, dt=0.005, batch=6, nrec=nrec)
    assert U.shape == (12, steps, 3 * nrec) and secs > 0
    one = SG.shot_problems(model, ijd[:1], M[:1], steps=steps, dt=0.005, nrec=nrec)[0]
    solver.drv_rk_curv_col_allstep(one)
    assert_parity(U[0], SG.seismograms(one, steps), "batched shot vs single run")
    scale = float(np.sqrt((U[:8].astype(np.float64) ** 2).mean()))
    net = SG.Surrogate(nrec=nrec, nt=steps, seed=2, scale=scale, lr=1e-3)
    pos = SG.normalise_positions(ijd, crop)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    tp, tM, tU = dev(pos[:8]), dev(M[:8]), dev(U[:8])
    norm = (tU.double() ** 2).reshape(8, -1).sum(1).float()
    first = last = None
    for it in range(150):
        loss_b = net.gradients(tp, tM, tU, norm)
        net.apply()
        v = float((loss_b / norm).mean().item())
        first = v if first is None else first
        last = v
    assert net.device_error() == 0
    assert last < 0.5 * first, (first, last)
    pred = net.predict(dev(pos[8:]), dev(M[8:])).cpu().numpy()
    assert pred.shape == (4, steps, 3 * nrec) and np.isfinite(pred).all()
    mis = SG.misfit(pred, U[8:])
    assert np.isfinite(mis).all()


def test_c_object_predicts_as_the_python_layer():
    """cgfd_sg_net_* (host descriptors in, host seismograms out) gives the
    Python layer's predictions bit for bit: one chunk of 40 shots, and 300
    shots in chunks of 256 + 44 against the two batches predicted apart."""
    import torch
    from cgfd3d_gb300 import surrogate as SG
    nrec, nt = 4, 1000
    sur = SG.Surrogate(nrec=nrec, nt=nt, seed=9, scale=0.37)
    net = SG.Net.of(sur)
    rng = np.random.default_rng(21)
    pos = rng.uniform(-1, 1, (300, 3)).astype(np.float32)
    M = rng.standard_normal((300, 6)).astype(np.float32)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    u40 = net.predict(pos[:40], M[:40])
    ref40 = sur.predict(dev(pos[:40]), dev(M[:40])).cpu().numpy()
    assert u40.shape == (40, nt, 3 * nrec)
    assert np.array_equal(u40, ref40)
    u = net.predict(pos, M)
    ref = np.concatenate([sur.predict(dev(pos[:256]), dev(M[:256])).cpu().numpy(),
                          sur.predict(dev(pos[256:]), dev(M[256:])).cpu().numpy()])
    assert np.array_equal(u, ref)
    assert np.isfinite(u).all() and np.abs(u).max() > 0
    with pytest.raises(Exception):
        SG.Net(sur.parameters()[:-1], nrec, nt, 1.0)     # wrong parameter count
    net.close()


@pytest.mark.parametrize("B,Tin,C", [(4, 16, 128), (2, 9, 12)])
def test_gather_kernels_match_torch(B, Tin, C):
    """im2col with up-sampling, its adjoint with GELU', and the transpose
    against torch, for a shape that takes the 16-byte paths (C % 8 == 0) and
    one that takes the scalar ones."""
    import ctypes as C_
    import torch
    L = _sglib()
    up, ks = 2, 5
    h, Tout = ks // 2, Tin * up
    g = torch.Generator(device="cpu").manual_seed(B * 100 + C)
    X = torch.randn(B, Tin, C, generator=g).to(torch.bfloat16).cuda()
    A = torch.empty(B * Tout, ks * C, dtype=torch.bfloat16, device="cuda")
    s = C_.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: C_.c_void_p(t.data_ptr())  # noqa: E731
    from cgfd3d_gb300 import _lib
    _lib.check(L.cgfd_sg_im2col_up(P(X), B, Tin, C, up, ks, P(A), s))
    t = torch.arange(Tout, device="cuda")
    ref = torch.zeros(B, Tout, ks, C, dtype=torch.bfloat16, device="cuda")
    for j in range(ks):
        tt = t + j - h
        ok = (tt >= 0) & (tt < Tout)
        ref[:, ok, j, :] = X[:, (tt[ok] // up), :]
    torch.cuda.synchronize()
    assert torch.equal(A.view(B, Tout, ks, C), ref)
    # adjoint: <im2col(x), y> = <x, col2im(y)> (no GELU factor), and GELU'
    dA = torch.randn(B * Tout, ks * C, generator=g).to(torch.bfloat16).cuda()
    dZ = torch.empty(B, Tin, C, dtype=torch.bfloat16, device="cuda")
    _lib.check(L.cgfd_sg_col2im_up_gelu(P(dA), B, Tin, C, up, ks, None, P(dZ), s))
    ref_dz = torch.zeros(B, Tin, C, dtype=torch.float64, device="cuda")
    d4 = dA.view(B, Tout, ks, C).double()
    for j in range(ks):
        tt = t + j - h
        ok = (tt >= 0) & (tt < Tout)
        ref_dz.index_add_(1, tt[ok] // up, d4[:, ok, j, :])
    torch.cuda.synchronize()
    assert torch.allclose(dZ.double(), ref_dz, rtol=1e-2, atol=1e-2)
    Z = torch.randn(B, Tin, C, generator=g).to(torch.bfloat16).cuda()
    dZg = torch.empty_like(dZ)
    _lib.check(L.cgfd_sg_col2im_up_gelu(P(dA), B, Tin, C, up, ks, P(Z), P(dZg), s))
    z = Z.double()
    c_, a_ = 0.7978845608028654, 0.044715
    th = torch.tanh(c_ * (z + a_ * z ** 3))
    gp = 0.5 * (1 + th) + 0.5 * z * (1 - th * th) * c_ * (1 + 3 * a_ * z * z)
    torch.cuda.synchronize()
    assert torch.allclose(dZg.double(), dZ.double() * gp, rtol=2e-2, atol=2e-2)
    # transpose of the im2col matrix (64-multiple shapes take the tiled path)
    rows, cols = A.shape
    Y = torch.empty(cols, rows, dtype=torch.bfloat16, device="cuda")
    _lib.check(L.cgfd_sg_transpose(P(A), rows, cols, cols, P(Y), rows, s))
    torch.cuda.synchronize()
    assert torch.equal(Y, A.t())
