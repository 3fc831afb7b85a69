"""Learned seismogram surrogate over the batched solver.

No counterpart in the reference, which runs the solver once per shot
(forward/main_curv_col_el_3d.c:849-858).  For a fixed model and receiver
set, a small network predicts the receivers' velocity seismograms of a shot
from its source position and moment tensor; the solver checks it and stays
the fallback.

Network (device work in cgfd_sg.cu and cgfd_sg_gemm.cu; this module
allocates buffers with torch and calls the C ABI):

  position (x, y, depth; normalised to [-1, 1]) -> Fourier features (128)
  encoder   3 x [GEMM 768 + bias + GELU] -> GEMM 4096 + GELU = 32 steps x 128
  decoder   5 x [2x nearest upsampling + 5-tap conv over time]: 128 channels,
            the last one 1152 = 6 moment components x 192 traces, no GELU
  output    u[b, t, r] = scale sum_k M[b, k] G[b, t, k, r], t < 1000

Because seismograms are linear in the moment tensor, the network predicts
the six Green's-function sets of the position and the contraction with M is
exact; the network has about 5.5 M parameters, bf16 weights and activations
with fp32 accumulation (tcgen05 tensor cores), fp32 master weights and AdamW.

The loss is the mean over shots of the squared relative L2 misfit, the
quantity the fallback rule tests (a shot passes at misfit <= 5 %).
"""

import ctypes as C
import math

import numpy as np

from . import _lib

NFEAT, NFREQ = 128, 20
HIDDEN = 768
T0, C0 = 32, 128
KS, UP = 5, 2
NDEC = 5
NMT = 6


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check(rc):
    _lib.check(rc)


class Layout:
    """Shapes of the network for `nrec` receivers x 3 components and `nt`
    samples (the decoder produces T0 * 2^NDEC >= nt steps)."""

    def __init__(self, nrec=64, nt=1000):
        self.R = 3 * nrec
        self.nt = nt
        self.T = T0 * UP ** NDEC
        if self.T < nt:
            raise ValueError("decoder length %d < %d samples" % (self.T, nt))
        self.enc = [(HIDDEN, NFEAT), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (T0 * C0, HIDDEN)]
        cout = [C0] * (NDEC - 1) + [NMT * self.R]
        self.dec = [(cout[l], KS * C0) for l in range(NDEC)]
        self.layers = self.enc + self.dec
        # flat parameter vector: per layer W (out x in) then bias (out)
        self.offsets = []
        off = 0
        for (o, i) in self.layers:
            self.offsets.append((off, off + o * i))
            off += o * i + o
        self.nparam = off


def _lib_sg():
    L = _lib.lib()
    if getattr(L, "_sg_ready", False):
        return L
    vp, ll, i, f = C.c_void_p, C.c_longlong, C.c_int, C.c_float
    L.cgfd_sg_gemm.argtypes = [vp, ll, vp, ll, vp, ll, i, i, i, f, vp, i, i, vp, i, vp, vp]
    L.cgfd_sg_features.argtypes = [vp, i, i, i, vp, vp]
    L.cgfd_sg_im2col_up.argtypes = [vp, i, i, i, i, i, vp, vp]
    L.cgfd_sg_col2im_up_gelu.argtypes = [vp, i, i, i, i, i, vp, vp, vp]
    L.cgfd_sg_gelu_bwd.argtypes = [vp, vp, ll, vp, vp]
    L.cgfd_sg_contract.argtypes = [vp, vp, i, i, i, i, f, vp, vp]
    L.cgfd_sg_contract_loss.argtypes = [vp, vp, i, i, i, i, f, vp, vp, vp, vp, vp]
    L.cgfd_sg_transpose.argtypes = [vp, i, i, ll, vp, ll, vp]
    L.cgfd_sg_colsum.argtypes = [vp, ll, i, ll, vp, vp]
    L.cgfd_sg_adamw.argtypes = [vp, vp, vp, vp, vp, ll, f, f, f, f, f, i, vp]
    L.cgfd_sg_to_bf16.argtypes = [vp, ll, vp, vp]
    L.cgfd_sg_net_nparam.argtypes = [i, i]
    L.cgfd_sg_net_nparam.restype = ll
    L.cgfd_sg_net_create.argtypes = [i, i, vp, ll, f, C.POINTER(vp)]
    L.cgfd_sg_net_predict.argtypes = [vp, i, vp, vp, vp]
    L.cgfd_sg_net_destroy.argtypes = [vp]
    L.cgfd_sg_net_destroy.restype = None
    L._sg_ready = True
    return L


class Surrogate:
    """The network's parameters, optimiser state and work buffers on cuda:0.

    scale: amplitude of the seismograms in the network's units (targets are
    divided by it in training and predictions multiplied by it)."""

    def __init__(self, nrec=64, nt=1000, seed=0, scale=1.0, lr=1e-3, wd=1e-4):
        import torch
        self.lay = Layout(nrec, nt)
        self.scale = float(scale)
        self.lr, self.wd = lr, wd
        self.step_n = 0
        dev = "cuda"
        g = torch.Generator(device="cpu").manual_seed(seed)
        w = torch.zeros(self.lay.nparam, dtype=torch.float32)
        for n, ((o, i), (a, b)) in enumerate(zip(self.lay.layers, self.lay.offsets)):
            std = math.sqrt(2.0 / i) if n < len(self.lay.layers) - 1 else 0.1 / math.sqrt(i)
            w[a:b] = torch.randn(o * i, generator=g) * std
        self.w = w.to(dev)
        self.w16 = torch.empty(self.lay.nparam, dtype=torch.bfloat16, device=dev)
        self.grad = torch.zeros(self.lay.nparam, dtype=torch.float32, device=dev)
        self.m = torch.zeros_like(self.w)
        self.v = torch.zeros_like(self.w)
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.launches = 0          # kernels this object has launched
        L = _lib_sg()
        _check(L.cgfd_sg_to_bf16(_ptr(self.w), self.lay.nparam, _ptr(self.w16), _stream()))
        # transposed bf16 weights (in x out) for the input-gradient products
        self.wt = [torch.empty(i * o, dtype=torch.bfloat16, device=dev)
                   for (o, i) in self.lay.layers]
        self._refresh_transposes()
        self._bufs = {}

    # -- parameters -----------------------------------------------------------
    def W(self, n, which="w16"):
        a, b = self.lay.offsets[n]
        return getattr(self, which)[a:b]

    def bias(self, n, which="w"):
        o, _ = self.lay.layers[n]
        _, b = self.lay.offsets[n]
        return getattr(self, which)[b:b + o]

    def _refresh_transposes(self):
        L = _lib_sg()
        for n, (o, i) in enumerate(self.lay.layers):
            _check(L.cgfd_sg_transpose(_ptr(self.W(n)), o, i, i, _ptr(self.wt[n]), o, _stream()))
        self.launches += len(self.lay.layers)

    # -- buffers ----------------------------------------------------------------
    def _buffers(self, B, train):
        import torch
        key = (B, train)
        if key in self._bufs:
            return self._bufs[key]
        bf = dict(dtype=torch.bfloat16, device="cuda")
        lay = self.lay
        d = {"x0": torch.empty(B * NFEAT, **bf)}
        for n, (o, _) in enumerate(lay.enc):
            d["z%d" % n] = torch.empty(B * o, **bf)
            d["h%d" % n] = torch.empty(B * o, **bf)
        tin = T0
        for l, (o, k) in enumerate(lay.dec):
            tout = tin * UP
            d["a_d%d" % l] = torch.empty(B * tout * k, **bf)
            d["z_d%d" % l] = torch.empty(B * tout * o, **bf)
            d["h_d%d" % l] = torch.empty(B * tout * o, **bf)
            tin = tout
        if train:
            big = max(B * lay.T * o for (o, _) in lay.dec)
            bigk = max(B * (T0 * UP ** (l + 1)) * k for l, (_, k) in enumerate(lay.dec))
            d["dz"] = torch.empty(big, **bf)
            d["dzt"] = torch.empty(big, **bf)
            d["at"] = torch.empty(max(bigk, B * max(i for _, i in lay.enc)), **bf)
            d["da"] = torch.empty(max(bigk, B * HIDDEN), **bf)
            d["dh"] = torch.empty(max(B * C0 * T0 * UP ** (NDEC - 1), B * T0 * C0, B * HIDDEN), **bf)
            d["loss"] = torch.zeros(B, dtype=torch.float32, device="cuda")
        self._bufs[key] = d
        return d

    # -- products -------------------------------------------------------------
    def _gemm(self, A, lda, Bm, ldb, Cm, ldc, M, N, K, bias=None, act=0, mode=0, Z=None,
              splits=1):
        L = _lib_sg()
        _check(L.cgfd_sg_gemm(_ptr(A), lda, _ptr(Bm), ldb, _ptr(Cm), ldc, M, N, K, 1.0,
                              None if bias is None else _ptr(bias), act, mode,
                              None if Z is None else _ptr(Z), splits, _ptr(self.err),
                              _stream()))
        self.launches += 1

    # -- forward ----------------------------------------------------------------
    def _forward(self, pos, d, B):
        """Activations of every layer for B shots; returns the G buffer."""
        L = _lib_sg()
        s = _stream()
        lay = self.lay
        _check(L.cgfd_sg_features(_ptr(pos), B, NFREQ, NFEAT, _ptr(d["x0"]), s))
        self.launches += 1
        x, xin = d["x0"], NFEAT
        for n, (o, i) in enumerate(lay.enc):
            self._gemm(x, xin, self.W(n), i, d["h%d" % n], o, B, o, i, bias=self.bias(n),
                       act=1, mode=0, Z=d["z%d" % n])
            x, xin = d["h%d" % n], o
        tin = T0
        ne = len(lay.enc)
        for l, (o, k) in enumerate(lay.dec):
            tout = tin * UP
            _check(L.cgfd_sg_im2col_up(_ptr(x), B, tin, C0, UP, KS, _ptr(d["a_d%d" % l]), s))
            self.launches += 1
            last = l == len(lay.dec) - 1
            self._gemm(d["a_d%d" % l], k, self.W(ne + l), k, d["h_d%d" % l], o, B * tout, o, k,
                       bias=self.bias(ne + l), act=0 if last else 1, mode=0,
                       Z=None if last else d["z_d%d" % l])
            x = d["h_d%d" % l]
            tin = tout
        return x

    def predict(self, pos, M):
        """Seismograms [B, nt, R] (float32 torch tensor on the device) of B
        shots: pos [B, 3] normalised positions, M [B, 6] moment tensors in
        the network's units (float32 device tensors)."""
        import torch
        B = pos.shape[0]
        d = self._buffers(B, False)
        G = self._forward(pos.contiguous(), d, B)
        U = torch.empty((B, self.lay.nt, self.lay.R), dtype=torch.float32, device="cuda")
        _check(_lib_sg().cgfd_sg_contract(_ptr(G), _ptr(M.contiguous()), B, self.lay.T,
                                          self.lay.nt, self.lay.R, self.scale, _ptr(U),
                                          _stream()))
        self.launches += 1
        return U

    # -- training ---------------------------------------------------------------
    def gradients(self, pos, M, U, norm):
        """Loss (device tensor [B] of squared misfits before the norm
        division) and parameter gradients in self.grad for one batch; U [B,
        nt, R] targets in physical units, norm [B] their squared norms."""
        L = _lib_sg()
        s = _stream()
        lay = self.lay
        B = pos.shape[0]
        d = self._buffers(B, True)
        G = self._forward(pos.contiguous(), d, B)
        self.grad.zero_()
        d["loss"].zero_()
        ne = len(lay.enc)
        # two gradient buffers in turn: the large one first holds dG (the
        # last decoder layer has no GELU, so its dZ is dG); every later dZ
        # fits either
        big, small = d["dz"], d["dh"]

        def other(t):
            return small if t is big else big

        dz = big
        _check(L.cgfd_sg_contract_loss(_ptr(G), _ptr(M), B, lay.T, lay.nt, lay.R, self.scale,
                                       _ptr(U), _ptr(norm), _ptr(d["loss"]), _ptr(dz), s))
        self.launches += 1
        tout = lay.T
        for l in range(len(lay.dec) - 1, -1, -1):
            o, k = lay.dec[l]
            tin = tout // UP
            rows = B * tout
            n = ne + l
            self._weight_grad(dz, rows, o, d["a_d%d" % l], k, n, d)
            # dA = dZ W  (W^T stored [k, o])
            self._gemm(dz, o, self.wt[n], o, d["da"], k, rows, k, o, mode=0)
            prev_z = d["z_d%d" % (l - 1)] if l > 0 else d["z%d" % (ne - 1)]
            nxt = other(dz)
            _check(L.cgfd_sg_col2im_up_gelu(_ptr(d["da"]), B, tin, C0, UP, KS, _ptr(prev_z),
                                            _ptr(nxt), s))
            self.launches += 1
            dz = nxt                              # the next layer's dZ
            tout = tin
        # encoder, last layer first; dz holds dZ of encoder layer ne-1
        for n in range(ne - 1, -1, -1):
            o, i = lay.enc[n]
            xin = d["x0"] if n == 0 else d["h%d" % (n - 1)]
            self._weight_grad(dz, B, o, xin, i, n, d)
            if n == 0:
                break
            self._gemm(dz, o, self.wt[n], o, d["da"], i, B, i, o, mode=0)
            nxt = other(dz)
            _check(L.cgfd_sg_gelu_bwd(_ptr(d["da"]), _ptr(d["z%d" % (n - 1)]), B * i,
                                      _ptr(nxt), s))
            self.launches += 1
            dz = nxt
        return d["loss"]

    def _weight_grad(self, dz, rows, o, x, i, n, d):
        """grad W_n += dZ^T X and grad b_n += column sums of dZ (rows x o,
        rows x i)."""
        L = _lib_sg()
        s = _stream()
        _check(L.cgfd_sg_transpose(_ptr(dz), rows, o, o, _ptr(d["dzt"]), rows, s))
        _check(L.cgfd_sg_transpose(_ptr(x), rows, i, i, _ptr(d["at"]), rows, s))
        tiles = ((o + 127) // 128) * ((i + 127) // 128)
        splits = max(1, min(rows // 1024, (2 * 152 + tiles - 1) // tiles))
        self._gemm(d["dzt"], rows, d["at"], rows, self.W(n, "grad"), i, o, i, rows, mode=2,
                   splits=splits)
        _check(L.cgfd_sg_colsum(_ptr(dz), rows, o, o, _ptr(self.bias(n, "grad")), s))
        self.launches += 3

    def apply(self, lr=None):
        """One AdamW step with the gradients in self.grad."""
        self.step_n += 1
        _check(_lib_sg().cgfd_sg_adamw(_ptr(self.w), _ptr(self.w16), _ptr(self.grad),
                                       _ptr(self.m), _ptr(self.v), self.lay.nparam,
                                       self.lr if lr is None else lr, 0.9, 0.999, 1e-8,
                                       self.wd, self.step_n, _stream()))
        self.launches += 1
        self._refresh_transposes()

    def device_error(self):
        return int(self.err.item())

    def sync_gradients(self, loss=None, group=None):
        """Data-parallel training over the ranks of `group`: every rank ran
        gradients() on its own share of the batch (shares of equal size);
        the mean over ranks of the gradients (and of `loss`, when given) is
        the whole batch's.  One all-reduce each; a no-op on one rank."""
        allreduce_mean(self.grad, group)
        if loss is not None:
            allreduce_mean(loss, group)
        return loss

    def parameters(self):
        """The flat fp32 parameter vector (host copy): per layer W (out x
        in), then its bias."""
        return self.w.cpu().numpy()


def allreduce_mean(t, group=None):
    """In place: t becomes the mean of t over the ranks of the initialised
    process group (NCCL for device tensors, gloo for host tensors); a no-op
    without a group or with one rank.  The only collective of data-parallel
    surrogate training."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return t
    world = dist.get_world_size(group)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        t.div_(world)
    return t


def nparam(nrec=64, nt=1000):
    """Parameters of the layout as the C library counts them (no GPU)."""
    return int(_lib_sg().cgfd_sg_net_nparam(int(nrec), int(nt)))


class Net:
    """A trained network as the library's C object (cgfd_sg_net_*): host
    positions and moment tensors in, host seismograms out, no torch on the
    way.  Chunks of CGFD_SG_NET_CHUNK (256) shots, each bit-identical to
    Surrogate.predict of the same shots as one batch."""

    CHUNK = 256

    def __init__(self, params, nrec=64, nt=1000, scale=1.0):
        w = np.ascontiguousarray(params, dtype=np.float32)
        self.nrec, self.nt = int(nrec), int(nt)
        self._h = C.c_void_p()
        _check(_lib_sg().cgfd_sg_net_create(self.nrec, self.nt, w.ctypes.data, w.size,
                                            float(scale), C.byref(self._h)))

    @classmethod
    def of(cls, sur):
        return cls(sur.parameters(), sur.lay.R // 3, sur.lay.nt, sur.scale)

    def predict(self, pos, M, out=None):
        """Seismograms [n, nt, 3 nrec] (into `out` when given: C-contiguous
        float32 of that shape, e.g. pinned for a fast copy back)."""
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        M = np.ascontiguousarray(M, dtype=np.float32)
        n = pos.shape[0]
        if pos.shape != (n, 3) or M.shape != (n, 6):
            raise ValueError("positions [n, 3] and moment tensors [n, 6]")
        shape = (n, self.nt, 3 * self.nrec)
        if out is None:
            u = np.empty(shape, np.float32)
        elif (not isinstance(out, np.ndarray) or out.shape != shape or out.dtype != np.float32
              or not out.flags.c_contiguous):
            raise ValueError("out: C-contiguous float32 array of shape %s" % (shape,))
        else:
            u = out
        _check(_lib_sg().cgfd_sg_net_predict(self._h, n, pos.ctypes.data, M.ctypes.data,
                                             u.ctypes.data))
        return u

    def close(self):
        if self._h:
            _lib_sg().cgfd_sg_net_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# data: shots of the batched solver on a fixed model
# ---------------------------------------------------------------------------

def crop_model(base, crop=(256, 256, 128)):
    """The fixed model: a crop of the topography model's grid, metrics and
    media (base: models._topo_base of the 400 x 400 x 200 model), centred
    in x and y, its top the model's surface."""
    X, Y, Z, met, vp, vs, rho = base
    nk_b, nj_b, ni_b = (s - 6 for s in Z.shape)
    ci, cj, ck = crop
    i0, j0, k0 = (ni_b - ci) // 2, (nj_b - cj) // 2, nk_b - ck
    sl = (slice(k0, k0 + ck + 6), slice(j0, j0 + cj + 6), slice(i0, i0 + ci + 6))
    return dict(crop=crop, X=X[sl], Y=Y[sl], Z=Z[sl],
                met={k: np.ascontiguousarray(v[sl]).ravel() for k, v in met.items()},
                vp=vp[sl], vs=vs[sl], rho=rho[sl])


def draw_sources(n, crop=(256, 256, 128), seed=0, npml=12, dh=100.0):
    """n sources uniform in the model's volume: grid indices (i, j) at least
    PML + 3 cells inside, depth 1-8 km below the top; moment tensors of six
    i.i.d. N(0, 1) components, Frobenius-normalised (unit norm).  Returns
    ijd [n, 3] (i, j physical indices, depth in cells) and M [n, 6]."""
    rng = np.random.default_rng(seed)
    ni, nj, nk = crop
    m = npml + 3
    i = rng.integers(m, ni - m, n)
    j = rng.integers(m, nj - m, n)
    dmax = min(8000.0, (nk - npml - 3) * dh)
    depth = np.rint(rng.uniform(1000.0, dmax, n) / dh).astype(np.int64)
    M = rng.standard_normal((n, 6))
    fro = np.sqrt((M[:, :3] ** 2).sum(1) + 2 * (M[:, 3:] ** 2).sum(1))
    return np.stack([i, j, depth], 1), (M / fro[:, None]).astype(np.float32)


def normalise_positions(ijd, crop=(256, 256, 128), npml=12, dh=100.0):
    """Source positions to [-1, 1]: x, y over the source region, depth over
    1-8 km."""
    ni, nj, nk = crop
    m = npml + 3
    dmax = min(8000.0, (nk - npml - 3) * dh) / dh
    x = 2.0 * (ijd[:, 0] - m) / max(ni - 2 * m - 1, 1) - 1.0
    y = 2.0 * (ijd[:, 1] - m) / max(nj - 2 * m - 1, 1) - 1.0
    z = 2.0 * (ijd[:, 2] - 10.0) / max(dmax - 10.0, 1.0) - 1.0
    return np.stack([x, y, z], 1).astype(np.float32)


def receiver_grid(crop=(256, 256, 128), nrec=64, npml=12):
    ni, nj, _ = crop
    side = int(round(math.sqrt(nrec)))
    return [(int(npml + 2 + (ni - 2 * npml - 4) * a / max(side - 1, 1)),
             int(npml + 2 + (nj - 2 * npml - 4) * b / max(side - 1, 1)))
            for a in range(side) for b in range(side)][:nrec]


def shot_problems(model, ijd, M, steps=1000, dt=0.01, m0=1e16, fc=2.0, t0=0.6, nrec=64,
                  npml=12):
    """Problems of the shots (all on the fixed model) for the solver."""
    from . import models
    from .problem import Problem
    ci, cj, ck = model["crop"]
    out = []
    for n in range(len(ijd)):
        p = Problem(ci, cj, ck, dt, steps + 1)
        p.metric = model["met"]
        models.set_iso_media(p, model["vp"], model["vs"], model["rho"])
        p.free_top = 1
        models.add_pml(p, model["X"], model["Y"], model["Z"], npml,
                       [(0, 0), (0, 1), (1, 0), (1, 1), (2, 0)], vref=6500.0,
                       alpha_max=math.pi * fc)
        i, j, dk = (int(v) for v in ijd[n])
        models.add_moment_source(p, p.ni1 + i, p.nj1 + j, p.nk2 - dk,
                                 tuple(float(m0 * v) for v in M[n]), fc=fc, t0=t0,
                                 stf_len=min(steps + 1, 400) * dt)
        models.add_surface_receivers(p, receiver_grid(model["crop"], nrec, npml))
        out.append(p)
    return out


def seismograms(p, nt):
    """Velocity seismograms [nt, 3 nrec] of a solved problem (receiver-major
    traces: r = 3 receiver + component)."""
    r = p.recv
    s = r["seismo"].reshape(r["n"], r["ncmp"], r["max_nt"])[:, :3, :nt]
    return np.ascontiguousarray(s.transpose(2, 0, 1).reshape(nt, 3 * r["n"]))


def solve_shots(model, ijd, M, steps=1000, dt=0.01, batch=64, **kw):
    """Seismograms [n, steps, 3 nrec] of the shots, `batch` shots per
    batched-solver launch; returns (seismograms, seconds of solver time)."""
    import time
    from .solver import Batch
    n = len(ijd)
    out = np.zeros((n, steps, 3 * kw.get("nrec", 64)), np.float32)
    secs = 0.0
    for a in range(0, n, batch):
        probs = shot_problems(model, ijd[a:a + batch], M[a:a + batch], steps=steps, dt=dt, **kw)
        t = time.perf_counter()
        with Batch(probs) as b:
            b.run(probs[0].nt_total)
            b.fetch_seismograms()
        secs += time.perf_counter() - t
        for q, p in enumerate(probs):
            out[a + q] = seismograms(p, steps)
    return out, secs


def misfit(pred, true):
    """Relative L2 misfit per shot."""
    d = (pred - true).reshape(len(true), -1)
    t = true.reshape(len(true), -1)
    return np.sqrt((d.astype(np.float64) ** 2).sum(1) / np.maximum((t.astype(np.float64) ** 2).sum(1), 1e-300))


def knn_green(pos_train, M_train, U_train, pos_query, M_query, k=12):
    """The method without the network: each query's six Green's-function
    sets fitted by least squares to the seismograms of its k nearest
    training shots (seismograms are linear in M; the Green's functions are
    taken as constant over the neighbourhood), then contracted with the
    query's moment tensor."""
    out = np.zeros((len(pos_query),) + U_train.shape[1:], np.float32)
    flat = U_train.reshape(len(U_train), -1)
    for q in range(len(pos_query)):
        dist = ((pos_train - pos_query[q]) ** 2).sum(1)
        nn = np.argsort(dist)[:k]
        A = M_train[nn].astype(np.float64)                  # k x 6
        G, *_ = np.linalg.lstsq(A, flat[nn].astype(np.float64), rcond=None)
        out[q] = (M_query[q].astype(np.float64) @ G).reshape(U_train.shape[1:])
    return out
