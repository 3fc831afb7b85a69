/*
 * cgfd_sg_net.cu -- the trained seismogram surrogate as one C object:
 * predictions for an array of per-shot descriptors (source position and
 * moment tensor) from host arrays to host seismograms, without Python.
 *
 * No counterpart in the reference, which runs the solver for every shot
 * (forward/main_curv_col_el_3d.c:849-858).  The network and its flat
 * parameter vector are those cgfd3d_gb300/surrogate.py trains (the same
 * layer table, the same order: per layer W (out x in) then the bias); the
 * forward pass issues the same device kernels in the same order with the
 * same shapes, so a batch of up to CGFD_SG_NET_CHUNK shots gives the Python
 * layer's predictions bit for bit.  Larger requests run in chunks of that
 * many shots.
 *
 *   position -> Fourier features (128) -> 3 x [768, GELU] -> [4096, GELU]
 *   (= 32 steps x 128 channels) -> 5 x [2x upsampling, 5-tap conv over
 *   time; 128 channels, the last 6 x 3 nrec, linear] -> G (1024 steps)
 *   -> u[b, t, r] = scale sum_k M[b, k] G[b, t, k, r], t < nt
 */
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "../../include/cgfd3d_gpu.h"

__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg);

namespace sgn {

constexpr int NFEAT = 128, NFREQ = 20, HIDDEN = 768, T0 = 32, C0 = 128, KS = 5, UP = 2,
              NDEC = 5, NMT = 6, NENC = 4, NLAY = NENC + NDEC;

static int net_err(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return cgfd_set_error_msg(code, buf);
}

/* the layer table of the network for R = 3 nrec traces */
struct Layers {
  int out[NLAY], in[NLAY];
  long long w[NLAY], b[NLAY];   /* offsets of W and bias in the flat vector */
  long long n;                  /* parameters in all */
};

static Layers layers_of(int R)
{
  Layers L;
  const int enc_o[NENC] = {HIDDEN, HIDDEN, HIDDEN, T0 * C0};
  const int enc_i[NENC] = {NFEAT, HIDDEN, HIDDEN, HIDDEN};
  for (int n = 0; n < NENC; n++) {
    L.out[n] = enc_o[n];
    L.in[n] = enc_i[n];
  }
  for (int l = 0; l < NDEC; l++) {
    L.out[NENC + l] = l == NDEC - 1 ? NMT * R : C0;
    L.in[NENC + l] = KS * C0;
  }
  long long off = 0;
  for (int n = 0; n < NLAY; n++) {
    L.w[n] = off;
    L.b[n] = off + (long long)L.out[n] * L.in[n];
    off = L.b[n] + L.out[n];
  }
  L.n = off;
  return L;
}

}  // namespace sgn

using namespace sgn;

struct cgfd_sg_net {
  int nrec, nt, R, T;
  float scale;
  Layers L;
  cudaStream_t st = nullptr;
  float *w = nullptr;          /* fp32 parameters (biases are read here) */
  void *w16 = nullptr;         /* bf16 copy (the products' weights) */
  int *d_err = nullptr;
  /* work buffers for CGFD_SG_NET_CHUNK shots */
  float *pos = nullptr, *mt = nullptr, *U = nullptr;
  void *x0 = nullptr, *h[NENC] = {}, *a[NDEC] = {}, *hd[NDEC] = {};
};

static void net_free(cgfd_sg_net_t *n)
{
  if (!n) return;
  void *p[] = {n->w, n->w16, n->d_err, n->pos, n->mt, n->U, n->x0};
  for (void *q : p)
    if (q) cudaFree(q);
  for (int k = 0; k < NENC; k++)
    if (n->h[k]) cudaFree(n->h[k]);
  for (int k = 0; k < NDEC; k++) {
    if (n->a[k]) cudaFree(n->a[k]);
    if (n->hd[k]) cudaFree(n->hd[k]);
  }
  if (n->st) cudaStreamDestroy(n->st);
  delete n;
}

extern "C" long long cgfd_sg_net_nparam(int nrec, int nt)
{
  if (nrec < 1 || nt < 1 || nt > T0 * (1 << NDEC)) return -1;
  return layers_of(3 * nrec).n;
}

extern "C" int cgfd_sg_net_create(int nrec, int nt, const float *params, long long nparam,
                                  float scale, cgfd_sg_net_t **out)
{
  if (!out) return net_err(CGFD_EINVAL, "sg_net_create: null output handle");
  *out = nullptr;
  const long long want = cgfd_sg_net_nparam(nrec, nt);
  if (want < 0)
    return net_err(CGFD_EINVAL, "sg_net_create: %d receivers, %d samples (1..%d samples)",
                   nrec, nt, T0 * (1 << NDEC));
  if (nrec % 4)
    return net_err(CGFD_EINVAL, "sg_net_create: %d receivers (a multiple of 4: the last "
                   "layer's 18 nrec outputs are stored in 16-byte rows)", nrec);
  if (!params || nparam != want)
    return net_err(CGFD_EINVAL, "sg_net_create: %lld parameters given, the layout has %lld",
                   nparam, want);
  if (!(scale == scale)) return net_err(CGFD_EINVAL, "sg_net_create: scale is NaN");
  cgfd_sg_net_t *n = new cgfd_sg_net_t();
  n->nrec = nrec;
  n->nt = nt;
  n->R = 3 * nrec;
  n->T = T0 * (1 << NDEC);
  n->scale = scale;
  n->L = layers_of(n->R);
  const int B = CGFD_SG_NET_CHUNK;
  cudaError_t e = cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking);
  auto alloc = [&](void **p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  alloc((void **)&n->w, (size_t)want * 4);
  alloc(&n->w16, (size_t)want * 2);
  alloc((void **)&n->d_err, 4);
  alloc((void **)&n->pos, (size_t)B * 3 * 4);
  alloc((void **)&n->mt, (size_t)B * NMT * 4);
  alloc((void **)&n->U, (size_t)B * nt * n->R * 4);
  alloc(&n->x0, (size_t)B * NFEAT * 2);
  for (int k = 0; k < NENC; k++) alloc(&n->h[k], (size_t)B * n->L.out[k] * 2);
  int tin = T0;
  for (int l = 0; l < NDEC; l++) {
    const int tout = tin * UP;
    alloc(&n->a[l], (size_t)B * tout * n->L.in[NENC + l] * 2);
    alloc(&n->hd[l], (size_t)B * tout * n->L.out[NENC + l] * 2);
    tin = tout;
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(n->d_err, 0, 4, n->st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(n->w, params, (size_t)want * 4, cudaMemcpyHostToDevice, n->st);
  if (e != cudaSuccess) {
    net_free(n);
    return net_err(e == cudaErrorMemoryAllocation ? CGFD_ENOMEM : CGFD_ECUDA,
                   "sg_net_create: %s", cudaGetErrorString(e));
  }
  int rc = cgfd_sg_to_bf16(n->w, want, n->w16, n->st);
  if (rc == 0 && cudaStreamSynchronize(n->st) != cudaSuccess)
    rc = net_err(CGFD_ECUDA, "sg_net_create: %s", cudaGetErrorString(cudaGetLastError()));
  if (rc) {
    net_free(n);
    return rc;
  }
  *out = n;
  return 0;
}

/* one chunk of nb shots already on the device: features, encoder,
 * decoder, contraction into n->U */
static int net_forward(cgfd_sg_net_t *n, int nb)
{
  const Layers &L = n->L;
  auto W = [&](int k) { return (const void *)((const char *)n->w16 + L.w[k] * 2); };
  auto bias = [&](int k) { return (const float *)(n->w + L.b[k]); };
  int rc = cgfd_sg_features(n->pos, nb, NFREQ, NFEAT, n->x0, n->st);
  const void *x = n->x0;
  int xin = NFEAT;
  for (int k = 0; k < NENC && rc == 0; k++) {
    rc = cgfd_sg_gemm(x, xin, W(k), L.in[k], n->h[k], L.out[k], nb, L.out[k], L.in[k], 1.0f,
                      bias(k), CGFD_SG_ACT_GELU, CGFD_SG_OUT_BF16, nullptr, 1, n->d_err, n->st);
    x = n->h[k];
    xin = L.out[k];
  }
  int tin = T0;
  for (int l = 0; l < NDEC && rc == 0; l++) {
    const int k = NENC + l, tout = tin * UP;
    rc = cgfd_sg_im2col_up(x, nb, tin, C0, UP, KS, n->a[l], n->st);
    if (rc) break;
    const bool last = l == NDEC - 1;
    rc = cgfd_sg_gemm(n->a[l], L.in[k], W(k), L.in[k], n->hd[l], L.out[k], nb * tout, L.out[k],
                      L.in[k], 1.0f, bias(k), last ? CGFD_SG_ACT_NONE : CGFD_SG_ACT_GELU,
                      CGFD_SG_OUT_BF16, nullptr, 1, n->d_err, n->st);
    x = n->hd[l];
    tin = tout;
  }
  if (rc == 0) rc = cgfd_sg_contract(x, n->mt, nb, n->T, n->nt, n->R, n->scale, n->U, n->st);
  return rc;
}

extern "C" int cgfd_sg_net_predict(cgfd_sg_net_t *n, int nshot, const float *pos,
                                   const float *mt, float *u)
{
  if (!n) return net_err(CGFD_EINVAL, "sg_net_predict: null network");
  if (nshot < 0 || (nshot > 0 && (!pos || !mt || !u)))
    return net_err(CGFD_EINVAL, "sg_net_predict: %d shots with a missing array", nshot);
  const size_t per = (size_t)n->nt * n->R;
  for (int b0 = 0; b0 < nshot; b0 += CGFD_SG_NET_CHUNK) {
    const int nb = nshot - b0 < CGFD_SG_NET_CHUNK ? nshot - b0 : CGFD_SG_NET_CHUNK;
    cudaError_t e = cudaMemcpyAsync(n->pos, pos + (size_t)b0 * 3, (size_t)nb * 3 * 4,
                                    cudaMemcpyHostToDevice, n->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(n->mt, mt + (size_t)b0 * NMT, (size_t)nb * NMT * 4,
                          cudaMemcpyHostToDevice, n->st);
    int rc = e == cudaSuccess ? net_forward(n, nb)
                              : net_err(CGFD_ECUDA, "sg_net_predict: %s", cudaGetErrorString(e));
    if (rc == 0) {
      e = cudaMemcpyAsync(u + (size_t)b0 * per, n->U, (size_t)nb * per * 4,
                          cudaMemcpyDeviceToHost, n->st);
      if (e != cudaSuccess)
        rc = net_err(CGFD_ECUDA, "sg_net_predict: %s", cudaGetErrorString(e));
    }
    if (rc) {
      /* nothing queued may still write into the caller's arrays */
      cudaStreamSynchronize(n->st);
      return rc;
    }
  }
  int herr = 0;
  cudaError_t e = cudaMemcpyAsync(&herr, n->d_err, 4, cudaMemcpyDeviceToHost, n->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(n->st);
  if (e != cudaSuccess) return net_err(CGFD_ECUDA, "sg_net_predict: %s", cudaGetErrorString(e));
  if (herr)
    return net_err(CGFD_ECUDA, "sg_net_predict: device wait timed out (code %d)", herr);
  return 0;
}

extern "C" void cgfd_sg_net_destroy(cgfd_sg_net_t *n) { net_free(n); }
