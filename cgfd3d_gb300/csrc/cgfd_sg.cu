/*
 * cgfd_sg.cu -- device kernels of the learned seismogram surrogate around
 * its matrix products (cgfd_sg_gemm.cu).
 *
 * The network (composed in cgfd3d_gb300/surrogate.py) maps a source
 * position to six sets of receiver Green's functions, one per moment-tensor
 * component, and contracts them with the moment tensor:
 *
 *   features   Fourier features of the normalised position   (k_features)
 *   encoder    GEMMs with bias + GELU                          (cgfd_sg_gemm)
 *   decoder    per layer: nearest 2x upsampling and a 5-tap 1-D convolution
 *              over time, as an im2col gather (k_im2col_up) and a GEMM
 *   output     G[b, t, k, r] (k: moment component, r: receiver x component)
 *              u[b, t, r] = sum_k M[b, k] G[b, t, k, r]        (k_contract)
 *
 * Training adds the loss and its gradient in the contraction (relative L2
 * misfit per shot, k_contract_loss), the adjoint of the im2col gather fused
 * with the GELU derivative (k_col2im_up_gelu), GELU derivative for the
 * encoder (k_gelu_bwd), column sums for bias gradients, transposes of the
 * operands of the weight-gradient products, and AdamW on fp32 master
 * weights with a bf16 copy for the products.  Layouts are row-major,
 * channels last ([B, T, C]); every kernel is a grid-stride loop.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>

#include "../../include/cgfd3d_gpu.h"

__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg);

namespace sg {

typedef __nv_bfloat16 bf16;

static int sg_err(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return cgfd_set_error_msg(code, buf);
}

static int launched(const char *what)
{
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return sg_err(CGFD_ECUDA, "%s: %s", what, cudaGetErrorString(e));
  return 0;
}

static inline int nblocks(long long n, int threads)
{
  long long b = (n + threads - 1) / threads;
  return (int)(b < 152 * 32 ? (b < 1 ? 1 : b) : 152 * 32);
}

#define GRID_LOOP(i, n) \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); \
       i += (long long)gridDim.x * blockDim.x)

__device__ __forceinline__ float gelu_grad(float x)
{
  const float c = 0.7978845608028654f, a = 0.044715f;
  const float u = c * (x + a * x * x * x);
  const float t = tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * a * x * x);
}

/* row b: [x, y, z, sin(pi f x), cos(pi f x) for f = 1..nfreq per coordinate,
 * zeros] -- nfeat >= 3 + 6 nfreq columns */
__global__ void k_features(const float *__restrict__ pos, int B, int nfreq, int nfeat,
                           bf16 *__restrict__ out)
{
  GRID_LOOP(i, (long long)B * nfeat)
  {
    const int b = (int)(i / nfeat), c = (int)(i % nfeat);
    float v = 0.0f;
    if (c < 3) {
      v = pos[3 * b + c];
    } else if (c < 3 + 6 * nfreq) {
      const int r = c - 3, d = r / (2 * nfreq), f = (r % (2 * nfreq)) / 2 + 1;
      const float a = 3.14159265358979f * (float)f * pos[3 * b + d];
      v = (r & 1) ? cosf(a) : sinf(a);
    }
    out[i] = __float2bfloat16_rn(v);
  }
}

/* A[(b, t), (j, c)] = X[b, (t + j - h) / up, c] for 0 <= t + j - h < Tin up,
 * else 0; h = ks / 2; X [B, Tin, C], A [B Tin up, ks C] */
__global__ void k_im2col_up(const bf16 *__restrict__ X, int B, int Tin, int C, int up, int ks,
                            bf16 *__restrict__ A)
{
  const int Tout = Tin * up, h = ks / 2;
  const long long n = (long long)B * Tout * ks * C;
  GRID_LOOP(i, n)
  {
    const int c = (int)(i % C);
    long long r = i / C;
    const int j = (int)(r % ks);
    r /= ks;
    const int t = (int)(r % Tout), b = (int)(r / Tout);
    const int tt = t + j - h;
    A[i] = (tt >= 0 && tt < Tout) ? X[((long long)b * Tin + tt / up) * C + c]
                                  : __float2bfloat16_rn(0.0f);
  }
}

/* k_im2col_up with 8 channels (16 bytes) per thread, 32-bit index math:
 * C % 8 == 0, 16-byte aligned X and A, fewer than 2^31 output vectors */
__global__ void k_im2col_up_v(const uint4 *__restrict__ X, int B, int Tin, int C8, int up,
                              int ks, uint4 *__restrict__ A)
{
  const int Tout = Tin * up, h = ks / 2;
  const unsigned segs = (unsigned)(ks * C8);
  const unsigned n = (unsigned)B * (unsigned)Tout * segs;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned row = i / segs, sg = i - row * segs;
    const int j = (int)(sg / (unsigned)C8), c8 = (int)(sg - (unsigned)j * C8);
    const int b = (int)(row / (unsigned)Tout), t = (int)(row - (unsigned)b * Tout);
    const int tt = t + j - h;
    A[i] = (tt >= 0 && tt < Tout) ? X[((size_t)b * Tin + tt / up) * C8 + c8]
                                  : make_uint4(0u, 0u, 0u, 0u);
  }
}

__device__ __forceinline__ void acc_bf16x8(float *acc, const uint4 v)
{
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int u = 0; u < 4; u++) {
    acc[2 * u] += __uint_as_float(w[u] << 16);
    acc[2 * u + 1] += __uint_as_float(w[u] & 0xffff0000u);
  }
}

/* k_col2im_up_gelu with 8 channels (16 bytes) per thread, the same
 * summation order per channel (bit-identical): C % 8 == 0, 16-byte aligned
 * arrays, fewer than 2^31 output vectors */
__global__ void k_col2im_up_gelu_v(const uint4 *__restrict__ dA, int B, int Tin, int C8, int up,
                                   int ks, const uint4 *__restrict__ Z, uint4 *__restrict__ dZ)
{
  const int Tout = Tin * up, h = ks / 2;
  const unsigned n = (unsigned)B * (unsigned)Tin * (unsigned)C8;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned r = i / (unsigned)C8;
    const int c8 = (int)(i - r * (unsigned)C8);
    const int b = (int)(r / (unsigned)Tin), s = (int)(r - (unsigned)b * Tin);
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int tt = s * up; tt < s * up + up; tt++)
      for (int j = 0; j < ks; j++) {
        const int t = tt - j + h;
        if (t < 0 || t >= Tout) continue;
        acc_bf16x8(acc, dA[(((size_t)b * Tout + t) * ks + j) * C8 + c8]);
      }
    if (Z) {
      const uint4 z = Z[i];
      const uint32_t w[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
      for (int u = 0; u < 4; u++) {
        acc[2 * u] *= gelu_grad(__uint_as_float(w[u] << 16));
        acc[2 * u + 1] *= gelu_grad(__uint_as_float(w[u] & 0xffff0000u));
      }
    }
    uint32_t o[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      __nv_bfloat162 p2 = __floats2bfloat162_rn(acc[2 * u], acc[2 * u + 1]);
      o[u] = *reinterpret_cast<uint32_t *>(&p2);
    }
    dZ[i] = make_uint4(o[0], o[1], o[2], o[3]);
  }
}

/* adjoint of k_im2col_up, times GELU'(Z): dZ[b, s, c] = GELU'(Z[b, s, c])
 * sum over (t, j) with (t + j - h) / up = s of dA[(b, t), (j, c)] (Z null:
 * no GELU factor) */
__global__ void k_col2im_up_gelu(const bf16 *__restrict__ dA, int B, int Tin, int C, int up,
                                 int ks, const bf16 *__restrict__ Z, bf16 *__restrict__ dZ)
{
  const int Tout = Tin * up, h = ks / 2;
  GRID_LOOP(i, (long long)B * Tin * C)
  {
    const int c = (int)(i % C);
    const long long r = i / C;
    const int s = (int)(r % Tin), b = (int)(r / Tin);
    float acc = 0.0f;
    for (int tt = s * up; tt < s * up + up; tt++)
      for (int j = 0; j < ks; j++) {
        const int t = tt - j + h;
        if (t < 0 || t >= Tout) continue;
        acc += __bfloat162float(dA[(((long long)b * Tout + t) * ks + j) * C + c]);
      }
    if (Z) acc *= gelu_grad(__bfloat162float(Z[i]));
    dZ[i] = __float2bfloat16_rn(acc);
  }
}

__global__ void k_gelu_bwd(const bf16 *__restrict__ dH, const bf16 *__restrict__ Z, long long n,
                           bf16 *__restrict__ dZ)
{
  GRID_LOOP(i, n)
  dZ[i] = __float2bfloat16_rn(__bfloat162float(dH[i]) * gelu_grad(__bfloat162float(Z[i])));
}

/* u[b, t, r] = scale sum_k M[b, k] G[b, t, k, r] for t < T (G holds Tg >= T
 * steps) */
__global__ void k_contract(const bf16 *__restrict__ G, const float *__restrict__ M, int B,
                           int Tg, int T, int R, float scale, float *__restrict__ U)
{
  GRID_LOOP(i, (long long)B * T * R)
  {
    const int r = (int)(i % R);
    const long long bt = i / R;
    const int t = (int)(bt % T), b = (int)(bt / T);
    const bf16 *g = G + ((long long)b * Tg + t) * 6 * R + r;
    float u = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++) u += M[6 * b + k] * __bfloat162float(g[k * R]);
    U[i] = scale * u;
  }
}

/* k_contract for 8 consecutive traces per thread (16-byte loads of G, two
 * 16-byte stores of U), the same sum per value: R % 8 == 0, aligned
 * arrays, fewer than 2^31 output vectors */
__global__ void k_contract_v(const uint4 *__restrict__ G, const float *__restrict__ M, int B,
                             int Tg, int T, int R8, float scale, float4 *__restrict__ U)
{
  const unsigned n = (unsigned)B * (unsigned)T * (unsigned)R8;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned bt = i / (unsigned)R8;
    const int r8 = (int)(i - bt * (unsigned)R8);
    const int b = (int)(bt / (unsigned)T), t = (int)(bt - (unsigned)b * T);
    const uint4 *g = G + ((size_t)b * Tg + t) * 6 * R8 + r8;
    float u[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const float mk = M[6 * b + k];
      const uint4 v = g[k * R8];
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int e = 0; e < 4; e++) {
        u[2 * e] += mk * __uint_as_float(w[e] << 16);
        u[2 * e + 1] += mk * __uint_as_float(w[e] & 0xffff0000u);
      }
    }
    U[2 * (size_t)i] = make_float4(scale * u[0], scale * u[1], scale * u[2], scale * u[3]);
    U[2 * (size_t)i + 1] = make_float4(scale * u[4], scale * u[5], scale * u[6], scale * u[7]);
  }
}

/* Training form of k_contract with the relative L2 misfit: per shot
 * err[b] += sum (u - Utrue)^2 (err zeroed by the caller), and the gradient of
 * loss = (1/B) sum_b err_b / norm_b:  dG[b, t, k, r] = M[b, k] scale 2 (u -
 * Utrue) / (B norm_b), zero for t >= T. */
__global__ void k_contract_loss(const bf16 *__restrict__ G, const float *__restrict__ M, int B,
                                int Tg, int T, int R, float scale,
                                const float *__restrict__ Utrue, const float *__restrict__ norm,
                                float *__restrict__ err, bf16 *__restrict__ dG)
{
  /* blockIdx.y: the shot; the block's squared misfits are summed in the
   * block and added to err[b] once */
  const int b = blockIdx.y;
  const long long n = (long long)Tg * R;
  float mb[6];
#pragma unroll
  for (int k = 0; k < 6; k++) mb[k] = M[6 * b + k];
  const float gscale = 2.0f * scale / ((float)B * norm[b]);
  float acc = 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % R), t = (int)(i / R);
    const long long bt = (long long)b * Tg + t;
    const bf16 *g = G + bt * 6 * R + r;
    bf16 *dg = dG + bt * 6 * R + r;
    if (t >= T) {
#pragma unroll
      for (int k = 0; k < 6; k++) dg[k * R] = __float2bfloat16_rn(0.0f);
      continue;
    }
    float u = 0.0f;
#pragma unroll
    for (int k = 0; k < 6; k++) u += mb[k] * __bfloat162float(g[k * R]);
    const float d = scale * u - Utrue[((long long)b * T + t) * R + r];
    acc += d * d;
    const float du = d * gscale;
#pragma unroll
    for (int k = 0; k < 6; k++) dg[k * R] = __float2bfloat16_rn(mb[k] * du);
  }
  __shared__ float part[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) part[warp] = acc;
  __syncthreads();
  if (warp == 0) {
    acc = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) atomicAdd(err + b, acc);
  }
}

/* Y[c, r] = X[r, c] (X rows x cols with row stride ldx; Y row stride ldy) */
__global__ void k_transpose(const bf16 *__restrict__ X, int rows, int cols, long long ldx,
                            bf16 *__restrict__ Y, long long ldy)
{
  __shared__ bf16 tile[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int r = r0 + k, c = c0 + threadIdx.x;
    tile[k][threadIdx.x] = (r < rows && c < cols) ? X[(long long)r * ldx + c]
                                                  : __float2bfloat16_rn(0.0f);
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int c = c0 + k, r = r0 + threadIdx.x;
    if (c < cols && r < rows) Y[(long long)c * ldy + r] = tile[threadIdx.x][k];
  }
}

/* k_transpose for whole 64 x 64 tiles with 16-byte loads and stores (rows
 * and cols multiples of 64, ldx and ldy multiples of 8, 16-byte aligned):
 * a warp reads 32 rows' 16-byte chunks into shared memory, then each lane
 * gathers one output row's 8 values from a tile column (consecutive lanes,
 * consecutive columns: no bank conflicts) and stores them as 16 bytes */
__global__ void __launch_bounds__(256) k_transpose64(const bf16 *__restrict__ X, long long ldx,
                                                     bf16 *__restrict__ Y, long long ldy)
{
  __shared__ __align__(16) unsigned short tile[64][72];
  const int c0 = blockIdx.x * 64, r0 = blockIdx.y * 64, t = threadIdx.x;
#pragma unroll
  for (int p = 0; p < 2; p++) {
    const int rr = (t >> 3) + 32 * p, q = t & 7;
    *reinterpret_cast<uint4 *>(&tile[rr][8 * q]) =
        *reinterpret_cast<const uint4 *>(X + (long long)(r0 + rr) * ldx + c0 + 8 * q);
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < 2; p++) {
    const int cc = (t & 31) + 32 * p, q = t >> 5;   /* output row c0 + cc, rows r0 + 8q .. */
    uint32_t w[4];
#pragma unroll
    for (int u = 0; u < 4; u++)
      w[u] = (uint32_t)tile[8 * q + 2 * u][cc] | ((uint32_t)tile[8 * q + 2 * u + 1][cc] << 16);
    *reinterpret_cast<uint4 *>(Y + (long long)(c0 + cc) * ldy + r0 + 8 * q) =
        make_uint4(w[0], w[1], w[2], w[3]);
  }
}

/* out[c] (+)= sum over rows of X[r, c] (fp32 accumulation) */
__global__ void k_colsum(const bf16 *__restrict__ X, long long rows, int cols, long long ld,
                         float *__restrict__ out)
{
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const long long per = (rows + gridDim.y - 1) / gridDim.y;
  const long long r0 = blockIdx.y * per, r1 = min(rows, r0 + per);
  float acc = 0.0f;
  for (long long r = r0; r < r1; r++) acc += __bfloat162float(X[r * ld + c]);
  atomicAdd(out + c, acc);
}

/* AdamW step on fp32 master weights, refreshing their bf16 copy */
__global__ void k_adamw(float *__restrict__ w, bf16 *__restrict__ w16,
                        const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                        long long n, float lr, float b1, float b2, float eps, float wd, float c1,
                        float c2)
{
  GRID_LOOP(i, n)
  {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = (mi / c1) / (sqrtf(vi / c2) + eps);
    const float wi = w[i] * (1.0f - lr * wd) - lr * upd;
    w[i] = wi;
    w16[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void k_f32_to_bf16(const float *__restrict__ x, long long n, bf16 *__restrict__ y)
{
  GRID_LOOP(i, n) y[i] = __float2bfloat16_rn(x[i]);
}

}  // namespace sg

using namespace sg;

#define SG_STREAM(s) ((cudaStream_t)(s))

extern "C" int cgfd_sg_features(const float *pos, int B, int nfreq, int nfeat, void *out,
                                void *stream)
{
  if (!pos || !out || B < 1 || nfreq < 0 || nfeat < 3 + 6 * nfreq)
    return sg_err(CGFD_EINVAL, "sg_features: %d shots, %d frequencies, %d features", B, nfreq,
                  nfeat);
  k_features<<<nblocks((long long)B * nfeat, 256), 256, 0, SG_STREAM(stream)>>>(
      pos, B, nfreq, nfeat, (bf16 *)out);
  return launched("sg_features");
}

extern "C" int cgfd_sg_im2col_up(const void *X, int B, int Tin, int C, int up, int ks, void *A,
                                 void *stream)
{
  if (!X || !A || B < 1 || Tin < 1 || C < 1 || up < 1 || ks < 1 || !(ks & 1))
    return sg_err(CGFD_EINVAL, "sg_im2col_up: B %d T %d C %d up %d ks %d", B, Tin, C, up, ks);
  const long long n = (long long)B * Tin * up * ks * C;
  if (C % 8 == 0 && !((uintptr_t)X & 15) && !((uintptr_t)A & 15) && n / 8 < (1LL << 31))
    k_im2col_up_v<<<nblocks(n / 8, 256), 256, 0, SG_STREAM(stream)>>>(
        (const uint4 *)X, B, Tin, C / 8, up, ks, (uint4 *)A);
  else
    k_im2col_up<<<nblocks(n, 256), 256, 0, SG_STREAM(stream)>>>((const bf16 *)X, B, Tin, C, up,
                                                                 ks, (bf16 *)A);
  return launched("sg_im2col_up");
}

extern "C" int cgfd_sg_col2im_up_gelu(const void *dA, int B, int Tin, int C, int up, int ks,
                                      const void *Z, void *dZ, void *stream)
{
  if (!dA || !dZ || B < 1 || Tin < 1 || C < 1 || up < 1 || ks < 1 || !(ks & 1))
    return sg_err(CGFD_EINVAL, "sg_col2im_up: B %d T %d C %d up %d ks %d", B, Tin, C, up, ks);
  const long long n = (long long)B * Tin * C;
  if (C % 8 == 0 && !((uintptr_t)dA & 15) && !((uintptr_t)dZ & 15) && !((uintptr_t)Z & 15) &&
      n / 8 < (1LL << 31))
    k_col2im_up_gelu_v<<<nblocks(n / 8, 256), 256, 0, SG_STREAM(stream)>>>(
        (const uint4 *)dA, B, Tin, C / 8, up, ks, (const uint4 *)Z, (uint4 *)dZ);
  else
    k_col2im_up_gelu<<<nblocks(n, 256), 256, 0, SG_STREAM(stream)>>>(
        (const bf16 *)dA, B, Tin, C, up, ks, (const bf16 *)Z, (bf16 *)dZ);
  return launched("sg_col2im_up");
}

extern "C" int cgfd_sg_gelu_bwd(const void *dH, const void *Z, long long n, void *dZ,
                                void *stream)
{
  if (!dH || !Z || !dZ || n < 0) return sg_err(CGFD_EINVAL, "sg_gelu_bwd: bad arguments");
  if (n == 0) return 0;
  k_gelu_bwd<<<nblocks(n, 256), 256, 0, SG_STREAM(stream)>>>((const bf16 *)dH, (const bf16 *)Z,
                                                              n, (bf16 *)dZ);
  return launched("sg_gelu_bwd");
}

extern "C" int cgfd_sg_contract(const void *G, const float *M, int B, int Tg, int T, int R,
                                float scale, float *U, void *stream)
{
  if (!G || !M || !U || B < 1 || T < 1 || Tg < T || R < 1)
    return sg_err(CGFD_EINVAL, "sg_contract: B %d Tg %d T %d R %d", B, Tg, T, R);
  const long long n = (long long)B * T * R;
  if (R % 8 == 0 && !((uintptr_t)G & 15) && !((uintptr_t)U & 15) && n / 8 < (1LL << 31))
    k_contract_v<<<nblocks(n / 8, 256), 256, 0, SG_STREAM(stream)>>>(
        (const uint4 *)G, M, B, Tg, T, R / 8, scale, (float4 *)U);
  else
    k_contract<<<nblocks(n, 256), 256, 0, SG_STREAM(stream)>>>((const bf16 *)G, M, B, Tg, T, R,
                                                                scale, U);
  return launched("sg_contract");
}

extern "C" int cgfd_sg_contract_loss(const void *G, const float *M, int B, int Tg, int T, int R,
                                     float scale, const float *Utrue, const float *norm,
                                     float *err, void *dG, void *stream)
{
  if (!G || !M || !Utrue || !norm || !err || !dG || B < 1 || T < 1 || Tg < T || R < 1)
    return sg_err(CGFD_EINVAL, "sg_contract_loss: B %d Tg %d T %d R %d", B, Tg, T, R);
  if (B > 65535) return sg_err(CGFD_EINVAL, "sg_contract_loss: %d shots (65535 at most)", B);
  const long long per = (long long)Tg * R;
  int bx = (int)((per + 255) / 256);
  const int cap = (152 * 16 + B - 1) / B;
  bx = bx < 1 ? 1 : (bx > cap ? cap : bx);
  k_contract_loss<<<dim3(bx, B), 256, 0, SG_STREAM(stream)>>>(
      (const bf16 *)G, M, B, Tg, T, R, scale, Utrue, norm, err, (bf16 *)dG);
  return launched("sg_contract_loss");
}

extern "C" int cgfd_sg_transpose(const void *X, int rows, int cols, long long ldx, void *Y,
                                 long long ldy, void *stream)
{
  if (!X || !Y || rows < 1 || cols < 1 || ldx < cols || ldy < rows)
    return sg_err(CGFD_EINVAL, "sg_transpose: %d x %d (ld %lld, %lld)", rows, cols, ldx, ldy);
  if (rows % 64 == 0 && cols % 64 == 0 && ldx % 8 == 0 && ldy % 8 == 0 &&
      !((uintptr_t)X & 15) && !((uintptr_t)Y & 15) && cols / 64 < 65536 && rows / 64 < 65536) {
    k_transpose64<<<dim3(cols / 64, rows / 64), 256, 0, SG_STREAM(stream)>>>((const bf16 *)X, ldx,
                                                                           (bf16 *)Y, ldy);
  } else {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
    k_transpose<<<grid, block, 0, SG_STREAM(stream)>>>((const bf16 *)X, rows, cols, ldx,
                                                       (bf16 *)Y, ldy);
  }
  return launched("sg_transpose");
}

extern "C" int cgfd_sg_colsum(const void *X, long long rows, int cols, long long ld, float *out,
                              void *stream)
{
  if (!X || !out || rows < 1 || cols < 1 || ld < cols)
    return sg_err(CGFD_EINVAL, "sg_colsum: %lld x %d", rows, cols);
  const int bx = (cols + 127) / 128;
  long long by = (rows + 511) / 512;
  if (by > 1024) by = 1024;
  k_colsum<<<dim3(bx, (unsigned)by), 128, 0, SG_STREAM(stream)>>>((const bf16 *)X, rows, cols,
                                                                   ld, out);
  return launched("sg_colsum");
}

extern "C" int cgfd_sg_adamw(float *w, void *w16, const float *g, float *m, float *v,
                             long long n, float lr, float b1, float b2, float eps, float wd,
                             int step, void *stream)
{
  if (!w || !w16 || !g || !m || !v || n < 1 || step < 1)
    return sg_err(CGFD_EINVAL, "sg_adamw: bad arguments");
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_adamw<<<nblocks(n, 256), 256, 0, SG_STREAM(stream)>>>(w, (bf16 *)w16, g, m, v, n, lr, b1, b2,
                                                          eps, wd, c1, c2);
  return launched("sg_adamw");
}

extern "C" int cgfd_sg_to_bf16(const float *x, long long n, void *y, void *stream)
{
  if (!x || !y || n < 0) return sg_err(CGFD_EINVAL, "sg_to_bf16: bad arguments");
  if (n == 0) return 0;
  k_f32_to_bf16<<<nblocks(n, 256), 256, 0, SG_STREAM(stream)>>>(x, n, (bf16 *)y);
  return launched("sg_to_bf16");
}
