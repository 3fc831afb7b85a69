/*
 * cgfd_media_layer.cu -- an elastic isotropic layered model discretised on
 * a curvilinear grid on the device, with the reference's "loc" method.
 *
 * The reference evaluates every grid point on the host
 * (media_layer2model_el_iso, media/media_layer2model.cpp:140-190, 422-560,
 * 1334-1384): the elevation of each interface interpolated bilinearly at the
 * point's (x, y) on the interfaces' uniform mesh
 * (media/media_utility.cpp:173-209), the layer whose top interface is the
 * lowest one at or above the point (:88-110), each property's value plus
 * gradient x (depth below that interface)^power, the mean with the layer
 * above for points on an interface (:119-140), then mu = vs^2 rho and
 * lambda = vp^2 rho - 2 mu.  Here one thread does one point in the same
 * float/double order; the file is compiled with --fmad=false.
 */
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "../../include/cgfd3d_gpu.h"

#define LAY_MAX 64

__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg);

static int lay_err(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return cgfd_set_error_msg(code, buf);
}

struct LayerMesh {
  int NI, NX, NY;
  float MINX, MINY, DX, DY;
  const float *rec;     /* [NI][NY][NX][10] */
};

__device__ float lay_bilinear(const LayerMesh &L, int col, int layer, float xq, float yq)
{
  const float x0 = L.MINX, x1 = L.MINX + L.DX, y0 = L.MINY, y1 = L.MINY + L.DY;
  int ix = (int)((xq - x0) / (x1 - x0));
  int iy = (int)((yq - y0) / (y1 - y0));
  if (ix < 0 || iy < 0) return FLT_MAX;
  /* the caller keeps (xq, yq) inside the mesh; an index rounded past its
   * last point is held there (the reference would read past its arrays) */
  ix = ix > L.NX - 1 ? L.NX - 1 : ix;
  iy = iy > L.NY - 1 ? L.NY - 1 : iy;
  const float *v = L.rec + (size_t)layer * L.NX * L.NY * 10 + col;
  const int indx = iy * L.NX + ix;
  if (ix == L.NX - 1 || iy == L.NY - 1) return v[indx * 10];
  const float xa = L.MINX + L.DX * ix, xb = L.MINX + L.DX * (ix + 1);
  const float ya = L.MINY + L.DY * iy, yb = L.MINY + L.DY * (iy + 1);
  const float area = (xb - xa) * (yb - ya);
  float vq = v[indx * 10] * (xb - xq) * (yb - yq) + v[(indx + 1) * 10] * (xq - xa) * (yb - yq) +
             v[(indx + L.NX) * 10] * (xb - xq) * (yq - ya) +
             v[(indx + 1 + L.NX) * 10] * (xq - xa) * (yq - ya);
  vq /= area;
  return vq;
}

__device__ int lay_last_ge(float value, const float *x, int n)
{
  if (value > x[0]) return -1;
  float dist = FLT_MAX;
  int indx = -1;
  for (int i = 0; i < n; i++) {
    if (x[i] == -FLT_MAX) continue;
    const float d = x[i] - value;
    if (d < 0) break;
    if (d >= 0 && d <= dist) { dist = d; indx = i; }
  }
  return indx;
}

__device__ int lay_first_ge(float value, const float *x, int n)
{
  float dist = FLT_MAX;
  int idx = -1;
  for (int i = 0; i < n; i++) {
    if (x[i] == -FLT_MAX) continue;
    const float d = x[i] - value;
    if (d >= 0 && d <= dist) {
      if (d <= 1e-6) return i;
      dist = d;
      idx = i;
    }
  }
  return idx;
}

/* value + pow(dz, power) * gradient of property column c of a layer */
__device__ float lay_value(const LayerMesh &L, int layer, int c, float dz, float x, float y)
{
  const float v = lay_bilinear(L, c, layer, x, y);
  const float g = lay_bilinear(L, c + 1, layer, x, y);
  const float pw = lay_bilinear(L, c + 2, layer, x, y);
  return (float)((double)v + pow((double)dz, (double)pw) * (double)g);
}

__global__ void k_layer_el_iso_loc(LayerMesh L, long long vol, const float *__restrict__ x3d,
                                   const float *__restrict__ y3d,
                                   const float *__restrict__ z3d, float *lam, float *mu,
                                   float *rho, int *bad)
{
  const float maxx = L.MINX + (L.NX - 1) * L.DX, maxy = L.MINY + (L.NY - 1) * L.DY;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < vol;
       q += (long long)gridDim.x * blockDim.x) {
    const float x = x3d[q], y = y3d[q], z = z3d[q];
    if (x < L.MINX || x > maxx || y < L.MINY || y > maxy) {
      atomicOr(bad, 1);
      continue;
    }
    float elev[LAY_MAX];
    for (int n = 0; n < L.NI; n++) elev[n] = lay_bilinear(L, 0, n, x, y);
    int mi = lay_last_ge(z, elev, L.NI);
    float r, vp, vs;
    if (mi == -1) {
      mi = lay_last_ge(elev[0], elev, L.NI);
      r = lay_bilinear(L, 1, mi, x, y);
      vp = lay_bilinear(L, 4, mi, x, y);
      vs = lay_bilinear(L, 7, mi, x, y);
    } else {
      const float dz = elev[mi] - z;
      vp = lay_value(L, mi, 4, dz, x, y);
      vs = lay_value(L, mi, 7, dz, x, y);
      r = lay_value(L, mi, 1, dz, x, y);
      if ((double)vp <= (double)vs * sqrt(2.0)) {
        atomicOr(bad, 2);
        continue;
      }
      if (fabsf(dz - 0.0f) < FLT_EPSILON) {
        const int m2 = lay_first_ge(z, elev, L.NI) - 1;
        if (m2 >= 0) {
          const float dz2 = elev[m2] - z;
          const float vp_top = lay_value(L, m2, 4, dz2, x, y);
          const float vs_top = lay_value(L, m2, 7, dz2, x, y);
          const float rho_top = lay_value(L, m2, 1, dz2, x, y);
          r = (float)((double)(r + rho_top) / 2.0);
          vp = (float)((double)(vp + vp_top) / 2.0);
          vs = (float)((double)(vs + vs_top) / 2.0);
        }
      }
    }
    const float m = vs * vs * r;
    mu[q] = m;
    lam[q] = (float)((double)(vp * vp * r) - 2.0 * (double)m);
    rho[q] = r;
  }
}

extern "C" int cgfd_media_layer_el_iso(int NI, int NX, int NY, float MINX, float MINY,
                                       float DX, float DY, const float *rec, int nx, int ny,
                                       int nz, const float *x3d, const float *y3d,
                                       const float *z3d, float *lam, float *mu, float *rho)
{
  if (NI < 1 || NI > LAY_MAX || NX < 2 || NY < 2 || !(DX > 0) || !(DY > 0))
    return lay_err(CGFD_EINVAL, "layered model: %d interfaces on a %dx%d mesh (1..%d "
                   "interfaces, at least 2x2 points, positive spacing)", NI, NX, NY, LAY_MAX);
  if (!rec || !x3d || !y3d || !z3d || !lam || !mu || !rho || nx < 1 || ny < 1 || nz < 1)
    return lay_err(CGFD_EINVAL, "layered model: missing array or empty grid");
  const size_t vol = (size_t)nx * ny * nz, nrec = (size_t)NI * NX * NY * 10;
  float *d = nullptr;
  int *d_bad = nullptr, bad = 0;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d, (6 * vol + nrec) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_bad, sizeof(int));
  float *dx = d, *dy = d + vol, *dz = d + 2 * vol, *dl = d + 3 * vol, *dm = d + 4 * vol,
        *dr = d + 5 * vol, *drec = d + 6 * vol;
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(drec, rec, nrec * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    LayerMesh L = {NI, NX, NY, MINX, MINY, DX, DY, drec};
    k_layer_el_iso_loc<<<152 * 8, 256, 0, st>>>(L, (long long)vol, dx, dy, dz, dl, dm, dr,
                                                 d_bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(lam, dl, vol * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(mu, dm, vol * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(rho, dr, vol * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d) cudaFree(d);
  if (d_bad) cudaFree(d_bad);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess)
    return lay_err(CGFD_ECUDA, "layered model: %s", cudaGetErrorString(e));
  if (bad & 1) return lay_err(CGFD_EINVAL, "layered model: a grid point lies outside the "
                              "interfaces' mesh");
  if (bad & 2) return lay_err(CGFD_EINVAL, "layered model: vp <= sqrt(2) vs at a grid point");
  return 0;
}
