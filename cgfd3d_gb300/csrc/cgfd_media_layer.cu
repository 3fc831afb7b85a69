/*
 * cgfd_media_layer.cu -- layered models (elastic isotropic and the three
 * elastic VTI parametrisations) discretised on a curvilinear grid on the
 * device, with the reference's equivalent-medium methods "loc", "har" and
 * "ari".
 *
 * The reference evaluates every grid point on the host
 * (media_layer2model_el_iso / _el_vti, media/media_layer2model.cpp:140-247,
 * 422-830, 1334-1438): the elevation of each interface interpolated
 * bilinearly at the point's (x, y) on the interfaces' uniform mesh
 * (media/media_utility.cpp:173-209), the layer whose top interface is the
 * lowest one at or above the point (:88-110), each property's value plus
 * gradient x (depth below that interface)^power, the mean with the layer
 * above for points on an interface (:119-140), then the medium: mu = vs^2
 * rho and lambda = vp^2 rho - 2 mu (isotropic) or the VTI stiffness of the
 * parametrisation (para2vti, media/media_utility.cpp:827-882).  Here one
 * thread does one point in the same float/double order; the file is
 * compiled with --fmad=false.
 *
 * The "har" and "ari" methods (media/media_layer2model.cpp:1984-2436) start
 * from "loc" and recompute each interior point whose cell -- the hexahedron
 * of the eight half-grid points (cell centres, media/media_utility.cpp:
 * 656-760) around it -- touches more than one layer: the cell is sampled at
 * 9^3 points (media/media_utility.cpp:627-654) and rho is averaged
 * arithmetically, the moduli harmonically ("har": kappa and mu, or c11 c13
 * c33 c55 c66) or arithmetically ("ari").  Here k_layer_mark gives every
 * half-grid point its layer, k_layer_mixed lists the points whose eight cell
 * vertices disagree, and k_layer_avg gives each listed point to one thread,
 * which adds its samples into the running sums in the reference's sample
 * order, so the float sums round as the reference's do.
 */
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

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

/* media kinds, with the reference's numbers (media/media_utility.hpp:40-43) */
#define LAY_ISO 21          /* rho vp vs */
#define LAY_VTI_PREM 22     /* rho vph vpv vsh vsv eta */
#define LAY_VTI_THOMSEN 23  /* rho vp0 vs0 epsilon delta gamma */
#define LAY_VTI_CIJ 24      /* rho c11 c33 c55 c66 c13 */

template <int KIND> struct LayKind {
  static constexpr int np = KIND == LAY_ISO ? 3 : 6;   /* properties per point */
  static constexpr int nout = np;                      /* output volumes */
};

/* Bounds self-checks of the kernels: an index out of its range records a
 * code in the call's check word (`chk`, device memory of that call alone)
 * and the access is skipped; the host reports a non-zero code as an
 * internal error (1 layer index, 2 listed point, 3 list position). */
struct LayerMesh {
  int NI, NX, NY, nc;   /* nc: record width, 1 + 3 x properties */
  float MINX, MINY, DX, DY;
  const float *rec;     /* [NI][NY][NX][nc] */
  int *chk;             /* the call's check word */
};

struct LayOut {
  float *v[6];          /* lambda mu rho, or c11 c33 c55 c66 c13 rho */
};

/* Bilinear interpolation on the interfaces' mesh (BilinearInterpolation,
 * media/media_utility.cpp:173-209), split in two: the cell and the weight
 * differences of a point, computed once, then the interpolation of any
 * column of any layer there -- the reference computes the same cell and
 * differences for every column, so the values are the same bits. */
struct LayW {
  int indx, edge, ok;
  float wxb, wxa, wyb, wya, area;
};

__device__ LayW lay_weights(const LayerMesh &L, float xq, float yq)
{
  LayW w;
  const float x0 = L.MINX, x1 = L.MINX + L.DX, y0 = L.MINY, y1 = L.MINY + L.DY;
  int ix = (int)((xq - x0) / (x1 - x0));
  int iy = (int)((yq - y0) / (y1 - y0));
  w.ok = !(ix < 0 || iy < 0);
  /* the caller keeps (xq, yq) inside the mesh; an index rounded past its
   * last point is held there (the reference would read past its arrays) */
  ix = ix < 0 ? 0 : ix > L.NX - 1 ? L.NX - 1 : ix;
  iy = iy < 0 ? 0 : iy > L.NY - 1 ? L.NY - 1 : iy;
  w.indx = iy * L.NX + ix;
  w.edge = ix == L.NX - 1 || iy == L.NY - 1;
  const float xa = L.MINX + L.DX * ix, xb = L.MINX + L.DX * (ix + 1);
  const float ya = L.MINY + L.DY * iy, yb = L.MINY + L.DY * (iy + 1);
  w.wxb = xb - xq;
  w.wxa = xq - xa;
  w.wyb = yb - yq;
  w.wya = yq - ya;
  w.area = (xb - xa) * (yb - ya);
  return w;
}

__device__ float lay_interp(const LayerMesh &L, const LayW &w, int col, int layer)
{
  if (!w.ok) return FLT_MAX;
  if (layer < 0 || layer >= L.NI || col < 0 || col >= L.nc) {
    atomicExch(L.chk, 1);
    return FLT_MAX;
  }
  const int nc = L.nc;
  const float *v = L.rec + (size_t)layer * L.NX * L.NY * nc + col;
  const int indx = w.indx;
  if (w.edge) return v[indx * nc];
  float vq = v[indx * nc] * w.wxb * w.wyb + v[(indx + 1) * nc] * w.wxa * w.wyb +
             v[(indx + L.NX) * nc] * w.wxb * w.wya + v[(indx + 1 + L.NX) * nc] * w.wxa * w.wya;
  vq /= w.area;
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

/* value + pow(dz, power) * gradient of property p of a layer, in
 * double as the reference's std::pow(float, float) promotes.  Two cases skip
 * the double pow and give the same bits: pow(dz, 1) is dz, and dz * g of two
 * floats is exact in double, so one double fma rounds v + dz g as the
 * reference's multiply-then-add does; a zero gradient with a power in [0, 8]
 * (pow finite for any float dz >= 0) adds a zero of the gradient's sign,
 * which the float add v + g gives exactly. */
__device__ float lay_value(const LayerMesh &L, const LayW &w, int layer, int p, float dz)
{
  const int c = 1 + 3 * p;
  const float v = lay_interp(L, w, c, layer);
  const float g = lay_interp(L, w, c + 1, layer);
  const float pw = lay_interp(L, w, c + 2, layer);
  if (pw == 1.0f) return (float)fma((double)dz, (double)g, (double)v);
  if (g == 0.0f && pw >= 0.0f && pw <= 8.0f) return v + g;
  return (float)((double)v + pow((double)dz, (double)pw) * (double)g);
}

/* vp <= sqrt(2) vs, compared in double as the reference does; a float
 * product within 2^-20 of the double one decides all but the points within
 * that margin, which take the double comparison. */
__device__ bool lay_vp_low(float vp, float vs)
{
  const float t = vs * 1.41421356f, mg = fabsf(t) * 0x1p-20f;
  if (vp > t + mg) return false;
  if (vp < t - mg) return true;
  return (double)vp <= (double)vs * sqrt(2.0);
}

/* lambda = vp vp rho - 2.0 mu as the reference rounds it (the float product
 * minus 2 mu in double, then to float).  The double difference of two floats
 * is exact, or the smaller is below 2^-28 of the larger and both roundings
 * give the larger: the float subtraction gives the same bits while 2 mu is
 * finite in float. */
__device__ float lay_lambda(float vp, float r, float m)
{
  const float a = vp * vp * r;
  if (fabsf(m) < 1e37f) return a - 2.0f * m;
  return (float)((double)a - 2.0 * (double)m);
}

/* the properties of one point (AssignLayerMediaPara2Point with
 * CalPointValue_layer, media/media_layer2model.cpp:422-830): var[0..np-1]
 * in the record's order; 0, or 1 outside the mesh, 2 where an isotropic
 * point has vp <= sqrt(2) vs (the reference exits on both). */
template <int KIND>
__device__ int lay_point(const LayerMesh &L, float x, float y, float z, float *elev, float *var)
{
  constexpr int NP = LayKind<KIND>::np;
  const float maxx = L.MINX + (L.NX - 1) * L.DX, maxy = L.MINY + (L.NY - 1) * L.DY;
  if (x < L.MINX || x > maxx || y < L.MINY || y > maxy) return 1;
  const LayW w = lay_weights(L, x, y);
  for (int n = 0; n < L.NI; n++) elev[n] = lay_interp(L, w, 0, n);
  int mi = lay_last_ge(z, elev, L.NI);
  if (mi == -1) {
    mi = lay_last_ge(elev[0], elev, L.NI);
    if (mi < 0) return 1;   /* only a NaN elevation or coordinate gets here */
#pragma unroll
    for (int p = 0; p < NP; p++) var[p] = lay_interp(L, w, 1 + 3 * p, mi);
    return 0;
  }
  const float dz = elev[mi] - z;
#pragma unroll
  for (int p = 0; p < NP; p++) var[p] = lay_value(L, w, mi, p, dz);
  if (KIND == LAY_ISO && lay_vp_low(var[1], var[2])) return 2;
  if (fabsf(dz - 0.0f) < FLT_EPSILON) {
    const int m2 = lay_first_ge(z, elev, L.NI) - 1;
    if (m2 >= 0) {
      /* the layer above at its own interface's depth, except for
       * elastic_vti_cij models, whose branch of the reference keeps the
       * point's dz (media/media_layer2model.cpp:742-774; the others
       * recompute it, :617, :690) */
      const float dz2 = KIND == LAY_VTI_CIJ ? dz : elev[m2] - z;
#pragma unroll
      for (int p = 0; p < NP; p++) {
        const float top = lay_value(L, w, m2, p, dz2);
        var[p] = (float)((double)(var[p] + top) / 2.0);
      }
    }
  }
  return 0;
}

/* VTI stiffness c11 c33 c55 c66 c13 rho of a point's parameters (para2vti,
 * media/media_utility.cpp:827-882), in the reference's float/double order */
template <int KIND> __device__ void lay_para2vti(const float *var, float *c)
{
  if (KIND == LAY_VTI_PREM) {
    const float vph = var[1], vpv = var[2], vsh = var[3], vsv = var[4], rho = var[0];
    const float eta = var[5];
    c[0] = vph * vph * rho;
    c[1] = vpv * vpv * rho;
    c[3] = vsh * vsh * rho;
    c[2] = vsv * vsv * rho;
    c[5] = rho;
    c[4] = (float)((double)eta * ((double)c[0] - 2.0 * (double)c[2]));
  } else if (KIND == LAY_VTI_THOMSEN) {
    const float rho = var[0], vp0 = var[1], vs0 = var[2], epsil = var[3], delta = var[4];
    const float gamma = var[5];
    const float c33 = vp0 * vp0 * rho, c55 = vs0 * vs0 * rho;
    const float d = c33 - c55;
    c[5] = rho;
    c[1] = c33;
    c[2] = c55;
    c[3] = (float)(2.0 * (double)gamma * (double)c55 + (double)c55);
    c[0] = (float)(2.0 * (double)epsil * (double)c33 + (double)c33);
    c[4] = (float)(sqrt(2.0 * (double)delta * (double)c33 * (double)d + (double)(d * d)) -
                   (double)c55);
  } else {
    c[0] = var[1];
    c[1] = var[2];
    c[2] = var[3];
    c[3] = var[4];
    c[4] = var[5];
    c[5] = var[0];
  }
}

template <int KIND>
__global__ void k_layer_loc(LayerMesh L, long long vol, const float *__restrict__ x3d,
                            const float *__restrict__ y3d, const float *__restrict__ z3d,
                            LayOut out, int *bad)
{
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < vol;
       q += (long long)gridDim.x * blockDim.x) {
    float elev[LAY_MAX], var[6];
    const int st = lay_point<KIND>(L, x3d[q], y3d[q], z3d[q], elev, var);
    if (st) {
      atomicOr(bad, st);
      continue;
    }
    if (KIND == LAY_ISO) {
      const float m = var[2] * var[2] * var[0];
      out.v[1][q] = m;
      out.v[0][q] = lay_lambda(var[1], var[0], m);
      out.v[2][q] = var[0];
    } else {
      float c[6];
      lay_para2vti<KIND>(var, c);
#pragma unroll
      for (int n = 0; n < 6; n++) out.v[n][q] = c[n];
    }
  }
}

/* half-grid coordinate at q (i, j, k): the mean of the cell's eight corners
 * above q, or the grid point itself on the last index of an axis */
__device__ float lay_half(const float *__restrict__ G, long long q, int i, int j, int k, int nx,
                          int ny, int nz)
{
  if (i >= nx - 1 || j >= ny - 1 || k >= nz - 1) return G[q];
  const long long line = nx, sl = (long long)nx * ny;
  const float s = G[q] + G[q + 1] + G[q + line + 1] + G[q + line] + G[q + sl] + G[q + sl + 1] +
                  G[q + sl + line + 1] + G[q + line + sl];
  return (float)((double)s / 8.0);
}

/* layer number of every half-grid point (MarkInterfaceNumber,
 * media/media_layer2model.cpp:1515-1598) */
__global__ void k_layer_mark(LayerMesh L, int nx, int ny, int nz, const float *__restrict__ x3d,
                             const float *__restrict__ y3d, const float *__restrict__ z3d,
                             signed char *mat)
{
  const long long vol = (long long)nx * ny * nz;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < vol;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / ((long long)nx * ny));
    const float hx = lay_half(x3d, q, i, j, k, nx, ny, nz);
    const float hy = lay_half(y3d, q, i, j, k, nx, ny, nz);
    const float hz = lay_half(z3d, q, i, j, k, nx, ny, nz);
    float elev[LAY_MAX];
    const LayW w = lay_weights(L, hx, hy);
    for (int n = 0; n < L.NI; n++) elev[n] = lay_interp(L, w, 0, n);
    int mi = lay_last_ge(hz, elev, L.NI);
    if (mi == -1) mi = lay_last_ge(elev[0], elev, L.NI);
    mat[q] = (signed char)mi;
  }
}

/* interior points whose eight cell vertices hold more than one layer (and
 * none -1: NumOfValues, media/media_utility.cpp:610-624) */
__global__ void k_layer_mixed(int nx, int ny, int nz, const signed char *__restrict__ mat,
                              long long *list, unsigned long long *count, int *chk)
{
  const long long vol = (long long)nx * ny * nz, line = nx, sl = (long long)nx * ny;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < vol;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx), j = (int)((q / nx) % ny), k = (int)(q / sl);
    if (i < 1 || i > nx - 2 || j < 1 || j > ny - 2 || k < 1 || k > nz - 2) continue;
    const int v[8] = {mat[q - 1 - line - sl], mat[q - line - sl], mat[q - sl], mat[q - 1 - sl],
                      mat[q - 1 - line], mat[q - line], mat[q], mat[q - 1]};
    unsigned long long seen = 0ull;   /* layer numbers are below LAY_MAX = 64 */
    int num = 0, neg = 0;
    for (int n = 0; n < 8; n++) {
      if (v[n] < 0) { neg = 1; break; }
      const unsigned long long bit = 1ull << v[n];
      if (!(seen & bit)) { seen |= bit; num++; }
    }
    if (!neg && num > 1) {
      const unsigned long long at = atomicAdd(count, 1ull);
      if (at < (unsigned long long)vol)
        list[at] = q;
      else
        atomicExch(chk, 3);
    }
  }
}

#define LAY_NG 8
#define LAY_NSG ((LAY_NG + 1) * (LAY_NG + 1) * (LAY_NG + 1))

/* one coordinate of sample (fi, fj, fk) of a cell from its eight vertices'
 * coordinates v0..v7 (MeshSubdivide, media/media_utility.cpp:627-654) */
__device__ __forceinline__ float lay_sub(float v0, float v1, float v2, float v3, float v4,
                                         float v5, float v6, float v7, float fi, float fj,
                                         float fk)
{
  const float ng = (float)LAY_NG;
  const float ly00 = v0 + (v1 - v0) / ng * fj;
  const float ly10 = v3 + (v2 - v3) / ng * fj;
  const float ly01 = v4 + (v5 - v4) / ng * fj;
  const float ly11 = v7 + (v6 - v7) / ng * fj;
  const float lxy0 = ly00 + (ly10 - ly00) / ng * fi;
  const float lxy1 = ly01 + (ly11 - ly01) / ng * fi;
  return lxy0 + (lxy1 - lxy0) / ng * fk;
}

/* a point's equivalent medium from 9^3 samples of its cell, one thread per
 * listed point (every thread runs the same 729 samples, so a warp stays
 * converged but for the layer lookups).  method 1: har, 2: ari
 * (media/media_layer2model.cpp:1984-2436); elastic isotropic and VTI
 * media. */
template <int KIND>
__global__ void __launch_bounds__(128) k_layer_avg(LayerMesh L, int method, int nx, int ny,
                                                   int nz, const float *__restrict__ x3d,
                                                   const float *__restrict__ y3d,
                                                   const float *__restrict__ z3d,
                                                   const long long *__restrict__ list,
                                                   const unsigned long long *count, LayOut out,
                                                   int *bad)
{
  const long long nlist = (long long)*count, line = nx, sl = (long long)nx * ny;
  for (long long w = blockIdx.x * (long long)blockDim.x + threadIdx.x; w < nlist;
       w += (long long)gridDim.x * blockDim.x) {
    const long long q = list[w];
    const long long vol = sl * nz;
    if (q < 1 + line + sl || q >= vol) {
      atomicExch(L.chk, 2);
      continue;
    }
    /* the cell's eight half-grid vertices, in the reference's order */
    const long long c[8] = {q - 1 - line - sl, q - 1 - sl, q - sl, q - line - sl,
                            q - 1 - line, q - 1, q, q - line};
    float vx[8], vy[8], vz[8];
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const long long p = c[n];
      const int i = (int)(p % nx), j = (int)((p / nx) % ny), k = (int)(p / sl);
      vx[n] = lay_half(x3d, p, i, j, k, nx, ny, nz);
      vy[n] = lay_half(y3d, p, i, j, k, nx, ny, nz);
      vz[n] = lay_half(z3d, p, i, j, k, nx, ny, nz);
    }
    /* isotropic: s[0] rho, s[1] kappa or lambda, s[2] mu;
     * VTI: s[0..4] c11 c33 c55 c66 c13, s[5] rho */
    float s[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    int st = 0;
    for (int kk = 0; kk <= LAY_NG; kk++)
      for (int jj = 0; jj <= LAY_NG; jj++)
        for (int ii = 0; ii <= LAY_NG; ii++) {
          const float fi = (float)ii, fj = (float)jj, fk = (float)kk;
          const float px = lay_sub(vx[0], vx[1], vx[2], vx[3], vx[4], vx[5], vx[6], vx[7], fi,
                                   fj, fk);
          const float py = lay_sub(vy[0], vy[1], vy[2], vy[3], vy[4], vy[5], vy[6], vy[7], fi,
                                   fj, fk);
          const float pz = lay_sub(vz[0], vz[1], vz[2], vz[3], vz[4], vz[5], vz[6], vz[7], fi,
                                   fj, fk);
          float elev[LAY_MAX], var[6] = {1.f, 1.f, 1.f, 1.f, 1.f, 1.f};
          st |= lay_point<KIND>(L, px, py, pz, elev, var);
          if (KIND == LAY_ISO) {
            const float m = var[2] * var[2] * var[0];
            const float lambda = lay_lambda(var[1], var[0], m);
            s[0] = s[0] + var[0];
            if (method == 1) {
              s[1] = (float)((double)s[1] + 1.0 / ((double)lambda + 2.0 / 3.0 * (double)m));
              s[2] = (float)((double)s[2] + 1.0 / (double)m);
            } else {
              s[1] = s[1] + lambda;
              s[2] = s[2] + m;
            }
          } else {
            float cp[6];
            lay_para2vti<KIND>(var, cp);
            if (method == 1) {
#pragma unroll
              for (int n = 0; n < 5; n++) s[n] = (float)((double)s[n] + 1.0 / (double)cp[n]);
            } else {
#pragma unroll
              for (int n = 0; n < 5; n++) s[n] = s[n] + cp[n];
            }
            s[5] = s[5] + cp[5];
          }
        }
    if (st) {
      atomicOr(bad, st);
    } else if (KIND == LAY_ISO && method == 1) {
      const float hm = (float)((double)LAY_NSG / (double)s[2]);
      const float hk = (float)((double)LAY_NSG / (double)s[1]);
      out.v[0][q] = (float)((double)hk - 2.0 / 3.0 * (double)hm);
      out.v[1][q] = hm;
      out.v[2][q] = (float)((double)s[0] / (double)LAY_NSG);
    } else if (KIND == LAY_ISO) {
      out.v[0][q] = (float)((double)s[1] / (double)LAY_NSG);
      out.v[1][q] = (float)((double)s[2] / (double)LAY_NSG);
      out.v[2][q] = (float)((double)s[0] / (double)LAY_NSG);
    } else {
      /* the VTI branches divide the float sums by the int count in float */
#pragma unroll
      for (int n = 0; n < 5; n++)
        out.v[n][q] = method == 1 ? (float)((double)LAY_NSG / (double)s[n])
                                  : s[n] / (float)LAY_NSG;
      out.v[5][q] = s[5] / (float)LAY_NSG;
    }
  }
}

/* ---- 3-D grid models (.md3grd), elastic isotropic ----------------------
 * NI grid levels (the "interfaces" of LayerMesh, nc = 4: elevation, rho, vp,
 * vs) in NL layers; start[l] is the first level of layer l
 * (media/media_grid2model.cpp:424-556, 1269-1356, 1819-2079). */
struct GridLayers {
  int NL;
  int start[LAY_MAX];
};

__device__ bool grd_is_start(const GridLayers &G, int mi)
{
  for (int l = 1; l < G.NL; l++)
    if (G.start[l] == mi) return true;
  return false;
}

/* the parameters at a point (rho vp vs, or the six of a VTI type), linear
 * between the two levels around it (AssignGridMediaPara2Point with
 * CalPointValue_grid); on: the point lies on a layer's top level.  0, or 1
 * outside the mesh, 2 for an isotropic point with vp <= sqrt(2) vs. */
template <int KIND>
__device__ int grd_point(const LayerMesh &L, const GridLayers &G, float x, float y, float z,
                         float *elev, float *var, int &on)
{
  constexpr int NP = LayKind<KIND>::np;
  const float maxx = L.MINX + (L.NX - 1) * L.DX, maxy = L.MINY + (L.NY - 1) * L.DY;
  on = 0;
  if (x < L.MINX || x > maxx || y < L.MINY || y > maxy) return 1;
  const LayW w = lay_weights(L, x, y);
  const int NI = L.NI;
  for (int n = 0; n < NI; n++) elev[n] = lay_interp(L, w, 0, n);
  int mi = lay_last_ge(z, elev, NI);
  on = mi >= 0 && grd_is_start(G, mi) && fabsf(z - elev[mi]) < FLT_EPSILON;
  float dis_r = 0.5f;
  if (mi >= 0 && mi + 1 < NI && (double)fabsf(elev[mi + 1] - elev[mi]) > 1e-6)
    dis_r = (z - elev[mi]) / (elev[mi + 1] - elev[mi]);
  if (mi == -1 || mi == NI - 1) {
    if (mi == -1) mi = lay_last_ge(elev[0], elev, NI);
    if (mi < 0) return 1;   /* only a NaN elevation or coordinate gets here */
#pragma unroll
    for (int p = 0; p < NP; p++) var[p] = lay_interp(L, w, 1 + p, mi);
    return 0;
  }
  if (mi > 0 && fabsf(elev[mi] - z) < FLT_EPSILON && grd_is_start(G, mi)) {
    mi--;
    dis_r = 0.5f;
  }
#pragma unroll
  for (int p = 0; p < NP; p++) {
    const float v0 = lay_interp(L, w, 1 + p, mi), v1 = lay_interp(L, w, 1 + p, mi + 1);
    var[p] = v0 + (v1 - v0) * dis_r;
  }
  if (KIND == LAY_ISO && lay_vp_low(var[1], var[2])) return 2;
  return 0;
}

/* out: rho, lambda, mu (isotropic, the reference's argument order) or c11
 * c33 c55 c66 c13 rho (VTI) */
template <int KIND>
__global__ void k_grid_loc(LayerMesh L, GridLayers G, long long vol, const float *__restrict__ x3d,
                           const float *__restrict__ y3d, const float *__restrict__ z3d,
                           LayOut out, int *bad)
{
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < vol;
       q += (long long)gridDim.x * blockDim.x) {
    float elev[LAY_MAX], var[6];
    int on;
    const int st = grd_point<KIND>(L, G, x3d[q], y3d[q], z3d[q], elev, var, on);
    if (st) {
      atomicOr(bad, st);
      continue;
    }
    if (KIND == LAY_ISO) {
      const float m = var[2] * var[2] * var[0];
      out.v[2][q] = m;
      out.v[1][q] = lay_lambda(var[1], var[0], m);
      out.v[0][q] = var[0];
    } else {
      float c[6];
      lay_para2vti<KIND>(var, c);
#pragma unroll
      for (int n = 0; n < 6; n++) out.v[n][q] = c[n];
    }
  }
}

/* Whether every (value, gradient, power) triple of a layered model with a
 * non-zero gradient has its power in [0, 1], the range that has run on the
 * device.  Other models are refused, because one-component models with a
 * power of 1.2 faulted on the device for a cause not found (unit powers
 * and zero gradients take no pow at all). */
extern "C" int cgfd_media_layer_pow_ok(int nc, const float *rec, size_t nrec)
{
  for (size_t r = 0; r < nrec; r++)
    for (int c = 1; c + 2 <= nc - 1; c += 3) {
      const float g = rec[r * nc + c + 1], pw = rec[r * nc + c + 2];
      if (g != 0.0f && !(pw >= 0.0f && pw <= 1.0f)) return 0;
    }
  return 1;
}

template <int KIND>
static void lay_launch(const LayerMesh &L, int meth, int nx, int ny, int nz, size_t vol,
                       const float *dx, const float *dy, const float *dz, const LayOut &o,
                       signed char *dmat, long long *dlist, unsigned long long *dcount,
                       int *d_bad, cudaStream_t st)
{
  k_layer_loc<KIND><<<152 * 8, 256, 0, st>>>(L, (long long)vol, dx, dy, dz, o, d_bad);
  if (meth) {
    k_layer_mark<<<152 * 8, 256, 0, st>>>(L, nx, ny, nz, dx, dy, dz, dmat);
    k_layer_mixed<<<152 * 8, 256, 0, st>>>(nx, ny, nz, dmat, dlist, dcount, L.chk);
    k_layer_avg<KIND><<<152 * 16, 128, 0, st>>>(L, meth, nx, ny, nz, dx, dy, dz, dlist, dcount,
                                                 o, d_bad);
  }
}

/* one call: upload, discretise, download; out holds nout host volumes */
static int lay_run(int kind, int NI, int NX, int NY, float MINX, float MINY, float DX, float DY,
                   const float *rec, int nx, int ny, int nz, const float *x3d,
                   const float *y3d, const float *z3d, const char *method, float **out)
{
  int meth = -1;
  if (method && strcmp(method, "loc") == 0) meth = 0;
  if (method && strcmp(method, "har") == 0) meth = 1;
  if (method && strcmp(method, "ari") == 0) meth = 2;
  if (meth < 0)
    return lay_err(CGFD_EINVAL, "layered model: equivalent medium method %s (loc, har or ari)",
                   method ? method : "(null)");
  if (NI < 1 || NI > LAY_MAX || NX < 2 || NY < 2 || !(DX > 0) || !(DY > 0))
    return lay_err(CGFD_EINVAL, "layered model: %d interfaces on a %dx%d mesh (1..%d "
                   "interfaces, at least 2x2 points, positive spacing)", NI, NX, NY, LAY_MAX);
  const int nout = kind == LAY_ISO ? 3 : 6, nc = 1 + 3 * nout;
  bool have_out = true;
  for (int n = 0; n < nout; n++) have_out = have_out && out[n];
  if (!rec || !x3d || !y3d || !z3d || !have_out || nx < 1 || ny < 1 || nz < 1)
    return lay_err(CGFD_EINVAL, "layered model: missing array or empty grid");
  const size_t vol = (size_t)nx * ny * nz, nrec = (size_t)NI * NX * NY * nc;
  /* powers outside [0, 1] on a non-zero gradient have not run on the
   * device (cgfd_media_layer_pow_ok): such models are refused */
  if (!cgfd_media_layer_pow_ok(nc, rec, nrec / nc))
    return lay_err(CGFD_EINVAL, "layered model: a power outside [0, 1] with a non-zero gradient "
                   "(not taken on the device)");
  /* device buffer: x, y, z, the outputs, the model; then for har/ari the
   * list of points to average, its counter and the layer numbers (bytes) */
  const size_t fl = (3 + nout) * vol + nrec, extra = meth ? vol * 8 + 8 + vol + 8 : 0;
  char *d = nullptr;
  int *d_bad = nullptr, bad = 0;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d, fl * sizeof(float) + extra);
  /* d_bad[0]: input errors (outside the mesh, vp <= sqrt(2) vs);
   * d_bad[1]: this call's bounds check word */
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_bad, 2 * sizeof(int));
  float *df = (float *)d;
  float *dx = df, *dy = df + vol, *dz = df + 2 * vol, *drec = df + (3 + nout) * vol;
  LayOut o = {};
  for (int n = 0; n < nout; n++) o.v[n] = df + (3 + n) * vol;
  /* 8-byte aligned start of the list: fl floats rounded up */
  const size_t off = (fl * sizeof(float) + 7) & ~(size_t)7;
  long long *dlist = meth ? (long long *)(d + off) : nullptr;
  unsigned long long *dcount = meth ? (unsigned long long *)(d + off + vol * 8) : nullptr;
  signed char *dmat = meth ? (signed char *)(d + off + vol * 8 + 8) : nullptr;
  int check = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, 2 * sizeof(int), st);
  if (e == cudaSuccess && meth) e = cudaMemsetAsync(dcount, 0, 8, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(drec, rec, nrec * 4, cudaMemcpyHostToDevice, st);
  const LayerMesh L = {NI, NX, NY, nc, MINX, MINY, DX, DY, drec, d_bad + 1};
  if (e == cudaSuccess) {
    switch (kind) {
      case LAY_ISO:
        lay_launch<LAY_ISO>(L, meth, nx, ny, nz, vol, dx, dy, dz, o, dmat, dlist, dcount, d_bad, st);
        break;
      case LAY_VTI_PREM:
        lay_launch<LAY_VTI_PREM>(L, meth, nx, ny, nz, vol, dx, dy, dz, o, dmat, dlist, dcount,
                                 d_bad, st);
        break;
      case LAY_VTI_THOMSEN:
        lay_launch<LAY_VTI_THOMSEN>(L, meth, nx, ny, nz, vol, dx, dy, dz, o, dmat, dlist, dcount,
                                    d_bad, st);
        break;
      default:
        lay_launch<LAY_VTI_CIJ>(L, meth, nx, ny, nz, vol, dx, dy, dz, o, dmat, dlist, dcount,
                                d_bad, st);
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&check, d_bad + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  for (int n = 0; n < nout && e == cudaSuccess; n++)
    e = cudaMemcpyAsync(out[n], o.v[n], vol * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d) cudaFree(d);
  if (d_bad) cudaFree(d_bad);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess)
    return lay_err(CGFD_ECUDA, "layered model: %s", cudaGetErrorString(e));
  if (check)
    return lay_err(CGFD_ECUDA, "layered model: internal bounds check %d failed", check);
  if (bad & 1) return lay_err(CGFD_EINVAL, "layered model: a grid point lies outside the "
                              "interfaces' mesh");
  if (bad & 2) return lay_err(CGFD_EINVAL, "layered model: vp <= sqrt(2) vs at a grid point");
  return 0;
}

extern "C" int cgfd_media_layer_el_iso(int NI, int NX, int NY, float MINX, float MINY,
                                       float DX, float DY, const float *rec, int nx, int ny,
                                       int nz, const float *x3d, const float *y3d,
                                       const float *z3d, const char *method, float *lam,
                                       float *mu, float *rho)
{
  float *out[3] = {lam, mu, rho};
  return lay_run(LAY_ISO, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d, z3d,
                 method, out);
}

extern "C" int cgfd_media_layer_el_vti(int media_type, int NI, int NX, int NY, float MINX,
                                       float MINY, float DX, float DY, const float *rec, int nx,
                                       int ny, int nz, const float *x3d, const float *y3d,
                                       const float *z3d, const char *method, float *c11,
                                       float *c33, float *c55, float *c66, float *c13,
                                       float *rho)
{
  if (media_type != LAY_VTI_PREM && media_type != LAY_VTI_THOMSEN && media_type != LAY_VTI_CIJ)
    return lay_err(CGFD_EINVAL, "layered model: VTI media type %d (22 prem, 23 thomsen, "
                   "24 cij)", media_type);
  float *out[6] = {c11, c33, c55, c66, c13, rho};
  return lay_run(media_type, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d, z3d,
                 method, out);
}

/* one grid-model call; out: 3 (isotropic) or 6 (VTI) host volumes */
static int grd_run(int kind, int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                   float MINY, float DX, float DY, const float *rec, int nx, int ny, int nz,
                   const float *x3d, const float *y3d, const float *z3d, const char *method,
                   float *const *out)
{
  const int nout = kind == LAY_ISO ? 3 : 6;
  int meth = -1;
  if (method && strcmp(method, "loc") == 0) meth = 0;
  if (method && strcmp(method, "har") == 0) meth = 1;
  if (method && strcmp(method, "ari") == 0) meth = 2;
  if (meth < 0)
    return lay_err(CGFD_EINVAL, "grid model: equivalent medium method %s (loc, har or ari)",
                   method ? method : "(null)");
  /* The cell averaging of grid models gave other values on the device than
   * the same kernel source built for the host (which equals the reference),
   * and other ones again with another register allocation; the cause is not
   * found, so grid models take "loc" on the device only. */
  if (meth != 0)
    return lay_err(CGFD_EINVAL, "grid model: the device takes the loc method (har and ari: the "
                   "reference's host routine)");
  if (NI < 1 || NI > LAY_MAX || NL < 1 || NL > NI || !ngz || NX < 2 || NY < 2 || !(DX > 0) ||
      !(DY > 0))
    return lay_err(CGFD_EINVAL, "grid model: %d levels in %d layers on a %dx%d mesh (1..%d "
                   "levels, at least 2x2 points, positive spacing)", NI, NL, NX, NY, LAY_MAX);
  GridLayers G = {};
  G.NL = NL;
  int acc = 0;
  for (int l = 0; l < NL; l++) {
    if (ngz[l] < 1) return lay_err(CGFD_EINVAL, "grid model: layer %d has %d levels", l, ngz[l]);
    G.start[l] = acc;
    acc += ngz[l];
  }
  if (acc != NI)
    return lay_err(CGFD_EINVAL, "grid model: the layers hold %d levels, not %d", acc, NI);
  bool have_out = true;
  for (int n = 0; n < nout; n++) have_out = have_out && out[n];
  if (!rec || !x3d || !y3d || !z3d || !have_out || nx < 1 || ny < 1 || nz < 1)
    return lay_err(CGFD_EINVAL, "grid model: missing array or empty grid");
  const int nc = 1 + nout;
  const size_t vol = (size_t)nx * ny * nz, nrec = (size_t)NI * NX * NY * nc;
  /* device buffer: x, y, z, the outputs, the model */
  const size_t fl = (3 + nout) * vol + nrec;
  char *d = nullptr;
  int *d_bad = nullptr, bad = 0, check = 0;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d, fl * sizeof(float));
  /* d_bad[0]: input errors; d_bad[1]: this call's bounds check word */
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_bad, 2 * sizeof(int));
  float *df = (float *)d;
  float *dx = df, *dy = df + vol, *dz = df + 2 * vol, *drec = df + (3 + nout) * vol;
  LayOut o = {};
  for (int n = 0; n < nout; n++) o.v[n] = df + (3 + n) * vol;
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, 2 * sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(drec, rec, nrec * 4, cudaMemcpyHostToDevice, st);
  const LayerMesh L = {NI, NX, NY, nc, MINX, MINY, DX, DY, drec, d_bad + 1};
  if (e == cudaSuccess) {
    switch (kind) {
      case LAY_ISO:
        k_grid_loc<LAY_ISO><<<152 * 8, 256, 0, st>>>(L, G, (long long)vol, dx, dy, dz, o, d_bad);
        break;
      case LAY_VTI_PREM:
        k_grid_loc<LAY_VTI_PREM><<<152 * 8, 256, 0, st>>>(L, G, (long long)vol, dx, dy, dz, o,
                                                           d_bad);
        break;
      case LAY_VTI_THOMSEN:
        k_grid_loc<LAY_VTI_THOMSEN><<<152 * 8, 256, 0, st>>>(L, G, (long long)vol, dx, dy, dz, o,
                                                              d_bad);
        break;
      default:
        k_grid_loc<LAY_VTI_CIJ><<<152 * 8, 256, 0, st>>>(L, G, (long long)vol, dx, dy, dz, o,
                                                          d_bad);
    }
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&check, d_bad + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  for (int n = 0; n < nout && e == cudaSuccess; n++)
    e = cudaMemcpyAsync(out[n], o.v[n], vol * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d) cudaFree(d);
  if (d_bad) cudaFree(d_bad);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess) return lay_err(CGFD_ECUDA, "grid model: %s", cudaGetErrorString(e));
  if (check) return lay_err(CGFD_ECUDA, "grid model: internal bounds check %d failed", check);
  if (bad & 1) return lay_err(CGFD_EINVAL, "grid model: a grid point lies outside the mesh");
  if (bad & 2) return lay_err(CGFD_EINVAL, "grid model: vp <= sqrt(2) vs at a grid point");
  return 0;
}

extern "C" int cgfd_media_grid_el_iso(int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                                      float MINY, float DX, float DY, const float *rec, int nx,
                                      int ny, int nz, const float *x3d, const float *y3d,
                                      const float *z3d, const char *method, float *rho,
                                      float *lam, float *mu)
{
  float *out[3] = {rho, lam, mu};
  return grd_run(LAY_ISO, NI, NL, ngz, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d,
                 z3d, method, out);
}

extern "C" int cgfd_media_grid_el_vti(int media_type, int NI, int NL, const int *ngz, int NX,
                                      int NY, float MINX, float MINY, float DX, float DY,
                                      const float *rec, int nx, int ny, int nz,
                                      const float *x3d, const float *y3d, const float *z3d,
                                      const char *method, float *c11, float *c33, float *c55,
                                      float *c66, float *c13, float *rho)
{
  if (media_type != LAY_VTI_PREM && media_type != LAY_VTI_THOMSEN && media_type != LAY_VTI_CIJ)
    return lay_err(CGFD_EINVAL, "grid model: VTI media type %d (22 prem, 23 thomsen, 24 cij)",
                   media_type);
  float *out[6] = {c11, c33, c55, c66, c13, rho};
  return grd_run(media_type, NI, NL, ngz, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d,
                 z3d, method, out);
}
