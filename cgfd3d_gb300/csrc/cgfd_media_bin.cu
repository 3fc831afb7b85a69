/*
 * cgfd_media_bin.cu -- a model given as binary volumes (rho, vp, vs or Qp,
 * Qs on a regular 3-D mesh, in any axis order) interpolated on a curvilinear
 * grid on the device.
 *
 * The reference reads the volumes on the host sample by sample, cropped to
 * the grid's x/y range, and interpolates every grid point trilinearly
 * (media_bin2model_el_iso / media_bin2model_vis_iso,
 * media/media_bin2model.cpp:27-432; TrilinearInterpolation,
 * media/media_utility.cpp:299-391).  Here the host works out the same crop
 * and coordinate vectors (cgfd_media_bin_crop gives callers the box of the
 * files it covers, so they can read only that), only the box goes to the
 * device, and one thread per grid point interpolates each volume through
 * the box's strides, in the reference's float order (--fmad=false);
 * rho, vp, vs become rho, lambda = vp^2 rho - 2 mu, mu = vs^2 rho.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/cgfd3d_gpu.h"

__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg);

static int bin_err(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return cgfd_set_error_msg(code, buf);
}

#define BIN_MAXN 65536   /* samples along an axis of the cropped model */

struct BinCrop {
  int dim[3];            /* file dimension holding x, y, z (host only) */
  int first[3];          /* first kept x, y, z sample of the files */
  int start[3];          /* offset of the crop's first sample in the volumes read */
  int n[3];              /* kept samples along x, y, z */
  long long st[3];       /* strides of the x, y, z axes in the volumes read */
  const float *xv, *yv, *zv;   /* device coordinate vectors */
};

struct BinVols {
  const float *v[3];
  float *out[3];
};

__device__ float bin_trilinear(const BinCrop &b, const float *__restrict__ v, float xq, float yq,
                               float zq)
{
  const float *x = b.xv, *y = b.yv, *z = b.zv;
  const int nx = b.n[0], ny = b.n[1], nz = b.n[2];
  const float dx = x[1] - x[0], dy = y[1] - y[0], dz = z[1] - z[0];
  int ix0 = (int)floorf((xq - x[0]) / dx), iy0 = (int)floorf((yq - y[0]) / dy);
  int ix2 = (int)ceilf((xq - x[0]) / dx), iy2 = (int)ceilf((yq - y[0]) / dy);
  ix0 = ix0 < 0 ? 0 : ix0;
  ix2 = ix2 < 0 ? 0 : ix2;
  ix0 = ix0 > nx - 1 ? nx - 1 : ix0;
  ix2 = ix2 > nx - 1 ? nx - 1 : ix2;
  iy0 = iy0 < 0 ? 0 : iy0;
  iy2 = iy2 < 0 ? 0 : iy2;
  iy0 = iy0 > ny - 1 ? ny - 1 : iy0;
  iy2 = iy2 > ny - 1 ? ny - 1 : iy2;
  int iz0 = (int)floorf((zq - z[0]) / dz), iz2 = (int)ceilf((zq - z[0]) / dz);
  iz0 = iz0 < 0 ? 0 : iz0;
  iz0 = iz0 > nz - 1 ? nz - 1 : iz0;
  iz2 = iz2 > nz - 1 ? nz - 1 : iz2;
  iz2 = iz2 < 0 ? 0 : iz2;
  auto at = [&](int i, int j, int k) {
    return v[(long long)(i + b.start[0]) * b.st[0] + (long long)(j + b.start[1]) * b.st[1] +
             (long long)(k + b.start[2]) * b.st[2]];
  };
  if (ix0 == ix2 && iy0 == iy2 && iz0 == iz2) return at(ix0, iy0, iz0);
  const float v000 = at(ix0, iy0, iz0), v002 = at(ix0, iy0, iz2);
  const float v200 = at(ix2, iy0, iz0), v202 = at(ix2, iy0, iz2);
  const float v020 = at(ix0, iy2, iz0), v022 = at(ix0, iy2, iz2);
  const float v220 = at(ix2, iy2, iz0), v222 = at(ix2, iy2, iz2);
  float v100, v102, v122, v120;
  if (ix0 == ix2) {
    v100 = v000;
    v102 = v002;
    v122 = v022;
    v120 = v020;
  } else {
    const float w = (xq - x[ix0]) / (x[ix2] - x[ix0]);
    v100 = v000 + w * (v200 - v000);
    v102 = v002 + w * (v202 - v002);
    v122 = v022 + w * (v222 - v022);
    v120 = v020 + w * (v220 - v020);
  }
  float v110, v112;
  if (iy0 == iy2) {
    v110 = v100;
    v112 = v102;
  } else {
    const float w = (yq - y[iy0]) / (y[iy2] - y[iy0]);
    v110 = v100 + w * (v120 - v100);
    v112 = v102 + w * (v122 - v102);
  }
  if (iz0 == iz2) return v110;
  return v110 + (zq - z[iz0]) / (z[iz2] - z[iz0]) * (v112 - v110);
}

/* vis 0: rho, lambda, mu from rho, vp, vs; vis 1: Qp, Qs */
__global__ void k_bin(BinCrop b, int vis, long long vol, const float *__restrict__ x3d,
                      const float *__restrict__ y3d, const float *__restrict__ z3d, BinVols bv)
{
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < vol;
       q += (long long)gridDim.x * blockDim.x) {
    const float x = x3d[q], y = y3d[q], z = z3d[q];
    if (vis) {
      bv.out[0][q] = bin_trilinear(b, bv.v[0], x, y, z);
      bv.out[1][q] = bin_trilinear(b, bv.v[1], x, y, z);
    } else {
      const float rho = bin_trilinear(b, bv.v[0], x, y, z);
      const float vp = bin_trilinear(b, bv.v[1], x, y, z);
      const float vs = bin_trilinear(b, bv.v[2], x, y, z);
      const float mu = vs * vs * rho;
      const float a = vp * vp * rho;
      /* a - 2.0 mu in double, then float: the float subtraction gives the
       * same bits while 2 mu is finite in float (the double difference of
       * two floats is exact, or both roundings give the larger operand) */
      bv.out[2][q] = mu;
      bv.out[1][q] = fabsf(mu) < 1e37f ? a - 2.0f * mu : (float)((double)a - 2.0 * (double)mu);
      bv.out[0][q] = rho;
    }
  }
}

/* The crop of media_bin2model_el_iso (media/media_bin2model.cpp:44-158),
 * worked out on the host; the coordinate vectors are filled in xv/yv/zv. */
static int bin_setup(const cgfd_bin_model_t *m, float xmin, float xmax, float ymin, float ymax,
                     const float *z3d, size_t vol, BinCrop &b, std::vector<float> &xv,
                     std::vector<float> &yv, std::vector<float> &zv)
{
  int dim[3] = {-1, -1, -1};
  for (int i = 0; i < 3; i++) {
    const int o = m->order[i];
    if (o < 0 || o > 2)
      return bin_err(CGFD_EINVAL, "binary model: bin_order[%d] = %d (0 x, 1 y, 2 z)", i, o);
    dim[o] = i;
  }
  if (dim[0] < 0 || dim[1] < 0 || dim[2] < 0)
    return bin_err(CGFD_EINVAL, "binary model: bin_order %d,%d,%d misses an axis", m->order[0],
                   m->order[1], m->order[2]);
  for (int i = 0; i < 3; i++)
    if (m->size[i] < 1)
      return bin_err(CGFD_EINVAL, "binary model: bin_size[%d] = %d", i, m->size[i]);
  const float bx0 = m->origin[dim[0]], by0 = m->origin[dim[1]], bz0 = m->origin[dim[2]];
  const float bdx = m->spacing[dim[0]], bdy = m->spacing[dim[1]], bdz = m->spacing[dim[2]];
  /* x and y increase along the files (the crop assumes it); z may decrease */
  if (!(bdx > 0.0f) || !(bdy > 0.0f) || !(bdz != 0.0f) || !std::isfinite(bdz))
    return bin_err(CGFD_EINVAL, "binary model: spacing x %g, y %g, z %g (x, y > 0, z != 0)",
                   bdx, bdy, bdz);
  if (!std::isfinite(xmin) || !std::isfinite(xmax) || !std::isfinite(ymin) ||
      !std::isfinite(ymax) || !std::isfinite(bx0) || !std::isfinite(by0) || !std::isfinite(bz0))
    return bin_err(CGFD_EINVAL, "binary model: non-finite extent or origin");
  const int ix_start = (int)(xmin < bx0 ? 0.0f : (xmin - bx0) / bdx);
  if (ix_start >= m->size[dim[0]] || xmax < bx0)
    return bin_err(CGFD_EINVAL, "binary model: the model does not cover the grid in x");
  int ix_end = (int)ceilf((xmax - bx0) / bdx);
  if (ix_end >= m->size[dim[0]]) ix_end = m->size[dim[0]] - 1;
  const int iy_start = (int)(ymin < by0 ? 0.0f : (ymin - by0) / bdy);
  if (iy_start >= m->size[dim[1]] || ymax < by0)
    return bin_err(CGFD_EINVAL, "binary model: the model does not cover the grid in y");
  int iy_end = (int)ceilf((ymax - by0) / bdy);
  if (iy_end >= m->size[dim[1]]) iy_end = m->size[dim[1]] - 1;
  float zmin = FLT_MAX, zmax = -FLT_MAX;
  for (size_t i = 0; i < vol; i++) {
    zmin = std::min(zmin, z3d[i]);
    zmax = std::max(zmax, z3d[i]);
  }
  const float bzn = bz0 + bdz * (m->size[dim[2]] - 1);
  if (zmin >= std::max(bzn, bz0) || zmax <= std::min(bz0, bzn))
    return bin_err(CGFD_EINVAL, "binary model: the model does not cover the grid in z");
  for (int d = 0; d < 3; d++) b.dim[d] = dim[d];
  b.first[0] = ix_start;
  b.first[1] = iy_start;
  b.first[2] = 0;
  b.n[0] = ix_end - ix_start + 1;
  b.n[1] = iy_end - iy_start + 1;
  b.n[2] = m->size[dim[2]];
  /* fewer than two samples: the reference's interpolation reads past its
   * coordinate vectors */
  for (int d = 0; d < 3; d++)
    if (b.n[d] < 2 || b.n[d] > BIN_MAXN)
      return bin_err(CGFD_EINVAL, "binary model: %d samples along axis %d after the crop "
                     "(2..%d)", b.n[d], d, BIN_MAXN);
  xv.resize(b.n[0]);
  yv.resize(b.n[1]);
  zv.resize(b.n[2]);
  for (size_t i = 0; i < (size_t)b.n[0]; i++) xv[i] = bx0 + (float)(ix_start + i) * bdx;
  for (size_t i = 0; i < (size_t)b.n[1]; i++) yv[i] = by0 + (float)(iy_start + i) * bdy;
  for (size_t i = 0; i < (size_t)b.n[2]; i++) zv[i] = bz0 + (float)i * bdz;
  return 0;
}

/* the box of the files (per file dimension: first sample, count) that a
 * crop covers */
static cgfd_bin_box_t bin_box_of(const BinCrop &b)
{
  cgfd_bin_box_t box;
  for (int d = 0; d < 3; d++) {
    box.first[b.dim[d]] = b.first[d];
    box.count[b.dim[d]] = b.n[d];
  }
  return box;
}

/* one call on volumes that hold `box` of the files (count[0] x count[1] x
 * count[2] floats each, file order): the box must contain the grid's crop */
static int bin_run_box(int vis, const cgfd_bin_model_t *m, const cgfd_bin_box_t *box,
                       float xmin, float xmax, float ymin, float ymax, const float *const *vols,
                       int nx, int ny, int nz, const float *x3d, const float *y3d,
                       const float *z3d, float *const *out)
{
  const int nv = vis ? 2 : 3;
  if (!m || !box || !x3d || !y3d || !z3d || nx < 1 || ny < 1 || nz < 1)
    return bin_err(CGFD_EINVAL, "binary model: missing argument or empty grid");
  for (int n = 0; n < nv; n++)
    if (!vols[n] || !out[n]) return bin_err(CGFD_EINVAL, "binary model: missing volume");
  const size_t vol = (size_t)nx * ny * nz;
  BinCrop b;
  std::vector<float> xv, yv, zv;
  const int rc = bin_setup(m, xmin, xmax, ymin, ymax, z3d, vol, b, xv, yv, zv);
  if (rc) return rc;
  for (int d = 0; d < 3; d++) {
    const int fd = b.dim[d];
    if (box->count[fd] < 1 || box->first[fd] < 0 || box->first[fd] > b.first[d] ||
        box->first[fd] + box->count[fd] < b.first[d] + b.n[d])
      return bin_err(CGFD_EINVAL, "binary model: the volumes' box (file dimension %d: %d + %d) "
                     "does not hold the crop (%d + %d)", fd, box->first[fd], box->count[fd],
                     b.first[d], b.n[d]);
    b.start[d] = b.first[d] - box->first[fd];
  }
  const long long bst[3] = {1, (long long)box->count[0],
                            (long long)box->count[0] * box->count[1]};
  for (int d = 0; d < 3; d++) b.st[d] = bst[b.dim[d]];
  const size_t bvol = (size_t)box->count[0] * box->count[1] * box->count[2];
  const size_t nvec = xv.size() + yv.size() + zv.size();
  /* device: x, y, z, the outputs, the volumes' boxes, the vectors */
  const size_t nfl = (3 + nv) * vol + nv * bvol + nvec;
  float *d = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d, nfl * sizeof(float));
  float *dx = d, *dy = d + vol, *dz = d + 2 * vol;
  BinVols bv = {};
  for (int n = 0; n < nv; n++) {
    bv.out[n] = d + (3 + n) * vol;
    bv.v[n] = d + (3 + nv) * vol + n * bvol;
  }
  float *dvec = d + (3 + nv) * vol + nv * bvol;
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y3d, vol * 4, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dz, z3d, vol * 4, cudaMemcpyHostToDevice, st);
  for (int n = 0; n < nv && e == cudaSuccess; n++)
    e = cudaMemcpyAsync((float *)bv.v[n], vols[n], bvol * 4, cudaMemcpyHostToDevice, st);
  std::vector<float> vec(xv);
  vec.insert(vec.end(), yv.begin(), yv.end());
  vec.insert(vec.end(), zv.begin(), zv.end());
  if (e == cudaSuccess) e = cudaMemcpyAsync(dvec, vec.data(), nvec * 4, cudaMemcpyHostToDevice, st);
  b.xv = dvec;
  b.yv = dvec + xv.size();
  b.zv = dvec + xv.size() + yv.size();
  if (e == cudaSuccess) {
    k_bin<<<152 * 8, 256, 0, st>>>(b, vis, (long long)vol, dx, dy, dz, bv);
    e = cudaGetLastError();
  }
  for (int n = 0; n < nv && e == cudaSuccess; n++)
    e = cudaMemcpyAsync(out[n], bv.out[n], vol * 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d) cudaFree(d);
  if (st) cudaStreamDestroy(st);
  if (e != cudaSuccess) return bin_err(CGFD_ECUDA, "binary model: %s", cudaGetErrorString(e));
  return 0;
}

/* whole files: the crop's box is gathered on the host (one copy per run of
 * the files' fastest dimension) and only it goes to the device */
static int bin_run(int vis, const cgfd_bin_model_t *m, float xmin, float xmax, float ymin,
                   float ymax, const float *const *vols, int nx, int ny, int nz,
                   const float *x3d, const float *y3d, const float *z3d, float *const *out)
{
  const int nv = vis ? 2 : 3;
  if (!m || !x3d || !y3d || !z3d || nx < 1 || ny < 1 || nz < 1)
    return bin_err(CGFD_EINVAL, "binary model: missing argument or empty grid");
  for (int n = 0; n < nv; n++)
    if (!vols[n] || !out[n]) return bin_err(CGFD_EINVAL, "binary model: missing volume");
  BinCrop b;
  std::vector<float> xv, yv, zv;
  const int rc = bin_setup(m, xmin, xmax, ymin, ymax, z3d, (size_t)nx * ny * nz, b, xv, yv, zv);
  if (rc) return rc;
  const cgfd_bin_box_t box = bin_box_of(b);
  const size_t run = (size_t)box.count[0];
  const size_t bvol = run * box.count[1] * box.count[2];
  std::vector<std::vector<float>> boxes(nv, std::vector<float>(bvol));
  const float *bp[3] = {nullptr, nullptr, nullptr};
  for (int n = 0; n < nv; n++) {
    float *dst = boxes[n].data();
    for (int c2 = 0; c2 < box.count[2]; c2++)
      for (int c1 = 0; c1 < box.count[1]; c1++) {
        const size_t src = ((size_t)(box.first[2] + c2) * m->size[1] + box.first[1] + c1) *
                               m->size[0] + box.first[0];
        memcpy(dst + ((size_t)c2 * box.count[1] + c1) * run, vols[n] + src, run * 4);
      }
    bp[n] = dst;
  }
  return bin_run_box(vis, m, &box, xmin, xmax, ymin, ymax, bp, nx, ny, nz, x3d, y3d, z3d, out);
}

extern "C" int cgfd_media_bin_crop(const cgfd_bin_model_t *model, float xmin, float xmax,
                                   float ymin, float ymax, int nx, int ny, int nz,
                                   const float *z3d, cgfd_bin_box_t *box)
{
  if (!model || !z3d || !box || nx < 1 || ny < 1 || nz < 1)
    return bin_err(CGFD_EINVAL, "binary model: missing argument or empty grid");
  BinCrop b;
  std::vector<float> xv, yv, zv;
  const int rc = bin_setup(model, xmin, xmax, ymin, ymax, z3d, (size_t)nx * ny * nz, b, xv,
                           yv, zv);
  if (rc) return rc;
  *box = bin_box_of(b);
  return 0;
}

extern "C" int cgfd_media_bin_el_iso_box(const cgfd_bin_model_t *model, const cgfd_bin_box_t *box,
                                         float xmin, float xmax, float ymin, float ymax,
                                         const float *rho_box, const float *vp_box,
                                         const float *vs_box, int nx, int ny, int nz,
                                         const float *x3d, const float *y3d, const float *z3d,
                                         float *rho, float *lam, float *mu)
{
  const float *v[3] = {rho_box, vp_box, vs_box};
  float *o[3] = {rho, lam, mu};
  return bin_run_box(0, model, box, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}

extern "C" int cgfd_media_bin_vis_iso_box(const cgfd_bin_model_t *model,
                                          const cgfd_bin_box_t *box, float xmin, float xmax,
                                          float ymin, float ymax, const float *qp_box,
                                          const float *qs_box, int nx, int ny, int nz,
                                          const float *x3d, const float *y3d, const float *z3d,
                                          float *qp, float *qs)
{
  const float *v[3] = {qp_box, qs_box, nullptr};
  float *o[3] = {qp, qs, nullptr};
  return bin_run_box(1, model, box, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}

extern "C" int cgfd_media_bin_el_iso(const cgfd_bin_model_t *model, float xmin, float xmax,
                                     float ymin, float ymax, const float *rho_vol,
                                     const float *vp_vol, const float *vs_vol, int nx, int ny,
                                     int nz, const float *x3d, const float *y3d,
                                     const float *z3d, float *rho, float *lam, float *mu)
{
  const float *v[3] = {rho_vol, vp_vol, vs_vol};
  float *o[3] = {rho, lam, mu};
  return bin_run(0, model, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}

extern "C" int cgfd_media_bin_vis_iso(const cgfd_bin_model_t *model, float xmin, float xmax,
                                      float ymin, float ymax, const float *qp_vol,
                                      const float *qs_vol, int nx, int ny, int nz,
                                      const float *x3d, const float *y3d, const float *z3d,
                                      float *qp, float *qs)
{
  const float *v[3] = {qp_vol, qs_vol, nullptr};
  float *o[3] = {qp, qs, nullptr};
  return bin_run(1, model, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}
