/*
 * cgfd_locate.cu -- stations and sources given by coordinates, located on a
 * curvilinear grid on the device.
 *
 * The reference locates every station and source of a run one after the
 * other on the host (gd_curv_coord_to_glob_indx, forward/gd_t.c:1917-1995):
 * a scan of 4x4x4 tiles and their cells by bounding boxes, a point-in-
 * hexahedron test (media/media_geometry3d.cpp:198-265), then the shift
 * inside the cell as the closest of 101^3 trilinear samples
 * (gd_curv_coord2shift_sample, forward/gd_t.c:2304-2370) -- about 10^6
 * samples per point, so set-up time grows with the number of stations and
 * dominates short batched runs.  Here the same steps run as kernels:
 *
 *   grid bounds   k_loc_global_bounds, k_loc_tile_bounds: gd_curv_set_minmax
 *                 (forward/gd_t.c:1708-1880): bounds of all points, and of
 *                 each tile as the bounds of the corner points of its cells;
 *   depth -> z    k_loc_depth, one block per point given by depth:
 *                 gd_curv_depth_to_axis (forward/gd_t.c:2179-2297), the top
 *                 cells in parallel, the first hit in the reference's scan
 *                 order kept by an atomic minimum of the scan position;
 *   cell search   k_loc_cells over (point, tile) pairs whose tile box holds
 *                 the point, every cell of the tile in parallel, again the
 *                 first hit in scan order (tile, then k, j, i);
 *   shift         k_loc_sample, one block per located point: the 101^3
 *                 samples split over the block, the closest (first on ties)
 *                 by a block reduction.
 *
 * The float arithmetic of each test and sample is written in the order the
 * reference evaluates it and this file is compiled with --fmad=false
 * (separate IEEE multiplies and adds; divisions and square roots are
 * correctly rounded by default), so the located indices and shifts equal
 * the reference's bit for bit.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/cgfd3d_gpu.h"

#define LOC_TILES 4     /* GD_TILE_NX/NY/NZ, forward/gd_t.h:9-11 */
#define LOC_NT (LOC_TILES * LOC_TILES * LOC_TILES)
#define LOC_SAMPLES 100 /* samples per direction: 0..100 */
#define LOC_GHOSTS 3
#define LOC_NONE 0xFFFFFFFFFFFFFFFFull

__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg);

static int loc_err(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return cgfd_set_error_msg(code, buf);
}

#define LCK(call)                                                              \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return loc_err(CGFD_ECUDA, "%s failed: %s (%s:%d)", #call,               \
                     cudaGetErrorString(e_), __FILE__, __LINE__);              \
  } while (0)

struct LocGrid {
  int nx, ny, nz;
  long long sl;
  const float *x, *y, *z;
  int ts[3][LOC_TILES], te[3][LOC_TILES];   /* tile cell ranges per axis */
};

struct V3 {
  float x, y, z;
};

/* ---- order-preserving float keys for atomic min / max ------------------- */

__device__ __forceinline__ unsigned ord_key(float f)
{
  unsigned b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

static float ord_val(unsigned k)
{
  unsigned b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
  float f;
  memcpy(&f, &b, 4);
  return f;
}

static unsigned ord_key_host(float f)
{
  unsigned b;
  memcpy(&b, &f, 4);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

/* ---- geometry in the reference's operation order ------------------------ */

__device__ __forceinline__ V3 v3_sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ float v3_dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 v3_cross(V3 a, V3 b)
{
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float v3_len(V3 a) { return sqrtf(v3_dot(a, a)); }
__device__ __forceinline__ float tri_area2(V3 a, V3 b, V3 c)
{
  return v3_len(v3_cross(v3_sub(b, a), v3_sub(c, a)));
}

/* a point on a triangle: the sub-areas add up to its area within 1e-6 */
__device__ __forceinline__ bool on_tri(V3 p, V3 a, V3 b, V3 c)
{
  float s = tri_area2(p, a, b) + tri_area2(p, b, c) + tri_area2(p, c, a) - tri_area2(a, b, c);
  return fabs((double)s) < 1e-6;
}

/* the hexahedron cut into five tetrahedra in two ways (ten in all), each
 * as four faces; corners numbered i + 2 j + 4 k */
__constant__ unsigned char c_tetra[10][4][3] = {
    {{0, 4, 2}, {2, 4, 1}, {1, 4, 0}, {0, 2, 1}},
    {{4, 6, 2}, {2, 6, 7}, {7, 6, 4}, {4, 2, 7}},
    {{2, 7, 3}, {3, 7, 1}, {1, 2, 3}, {1, 7, 2}},
    {{7, 4, 5}, {1, 7, 5}, {5, 4, 1}, {1, 4, 7}},
    {{2, 4, 7}, {7, 4, 1}, {2, 7, 1}, {4, 2, 1}},
    {{4, 5, 6}, {4, 6, 0}, {4, 0, 5}, {6, 5, 0}},
    {{6, 2, 0}, {6, 3, 2}, {0, 2, 3}, {3, 6, 0}},
    {{6, 5, 7}, {3, 6, 7}, {7, 5, 3}, {5, 6, 3}},
    {{5, 0, 1}, {3, 5, 1}, {0, 3, 1}, {0, 5, 3}},
    {{5, 6, 0}, {5, 0, 3}, {0, 6, 3}, {3, 6, 5}}};

__device__ bool in_hexahedron(V3 p, const V3 *v)
{
  for (int t = 0; t < 10; t++) {
    bool inside = true;
    for (int f = 0; f < 4 && inside; f++) {
      const V3 a = v[c_tetra[t][f][0]], b = v[c_tetra[t][f][1]], c = v[c_tetra[t][f][2]];
      if (on_tri(p, a, b, c)) break;
      V3 p2f = v3_sub(a, p);
      V3 n = v3_cross(v3_sub(b, a), v3_sub(c, a));
      float d = v3_len(n);
      n.x = n.x / d;
      n.y = n.y / d;
      n.z = n.z / d;
      float sign = v3_dot(p2f, n);
      sign /= v3_len(p2f);
      if (sign <= -1.0e-6f) inside = false;
    }
    if (inside) return true;
  }
  return false;
}

/* 2-D point in triangle (lib/fdlib_math.c:246-266): the edge sign divided
 * by the edge length in double, as the reference's sqrt of a float sum */
__device__ bool in_tri2(float px, float py, const float *vx, const float *vy)
{
  for (int i = 0; i < 3; i++) {
    float ex = i == 2 ? vx[0] - vx[2] : vx[i + 1] - vx[i];
    float ey = i == 2 ? vy[0] - vy[2] : vy[i + 1] - vy[i];
    float tx = px - vx[i], ty = py - vy[i];
    float sign = ex * ty - ey * tx;
    sign = (float)((double)sign / sqrt((double)(ex * ex + ey * ey)));
    if (sign < 0) return false;
  }
  return true;
}

__device__ float z_on_tri(float x, float y, V3 p1, V3 p2, V3 p3)
{
  float v1x = p2.x - p1.x, v1y = p2.y - p1.y, v1z = p2.z - p1.z;
  float v2x = p3.x - p1.x, v2y = p3.y - p1.y, v2z = p3.z - p1.z;
  float a = v1y * v2z - v1z * v2y;
  float b = v1z * v2x - v1x * v2z;
  float c = v1x * v2y - v1y * v2x;
  float d = -(a * p1.x + b * p1.y + c * p1.z);
  return -(a * x + b * y + d) / c;
}

__device__ __forceinline__ V3 gpt(const LocGrid &g, int i, int j, int k)
{
  long long q = (long long)i + (long long)j * g.nx + (long long)k * g.sl;
  return {g.x[q], g.y[q], g.z[q]};
}

/* tile of index a along axis d (a within the tiles' cell range) */
__device__ __forceinline__ int tile_of(const LocGrid &g, int d, int a)
{
  int t = 0;
  while (t < LOC_TILES - 1 && a > g.te[d][t]) t++;
  return t;
}

/* ---- grid bounds ---------------------------------------------------------- */

__device__ __forceinline__ void warp_minmax(float &lo, float &hi)
{
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
}

/* bounds of every point (ghosts included): keys xmin, xmax, ymin, ... */
__global__ void k_loc_global_bounds(const float *__restrict__ x, const float *__restrict__ y,
                                    const float *__restrict__ z, long long n, unsigned *bnd)
{
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    lo[0] = fminf(lo[0], x[q]); hi[0] = fmaxf(hi[0], x[q]);
    lo[1] = fminf(lo[1], y[q]); hi[1] = fmaxf(hi[1], y[q]);
    lo[2] = fminf(lo[2], z[q]); hi[2] = fmaxf(hi[2], z[q]);
  }
  for (int d = 0; d < 3; d++) {
    warp_minmax(lo[d], hi[d]);
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&bnd[2 * d], ord_key(lo[d] + 0.0f));
      atomicMax(&bnd[2 * d + 1], ord_key(hi[d] + 0.0f));
    }
  }
}

/* bounds of tile blockIdx.y: the corner points of its cells */
__global__ void k_loc_tile_bounds(LocGrid g, unsigned *tb)
{
  const int t = blockIdx.y;
  const int it = t % LOC_TILES, jt = (t / LOC_TILES) % LOC_TILES, kt = t / (LOC_TILES * LOC_TILES);
  const int i0 = g.ts[0][it], j0 = g.ts[1][jt], k0 = g.ts[2][kt];
  const int ni = g.te[0][it] - i0 + 2, nj = g.te[1][jt] - j0 + 2, nk = g.te[2][kt] - k0 + 2;
  if (ni < 2 || nj < 2 || nk < 2) return;       /* a tile without cells */
  const long long np = (long long)ni * nj * nk;
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np;
       p += (long long)gridDim.x * blockDim.x) {
    int a = (int)(p % ni), b = (int)((p / ni) % nj), c = (int)(p / ((long long)ni * nj));
    V3 v = gpt(g, i0 + a, j0 + b, k0 + c);
    lo[0] = fminf(lo[0], v.x); hi[0] = fmaxf(hi[0], v.x);
    lo[1] = fminf(lo[1], v.y); hi[1] = fmaxf(hi[1], v.y);
    lo[2] = fminf(lo[2], v.z); hi[2] = fmaxf(hi[2], v.z);
  }
  for (int d = 0; d < 3; d++) {
    warp_minmax(lo[d], hi[d]);
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&tb[t * 6 + 2 * d], ord_key(lo[d] + 0.0f));
      atomicMax(&tb[t * 6 + 2 * d + 1], ord_key(hi[d] + 0.0f));
    }
  }
}

/* ---- depth to z --------------------------------------------------------- */

struct LocBounds {
  float g[6];                 /* xmin, xmax, ymin, ymax, zmin, zmax */
  float t[LOC_NT][6];         /* per tile, tile index (kt * 4 + jt) * 4 + it */
};

/* cell (i, j, k) xy bounds from its 8 corners */
__device__ void cell_xy(const LocGrid &g, int i, int j, int k, float *b)
{
  V3 p = gpt(g, i, j, k);
  b[0] = b[1] = p.x;
  b[2] = b[3] = p.y;
  for (int c = 1; c < 8; c++) {
    V3 q = gpt(g, i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2));
    b[0] = fminf(b[0], q.x); b[1] = fmaxf(b[1], q.x);
    b[2] = fminf(b[2], q.y); b[3] = fmaxf(b[3], q.y);
  }
}

/* which triangle of the top face of cell (i, j) holds (sx, sy): 2 for
 * corners (3, 2, 0), 1 for (0, 1, 3), 0 for none (lib/fdlib_math.c:286-304) */
__device__ int top_tri(const LocGrid &g, int i, int j, int k, float sx, float sy, V3 *p)
{
  for (int c = 0; c < 4; c++) p[c] = gpt(g, i + (c & 1), j + (c >> 1), k);
  float vx[5] = {p[0].x, p[1].x, p[3].x, p[2].x, p[0].x};
  float vy[5] = {p[0].y, p[1].y, p[3].y, p[2].y, p[0].y};
  if (in_tri2(sx, sy, vx + 2, vy + 2)) return 2;
  if (in_tri2(sx, sy, vx, vy)) return 1;
  return 0;
}

__global__ void k_loc_depth(LocGrid g, const LocBounds *__restrict__ bd,
                            const int *__restrict__ list, const float *__restrict__ qx,
                            const float *__restrict__ qy, float *qz)
{
  const int q = list[blockIdx.x];
  const float sx = qx[q], sy = qy[q];
  if (sx < bd->g[0] || sx > bd->g[1] || sy < bd->g[2] || sy > bd->g[3]) return;
  __shared__ unsigned long long best;
  if (threadIdx.x == 0) best = LOC_NONE;
  __syncthreads();
  const int kt = LOC_TILES - 1, k = g.te[2][kt];
  const int i0 = g.ts[0][0], j0 = g.ts[1][0];
  const int ni = g.te[0][LOC_TILES - 1] - i0 + 1, nj = g.te[1][LOC_TILES - 1] - j0 + 1;
  for (int c = threadIdx.x; c < ni * nj; c += blockDim.x) {
    const int i = i0 + c % ni, j = j0 + c / ni;
    const int it = tile_of(g, 0, i), jt = tile_of(g, 1, j);
    const float *tb = bd->t[(kt * LOC_TILES + jt) * LOC_TILES + it];
    if (sx < tb[0] || sx > tb[1] || sy < tb[2] || sy > tb[3]) continue;
    float b[4];
    cell_xy(g, i, j, k, b);
    if (sx < b[0] || sx > b[1] || sy < b[2] || sy > b[3]) continue;
    V3 p[4];
    if (!top_tri(g, i, j, k, sx, sy, p)) continue;
    const int tni = g.te[0][it] - g.ts[0][it] + 1;
    unsigned long long key = ((unsigned long long)(jt * LOC_TILES + it) << 40) |
                             (unsigned long long)((j - g.ts[1][jt]) * tni + (i - g.ts[0][it]));
    atomicMin(&best, key);
  }
  __syncthreads();
  if (threadIdx.x == 0 && best != LOC_NONE) {
    const int tile = (int)(best >> 40), jt = tile / LOC_TILES, it = tile % LOC_TILES;
    const int local = (int)(best & 0xFFFFFFFFFFull);
    const int tni = g.te[0][it] - g.ts[0][it] + 1;
    const int i = g.ts[0][it] + local % tni, j = g.ts[1][jt] + local / tni;
    V3 p[4];
    const int id = top_tri(g, i, j, k, sx, sy, p);
    const float ztopo = id == 2 ? z_on_tri(sx, sy, p[3], p[2], p[0])
                                : z_on_tri(sx, sy, p[0], p[1], p[3]);
    qz[q] = ztopo - qz[q];
  }
}

/* ---- cell search ---------------------------------------------------------- */

#define LOC_CELLS_PER_THREAD 4

/* items[y] = (point, tile): every cell of the tile against the point; the
 * first hit in scan order (tile, k, j, i) by an atomic minimum */
__global__ void k_loc_cells(LocGrid g, const int2 *__restrict__ items,
                            const float *__restrict__ qx, const float *__restrict__ qy,
                            const float *__restrict__ qz, unsigned long long *key)
{
  const int2 it2 = items[blockIdx.y];
  const int q = it2.x, t = it2.y;
  const int it = t % LOC_TILES, jt = (t / LOC_TILES) % LOC_TILES, kt = t / (LOC_TILES * LOC_TILES);
  if ((*(volatile unsigned long long *)&key[q] >> 40) < (unsigned long long)t) return;
  const int i0 = g.ts[0][it], j0 = g.ts[1][jt], k0 = g.ts[2][kt];
  const int ni = g.te[0][it] - i0 + 1, nj = g.te[1][jt] - j0 + 1, nk = g.te[2][kt] - k0 + 1;
  const long long ncell = (long long)ni * nj * nk;
  const V3 p = {qx[q], qy[q], qz[q]};
  for (int m = 0; m < LOC_CELLS_PER_THREAD; m++) {
    const long long c = ((long long)blockIdx.x * LOC_CELLS_PER_THREAD + m) * blockDim.x + threadIdx.x;
    if (c >= ncell) break;
    const int i = i0 + (int)(c % ni), j = j0 + (int)((c / ni) % nj);
    const int k = k0 + (int)(c / ((long long)ni * nj));
    V3 v[8];
    float zlo = INFINITY, zhi = -INFINITY;
    for (int e = 0; e < 8; e++) {
      v[e].z = g.z[(long long)(i + (e & 1)) + (long long)(j + ((e >> 1) & 1)) * g.nx +
                   (long long)(k + (e >> 2)) * g.sl];
      zlo = fminf(zlo, v[e].z);
      zhi = fmaxf(zhi, v[e].z);
    }
    if (p.z < zlo || p.z > zhi) continue;
    float xlo = INFINITY, xhi = -INFINITY, ylo = INFINITY, yhi = -INFINITY;
    for (int e = 0; e < 8; e++) {
      V3 w = gpt(g, i + (e & 1), j + ((e >> 1) & 1), k + (e >> 2));
      v[e].x = w.x;
      v[e].y = w.y;
      xlo = fminf(xlo, w.x); xhi = fmaxf(xhi, w.x);
      ylo = fminf(ylo, w.y); yhi = fmaxf(yhi, w.y);
    }
    if (p.x < xlo || p.x > xhi || p.y < ylo || p.y > yhi) continue;
    if (!in_hexahedron(p, v)) continue;
    atomicMin(&key[q], ((unsigned long long)t << 40) | (unsigned long long)c);
  }
}

/* ---- shift inside the cell ---------------------------------------------- */

#define LOC_SAMPLE_THREADS 1024

__device__ __forceinline__ void better(float &d, int &s, float d2, int s2)
{
  if (d2 < d || (d2 == d && s2 < s)) {
    d = d2;
    s = s2;
  }
}

__global__ void __launch_bounds__(LOC_SAMPLE_THREADS)
k_loc_sample(LocGrid g, const float *__restrict__ qx, const float *__restrict__ qy,
             const float *__restrict__ qz, const unsigned long long *__restrict__ key,
             int *found, int *idx, float *shift)
{
  const int q = blockIdx.x;
  const unsigned long long kq = key[q];
  if (kq == LOC_NONE) {
    if (threadIdx.x == 0) {
      found[q] = 0;
      idx[3 * q] = idx[3 * q + 1] = idx[3 * q + 2] = -1000;
      shift[3 * q] = shift[3 * q + 1] = shift[3 * q + 2] = 0.0f;
    }
    return;
  }
  const int t = (int)(kq >> 40);
  const long long c = (long long)(kq & 0xFFFFFFFFFFull);
  const int it = t % LOC_TILES, jt = (t / LOC_TILES) % LOC_TILES, kt = t / (LOC_TILES * LOC_TILES);
  const int ni = g.te[0][it] - g.ts[0][it] + 1, nj = g.te[1][jt] - g.ts[1][jt] + 1;
  const int i = g.ts[0][it] + (int)(c % ni), j = g.ts[1][jt] + (int)((c / ni) % nj);
  const int k = g.ts[2][kt] + (int)(c / ((long long)ni * nj));
  V3 v[8];
  for (int e = 0; e < 8; e++) v[e] = gpt(g, i + (e & 1), j + ((e >> 1) & 1), k + (e >> 2));
  const V3 p = {qx[q], qy[q], qz[q]};
  constexpr int NS = LOC_SAMPLES + 1;
  float bd = INFINITY;
  int bs = 0x7fffffff;
  for (int s = threadIdx.x; s < NS * NS * NS; s += blockDim.x) {
    const int n1 = s % NS, n2 = (s / NS) % NS, n3 = s / (NS * NS);
    float lx[2], ly[2], lz[2];
    lz[1] = (float)n3 / (float)LOC_SAMPLES;
    lz[0] = (float)(1.0 - (double)lz[1]);
    ly[1] = (float)n2 / (float)LOC_SAMPLES;
    ly[0] = (float)(1.0 - (double)ly[1]);
    lx[1] = (float)n1 / (float)LOC_SAMPLES;
    lx[0] = (float)(1.0 - (double)lx[1]);
    float x = 0.f, y = 0.f, z = 0.f;
    for (int e = 0; e < 8; e++) {
      const float w = lx[e & 1] * ly[(e >> 1) & 1] * lz[e >> 2];
      x += w * v[e].x;
      y += w * v[e].y;
      z += w * v[e].z;
    }
    const float d = sqrtf((p.x - x) * (p.x - x) + (p.y - y) * (p.y - y) + (p.z - z) * (p.z - z));
    better(bd, bs, d, s);
  }
  for (int o = 16; o > 0; o >>= 1) {
    float d2 = __shfl_xor_sync(0xffffffffu, bd, o);
    int s2 = __shfl_xor_sync(0xffffffffu, bs, o);
    better(bd, bs, d2, s2);
  }
  __shared__ float sd[LOC_SAMPLE_THREADS / 32];
  __shared__ int ss[LOC_SAMPLE_THREADS / 32];
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sd[w] = bd;
    ss[w] = bs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int u = 1; u < nw; u++) better(bd, bs, sd[u], ss[u]);
    const int b[3] = {bs % NS, (bs / NS) % NS, bs / (NS * NS)};
    const int li[3] = {i, j, k};
    for (int d = 0; d < 3; d++) {
      float sh = (float)b[d] / (float)LOC_SAMPLES;
      int l = li[d];
      if (sh > 0.5f) {
        l += 1;
        sh = (float)((double)sh - 1.0);
      }
      idx[3 * q + d] = l - LOC_GHOSTS;
      shift[3 * q + d] = sh;
    }
    found[q] = 1;
  }
}

/* ---- host API ------------------------------------------------------------- */

struct cgfd_locator {
  LocGrid g;
  float *d_xyz;
  LocBounds hb;                  /* bounds on the host */
  LocBounds *d_bd;
  cudaStream_t st;
};

static void tile_ranges(LocGrid &g)
{
  const int n[3] = {g.nx - 2 * LOC_GHOSTS, g.ny - 2 * LOC_GHOSTS, g.nz - 2 * LOC_GHOSTS};
  for (int d = 0; d < 3; d++) {
    const int avg = n[d] / LOC_TILES, left = n[d] % LOC_TILES;
    for (int t = 0; t < LOC_TILES; t++) {
      g.ts[d][t] = t == 0 ? LOC_GHOSTS : g.te[d][t - 1] + 1;
      g.te[d][t] = g.ts[d][t] + avg - 1 + (t < left ? 1 : 0);
    }
  }
}

extern "C" void cgfd_locator_destroy(cgfd_locator_t *L)
{
  if (!L) return;
  if (L->d_xyz) cudaFree(L->d_xyz);
  if (L->d_bd) cudaFree(L->d_bd);
  if (L->st) cudaStreamDestroy(L->st);
  delete L;
}

extern "C" int cgfd_locator_create(int nx, int ny, int nz, const float *x3d,
                                   const float *y3d, const float *z3d, cgfd_locator_t **out)
{
  if (!out) return loc_err(CGFD_EINVAL, "null output handle");
  *out = nullptr;
  if (nx < 2 * LOC_GHOSTS + 1 || ny < 2 * LOC_GHOSTS + 1 || nz < 2 * LOC_GHOSTS + 1)
    return loc_err(CGFD_EINVAL, "grid %dx%dx%d: needs at least one point inside 3 ghost "
                                "layers per side", nx, ny, nz);
  if (!x3d || !y3d || !z3d) return loc_err(CGFD_EINVAL, "grid coordinates missing");
  cgfd_locator_t *L = new cgfd_locator_t();
  L->g.nx = nx;
  L->g.ny = ny;
  L->g.nz = nz;
  L->g.sl = (long long)nx * ny;
  tile_ranges(L->g);
  const size_t vol = (size_t)L->g.sl * nz;
#define LTRY(call)                                                             \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      int r_ = loc_err(CGFD_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
      cgfd_locator_destroy(L);                                                 \
      return r_;                                                               \
    }                                                                          \
  } while (0)
  LTRY(cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking));
  LTRY(cudaMalloc((void **)&L->d_xyz, 3 * vol * sizeof(float)));
  LTRY(cudaMalloc((void **)&L->d_bd, sizeof(LocBounds)));
  L->g.x = L->d_xyz;
  L->g.y = L->d_xyz + vol;
  L->g.z = L->d_xyz + 2 * vol;
  LTRY(cudaMemcpyAsync(L->d_xyz, x3d, vol * sizeof(float), cudaMemcpyHostToDevice, L->st));
  LTRY(cudaMemcpyAsync(L->d_xyz + vol, y3d, vol * sizeof(float), cudaMemcpyHostToDevice, L->st));
  LTRY(cudaMemcpyAsync(L->d_xyz + 2 * vol, z3d, vol * sizeof(float), cudaMemcpyHostToDevice,
                       L->st));
  /* bound keys: global min/max start at the extremes, tiles at +-1e26 as
   * the reference initialises them (forward/gd_t.c:1837-1843) */
  std::vector<unsigned> keys(6 + 6 * LOC_NT);
  for (int e = 0; e < 6; e++) keys[e] = e % 2 ? 0u : 0xFFFFFFFFu;
  for (int t = 0; t < LOC_NT; t++)
    for (int e = 0; e < 6; e++) keys[6 + 6 * t + e] = ord_key_host(e % 2 ? -1.0e26f : 1.0e26f);
  unsigned *d_keys = nullptr;
  LTRY(cudaMalloc((void **)&d_keys, keys.size() * sizeof(unsigned)));
  cudaError_t e = cudaMemcpyAsync(d_keys, keys.data(), keys.size() * sizeof(unsigned),
                                  cudaMemcpyHostToDevice, L->st);
  if (e == cudaSuccess) {
    k_loc_global_bounds<<<152 * 4, 256, 0, L->st>>>(L->g.x, L->g.y, L->g.z, (long long)vol,
                                                    d_keys);
    k_loc_tile_bounds<<<dim3(32, LOC_NT), 256, 0, L->st>>>(L->g, d_keys + 6);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(keys.data(), d_keys, keys.size() * sizeof(unsigned),
                        cudaMemcpyDeviceToHost, L->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L->st);
  cudaFree(d_keys);
  LTRY(e);
  for (int v = 0; v < 6; v++) L->hb.g[v] = ord_val(keys[v]);
  for (int t = 0; t < LOC_NT; t++)
    for (int v = 0; v < 6; v++) L->hb.t[t][v] = ord_val(keys[6 + 6 * t + v]);
  LTRY(cudaMemcpyAsync(L->d_bd, &L->hb, sizeof(LocBounds), cudaMemcpyHostToDevice, L->st));
  LTRY(cudaStreamSynchronize(L->st));
#undef LTRY
  *out = L;
  return 0;
}

extern "C" int cgfd_locator_locate(cgfd_locator_t *L, int n, const float *x, const float *y,
                                   const float *z, const int *is_depth, int *found,
                                   int *index, float *shift, float *z_located)
{
  if (!L) return loc_err(CGFD_EINVAL, "null locator");
  if (n < 0) return loc_err(CGFD_EINVAL, "negative point count");
  if (n == 0) return 0;
  if (!x || !y || !z || !found || !index || !shift)
    return loc_err(CGFD_EINVAL, "null point or output array");
  float *d_q = nullptr;
  int *d_i = nullptr;
  unsigned long long *d_key = nullptr;
  int2 *d_items = nullptr;
  int rc = 0;
  std::vector<int> dl;
  for (int q = 0; q < n; q++)
    if (is_depth && is_depth[q]) dl.push_back(q);
  std::vector<float> zq(z, z + n);
  std::vector<int2> items;
  cudaError_t e;
#define LGO(call)                                                              \
  do {                                                                         \
    e = (call);                                                                \
    if (e != cudaSuccess) {                                                    \
      rc = loc_err(CGFD_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e)); \
      goto done;                                                               \
    }                                                                          \
  } while (0)
  LGO(cudaMalloc((void **)&d_q, 3 * (size_t)n * sizeof(float)));
  LGO(cudaMalloc((void **)&d_i, (size_t)(n + 4 * n) * sizeof(int) + 3 * (size_t)n * sizeof(float)));
  LGO(cudaMalloc((void **)&d_key, (size_t)n * sizeof(unsigned long long)));
  LGO(cudaMemcpyAsync(d_q, x, n * sizeof(float), cudaMemcpyHostToDevice, L->st));
  LGO(cudaMemcpyAsync(d_q + n, y, n * sizeof(float), cudaMemcpyHostToDevice, L->st));
  LGO(cudaMemcpyAsync(d_q + 2 * n, z, n * sizeof(float), cudaMemcpyHostToDevice, L->st));
  if (!dl.empty()) {
    LGO(cudaMemcpyAsync(d_i, dl.data(), dl.size() * sizeof(int), cudaMemcpyHostToDevice, L->st));
    k_loc_depth<<<(int)dl.size(), 256, 0, L->st>>>(L->g, L->d_bd, d_i, d_q, d_q + n, d_q + 2 * n);
    LGO(cudaGetLastError());
    LGO(cudaMemcpyAsync(zq.data(), d_q + 2 * n, n * sizeof(float), cudaMemcpyDeviceToHost, L->st));
    LGO(cudaStreamSynchronize(L->st));
  }
  /* (point, tile) pairs whose tile box holds the point, in scan order */
  for (int q = 0; q < n; q++) {
    const float sx = x[q], sy = y[q], sz = zq[q];
    const float *gb = L->hb.g;
    if (sx < gb[0] || sx > gb[1] || sy < gb[2] || sy > gb[3] || sz < gb[4] || sz > gb[5])
      continue;
    for (int t = 0; t < LOC_NT; t++) {
      const float *tb = L->hb.t[t];
      if (sx < tb[0] || sx > tb[1] || sy < tb[2] || sy > tb[3] || sz < tb[4] || sz > tb[5])
        continue;
      items.push_back(make_int2(q, t));
    }
  }
  LGO(cudaMemsetAsync(d_key, 0xFF, (size_t)n * sizeof(unsigned long long), L->st));
  if (!items.empty()) {
    LGO(cudaMalloc((void **)&d_items, items.size() * sizeof(int2)));
    LGO(cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(int2),
                        cudaMemcpyHostToDevice, L->st));
    long long maxcell = 0;
    for (int t = 0; t < LOC_NT; t++) {
      const int it = t % LOC_TILES, jt = (t / LOC_TILES) % LOC_TILES, kt = t / 16;
      long long c = (long long)(L->g.te[0][it] - L->g.ts[0][it] + 1) *
                    (L->g.te[1][jt] - L->g.ts[1][jt] + 1) * (L->g.te[2][kt] - L->g.ts[2][kt] + 1);
      if (c > maxcell) maxcell = c;
    }
    const int per_block = 256 * LOC_CELLS_PER_THREAD;
    const int nbx = (int)((maxcell + per_block - 1) / per_block);
    for (size_t b0 = 0; b0 < items.size(); b0 += 65535) {
      const int ny = (int)std::min<size_t>(65535, items.size() - b0);
      k_loc_cells<<<dim3(nbx, ny), 256, 0, L->st>>>(L->g, d_items + b0, d_q, d_q + n,
                                                     d_q + 2 * n, d_key);
      LGO(cudaGetLastError());
    }
  }
  {
    int *d_found = d_i + n, *d_idx = d_i + 2 * n;
    float *d_shift = (float *)(d_i + 5 * n);
    k_loc_sample<<<n, LOC_SAMPLE_THREADS, 0, L->st>>>(L->g, d_q, d_q + n, d_q + 2 * n, d_key,
                                                      d_found, d_idx, d_shift);
    LGO(cudaGetLastError());
    LGO(cudaMemcpyAsync(found, d_found, n * sizeof(int), cudaMemcpyDeviceToHost, L->st));
    LGO(cudaMemcpyAsync(index, d_idx, 3 * (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, L->st));
    LGO(cudaMemcpyAsync(shift, d_shift, 3 * (size_t)n * sizeof(float), cudaMemcpyDeviceToHost,
                        L->st));
    LGO(cudaStreamSynchronize(L->st));
  }
  if (z_located) memcpy(z_located, zq.data(), n * sizeof(float));
done:
#undef LGO
  if (e != cudaSuccess) cudaStreamSynchronize(L->st);
  if (d_q) cudaFree(d_q);
  if (d_i) cudaFree(d_i);
  if (d_key) cudaFree(d_key);
  if (d_items) cudaFree(d_items);
  return rc;
}
