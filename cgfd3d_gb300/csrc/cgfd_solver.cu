/*
 * cgfd_solver.cu -- device-resident RK4 time loop for CGFD3D, sm_103a.
 *
 * Implements the flat C ABI of include/cgfd3d_gpu.h.  One solver object
 * owns every array the time loop touches in HBM; a step is, per RK stage,
 * one fused interior stage launch (cgfd_stage3.cuh) and one CFS-PML launch
 * per enabled face (cgfd_pml.cuh), then the surface and receiver launches.
 * Media: isotropic elastic, VTI elastic and GMB visco-elastic isotropic
 * (cgfd_media.cuh); their kernels are compiled in cgfd_launch_*.cu.
 *
 * Reference: forward/drv_rk_curv_col.c:27-556 (time loop),
 * forward/sv_curv_col_el_iso.c:1258-1375, forward/sv_curv_col_el_vti.c:
 * 1085-1206, forward/sv_curv_col_vis_iso.c:353-507 (free-surface matrices),
 * forward/sv_curv_col_vis_iso.c:509-623 (visco surface stress rotation),
 * forward/io_funcs.c:1584-1645 (receivers, lines).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cgfd3d_gpu.h"
#include "cgfd_common.h"
#include "cgfd_launch.h"
#include "cgfd_media.cuh"
#include "cgfd_stage2.cuh"
#include "cgfd_stage3.cuh"

/* ------------------------------------------------------------------------ */
/* errors                                                                    */
/* ------------------------------------------------------------------------ */

static thread_local std::string g_err;

static int set_err(int code, const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

/* CGFD_TRACE=1: phase timings of the solver set-up on stderr (the device
 * work of each phase is waited for, so the trace changes the timing) */
struct SetupTrace {
  bool on = false;
  cudaStream_t st = nullptr;
  double t0 = 0.0;
  static double now()
  {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
  }
  void start(cudaStream_t s)
  {
    const char *e = getenv("CGFD_TRACE");
    on = e && atoi(e) != 0;
    st = s;
    t0 = now();
  }
  void mark(const char *what)
  {
    if (!on) return;
    cudaStreamSynchronize(st);
    double t = now();
    fprintf(stderr, "cgfd trace: %-28s %8.2f ms\n", what, 1e3 * (t - t0));
    t0 = t;
  }
};

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return set_err(CGFD_ECUDA, "%s failed: %s (%s:%d)", #call,              \
                     cudaGetErrorString(e_), __FILE__, __LINE__);             \
  } while (0)

extern "C" const char *cgfd_last_error(void) { return g_err.c_str(); }

__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg)
{
  g_err = msg;
  return code;
}
extern "C" int cgfd_abi_version(void) { return CGFD_ABI_VERSION; }

/* ------------------------------------------------------------------------ */
/* kernels                                                                   */
/* ------------------------------------------------------------------------ */

#define V1_TX 32
#define V1_TY 4
#define V1_KCHUNK 8

template <int BX, int BY, int BZ, int KIND>
__global__ void __launch_bounds__(V1_TX *V1_TY)
    k_stage(const __grid_constant__ StageArgs a)
{
  int i = a.g.ni1 + blockIdx.x * V1_TX + threadIdx.x;
  int j = a.g.nj1 + blockIdx.y * V1_TY + threadIdx.y;
  if (i > a.g.ni2 || j > a.g.nj2) return;
  int k0 = a.g.nk1 + blockIdx.z * V1_KCHUNK;
  int k1 = min(k0 + V1_KCHUNK - 1, a.g.nk2);
  for (int k = k0; k <= k1; k++) stage_point<BX, BY, BZ, KIND>(a, i, j, k);
}

/* free-surface conversion matrices A^-1 B, A^-1 C, A^-1 per surface point
 * (forward/sv_curv_col_el_iso.c:1304-1372, inverse lib/fdlib_math.c:8-35) */
__global__ void k_dvh2dvz_iso(DevGrid g, const float *__restrict__ xix,
                              const float *__restrict__ xiy,
                              const float *__restrict__ xiz,
                              const float *__restrict__ etx,
                              const float *__restrict__ ety,
                              const float *__restrict__ etz,
                              const float *__restrict__ ztx,
                              const float *__restrict__ zty,
                              const float *__restrict__ ztz,
                              const float *__restrict__ lam3,
                              const float *__restrict__ mu3, float *mVx,
                              float *mVy, float *mF)
{
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  long long q = (i + g.xoff) + (long long)j * g.px + (long long)g.nk2 * g.sl;
  float e11 = xix[q], e12 = xiy[q], e13 = xiz[q];
  float e21 = etx[q], e22 = ety[q], e23 = etz[q];
  float e31 = ztx[q], e32 = zty[q], e33 = ztz[q];
  float lam = lam3[q], mu = mu3[q];
  float l2m = lam + 2.0f * mu;
  float A[3][3], B[3][3], C[3][3];
  A[0][0] = l2m * e31 * e31 + mu * (e32 * e32 + e33 * e33);
  A[0][1] = lam * e31 * e32 + mu * e32 * e31;
  A[0][2] = lam * e31 * e33 + mu * e33 * e31;
  A[1][0] = lam * e32 * e31 + mu * e31 * e32;
  A[1][1] = l2m * e32 * e32 + mu * (e31 * e31 + e33 * e33);
  A[1][2] = lam * e32 * e33 + mu * e33 * e32;
  A[2][0] = lam * e33 * e31 + mu * e31 * e33;
  A[2][1] = lam * e33 * e32 + mu * e32 * e33;
  A[2][2] = l2m * e33 * e33 + mu * (e31 * e31 + e32 * e32);
  /* adjugate / determinant */
  float v[3][3];
  v[0][0] = A[1][1] * A[2][2] - A[2][1] * A[1][2];
  v[0][1] = A[2][1] * A[0][2] - A[0][1] * A[2][2];
  v[0][2] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  v[1][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  v[1][1] = A[0][0] * A[2][2] - A[2][0] * A[0][2];
  v[1][2] = A[1][0] * A[0][2] - A[0][0] * A[1][2];
  v[2][0] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  v[2][1] = A[2][0] * A[0][1] - A[0][0] * A[2][1];
  v[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  float det = v[0][0] * A[0][0] + v[0][1] * A[1][0] + v[0][2] * A[2][0];
  det = 1.0f / det;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) A[r][c] = v[r][c] * det;
  B[0][0] = -l2m * e31 * e11 - mu * (e32 * e12 + e33 * e13);
  B[0][1] = -lam * e31 * e12 - mu * e32 * e11;
  B[0][2] = -lam * e31 * e13 - mu * e33 * e11;
  B[1][0] = -lam * e32 * e11 - mu * e31 * e12;
  B[1][1] = -l2m * e32 * e12 - mu * (e31 * e11 + e33 * e13);
  B[1][2] = -lam * e32 * e13 - mu * e33 * e12;
  B[2][0] = -lam * e33 * e11 - mu * e31 * e13;
  B[2][1] = -lam * e33 * e12 - mu * e32 * e13;
  B[2][2] = -l2m * e33 * e13 - mu * (e31 * e11 + e32 * e12);
  C[0][0] = -l2m * e31 * e21 - mu * (e32 * e22 + e33 * e23);
  C[0][1] = -lam * e31 * e22 - mu * e32 * e21;
  C[0][2] = -lam * e31 * e23 - mu * e33 * e21;
  C[1][0] = -lam * e32 * e21 - mu * e31 * e22;
  C[1][1] = -l2m * e32 * e22 - mu * (e31 * e21 + e33 * e23);
  C[1][2] = -lam * e32 * e23 - mu * e33 * e22;
  C[2][0] = -lam * e33 * e21 - mu * e31 * e23;
  C[2][1] = -lam * e33 * e22 - mu * e32 * e23;
  C[2][2] = -l2m * e33 * e23 - mu * (e31 * e21 + e32 * e22);
  long long ij = (i + (long long)j * g.nx) * 9;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      float ab = 0.f, ac = 0.f;
      for (int m = 0; m < 3; m++) {
        ab += A[r][m] * B[m][c];
        ac += A[r][m] * C[m][c];
      }
      mVx[ij + r * 3 + c] = ab;
      mVy[ij + r * 3 + c] = ac;
      mF[ij + r * 3 + c] = A[r][c];
    }
}

/* 3x3 inverse by adjugate / determinant, as lib/fdlib_math.c:8-35 */
__device__ __forceinline__ void inv3_dev(float A[3][3])
{
  float v[3][3];
  v[0][0] = A[1][1] * A[2][2] - A[2][1] * A[1][2];
  v[0][1] = A[2][1] * A[0][2] - A[0][1] * A[2][2];
  v[0][2] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
  v[1][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
  v[1][1] = A[0][0] * A[2][2] - A[2][0] * A[0][2];
  v[1][2] = A[1][0] * A[0][2] - A[0][0] * A[1][2];
  v[2][0] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
  v[2][1] = A[2][0] * A[0][1] - A[0][0] * A[2][1];
  v[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
  float det = 1.0f / (v[0][0] * A[0][0] + v[0][1] * A[1][0] + v[0][2] * A[2][0]);
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) A[r][c] = v[r][c] * det;
}

/* VTI free-surface matrices -A^-1 B, -A^-1 C per surface point
 * (forward/sv_curv_col_el_vti.c:1149-1203): A, B, C are the zeta-zeta,
 * zeta-xi and zeta-eta contractions of the VTI stiffness */
__global__ void k_dvh2dvz_vti(DevGrid g, const float *__restrict__ M,
                              const float *__restrict__ med, float *mVx,
                              float *mVy)
{
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  long long q = (i + g.xoff) + (long long)j * g.px + (long long)g.nk2 * g.sl;
  const long long v = g.vol;
  float xi[3] = {M[v + q], M[2 * v + q], M[3 * v + q]};
  float et[3] = {M[4 * v + q], M[5 * v + q], M[6 * v + q]};
  float zt[3] = {M[7 * v + q], M[8 * v + q], M[9 * v + q]};
  MedPt m = med_from<MED_VTI, true>(med + q, v);
  /* K(a, b)[r][c]: row r of the traction on the plane of normal a produced
   * by the velocity gradient along direction b, component c (VTI stiffness) */
  auto K = [&](const float *a, const float *b, float out[3][3]) {
    out[0][0] = m.c11 * b[0] * a[0] + m.c66 * b[1] * a[1] + m.c55 * b[2] * a[2];
    out[0][1] = m.c12 * b[1] * a[0] + m.c66 * b[0] * a[1];
    out[0][2] = m.c13 * b[2] * a[0] + m.c55 * b[0] * a[2];
    out[1][0] = m.c66 * b[1] * a[0] + m.c12 * b[0] * a[1];
    out[1][1] = m.c66 * b[0] * a[0] + m.c11 * b[1] * a[1] + m.c55 * b[2] * a[2];
    out[1][2] = m.c13 * b[2] * a[1] + m.c55 * b[1] * a[2];
    out[2][0] = m.c55 * b[2] * a[0] + m.c13 * b[0] * a[2];
    out[2][1] = m.c55 * b[2] * a[1] + m.c13 * b[1] * a[2];
    out[2][2] = m.c55 * b[0] * a[0] + m.c55 * b[1] * a[1] + m.c33 * b[2] * a[2];
  };
  float A[3][3], B[3][3], C[3][3];
  K(zt, zt, A);
  K(zt, xi, B);
  K(zt, et, C);
  inv3_dev(A);
  long long ij = (i + (long long)j * g.nx) * 9;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      float ab = 0.f, ac = 0.f;
      for (int k = 0; k < 3; k++) {
        ab += A[r][k] * B[k][c];
        ac += A[r][k] * C[k][c];
      }
      mVx[ij + r * 3 + c] = -ab;
      mVy[ij + r * 3 + c] = -ac;
    }
}

/* anisotropic free-surface matrices (forward/sv_curv_col_el_aniso.c:
 * 1267-1423): matVx2Vz = -A^-1 B, matVy2Vz = -A^-1 C with
 * K(a, b)[r][c] = sum over n, m of C(V(r,n), V(c,m)) b_m a_n, the traction
 * on the plane of normal a from the gradient along b (A = K(zt, zt),
 * B = K(zt, xi), C = K(zt, et)) */
__global__ void k_dvh2dvz_ani(DevGrid g, const float *__restrict__ M,
                              const float *__restrict__ med, float *mVx, float *mVy)
{
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  long long q = (i + g.xoff) + (long long)j * g.px + (long long)g.nk2 * g.sl;
  const long long v = g.vol;
  float xi[3] = {M[v + q], M[2 * v + q], M[3 * v + q]};
  float et[3] = {M[4 * v + q], M[5 * v + q], M[6 * v + q]};
  float zt[3] = {M[7 * v + q], M[8 * v + q], M[9 * v + q]};
  float c[21];
  for (int n = 0; n < 21; n++) c[n] = med[(n + 1) * v + q];
  const int vg[3][3] = {{1, 6, 5}, {6, 2, 4}, {5, 4, 3}};
  const int off[7] = {0, 0, 6, 11, 15, 18, 20};
  auto C = [&](int I, int J) {
    int a = I < J ? I : J, b = I < J ? J : I;
    return c[off[a] + b - a];
  };
  auto K = [&](const float *a, const float *b, float out[3][3]) {
    for (int r = 0; r < 3; r++)
      for (int cc = 0; cc < 3; cc++) {
        float s = 0.f;
        for (int n = 0; n < 3; n++)
          for (int m = 0; m < 3; m++) s += C(vg[r][n], vg[cc][m]) * b[m] * a[n];
        out[r][cc] = s;
      }
  };
  float A[3][3], B[3][3], Cm[3][3];
  K(zt, zt, A);
  K(zt, xi, B);
  K(zt, et, Cm);
  inv3_dev(A);
  long long ij = (i + (long long)j * g.nx) * 9;
  for (int r = 0; r < 3; r++)
    for (int cc = 0; cc < 3; cc++) {
      float ab = 0.f, ac = 0.f;
      for (int k = 0; k < 3; k++) {
        ab += A[r][k] * B[k][cc];
        ac += A[r][k] * Cm[k][cc];
      }
      mVx[ij + r * 3 + cc] = -ab;
      mVy[ij + r * 3 + cc] = -ac;
    }
}

/* visco-elastic free-surface matrices (forward/sv_curv_col_vis_iso.c:
 * 416-503): the isotropic A^-1 B, A^-1 C and the rotation matrix D of the
 * local surface frame (rows: the in-plane direction normal to the eta
 * tangent, the eta tangent, the zeta normal), from the grid's eta tangent
 * (centred 7-point operator along j on the coordinates of the surface
 * plane, forward/fd_t.c:152-176) */
__global__ void k_dvh2dvz_vis(DevGrid g, const float *__restrict__ M,
                              const float *__restrict__ med,
                              const float *__restrict__ x2,
                              const float *__restrict__ y2,
                              const float *__restrict__ z2, float *mVx,
                              float *mVy, float *mD)
{
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  long long q = (i + g.xoff) + (long long)j * g.px + (long long)g.nk2 * g.sl;
  const long long v = g.vol;
  const float e11 = M[v + q], e12 = M[2 * v + q], e13 = M[3 * v + q];
  const float e21 = M[4 * v + q], e22 = M[5 * v + q], e23 = M[6 * v + q];
  const float e31 = M[7 * v + q], e32 = M[8 * v + q], e33 = M[9 * v + q];
  const float lam = med[v + q], mu = med[2 * v + q];
  const float l2m = lam + 2.0f * mu;
  const float fc[7] = {-0.02084f, 0.1667f, -0.7709f, 0.0f, 0.7709f, -0.1667f, 0.02084f};
  float xet = 0.f, yet = 0.f, zet = 0.f;
  for (int n = 0; n < 7; n++) {
    long long p2 = i + (long long)(j + n - 3) * g.nx;
    xet += fc[n] * x2[p2];
    yet += fc[n] * y2[p2];
    zet += fc[n] * z2[p2];
  }
  float e_n = 1.0f / sqrtf(xet * xet + yet * yet + zet * zet);
  float e_m = 1.0f / sqrtf(e31 * e31 + e32 * e32 + e33 * e33);
  float e_nm = e_n * e_m;
  float A[3][3], B[3][3], C[3][3];
  A[0][0] = l2m * e31 * e31 + mu * (e32 * e32 + e33 * e33);
  A[0][1] = lam * e31 * e32 + mu * e32 * e31;
  A[0][2] = lam * e31 * e33 + mu * e33 * e31;
  A[1][0] = lam * e32 * e31 + mu * e31 * e32;
  A[1][1] = l2m * e32 * e32 + mu * (e31 * e31 + e33 * e33);
  A[1][2] = lam * e32 * e33 + mu * e33 * e32;
  A[2][0] = lam * e33 * e31 + mu * e31 * e33;
  A[2][1] = lam * e33 * e32 + mu * e32 * e33;
  A[2][2] = l2m * e33 * e33 + mu * (e31 * e31 + e32 * e32);
  inv3_dev(A);
  B[0][0] = -l2m * e31 * e11 - mu * (e32 * e12 + e33 * e13);
  B[0][1] = -lam * e31 * e12 - mu * e32 * e11;
  B[0][2] = -lam * e31 * e13 - mu * e33 * e11;
  B[1][0] = -lam * e32 * e11 - mu * e31 * e12;
  B[1][1] = -l2m * e32 * e12 - mu * (e31 * e11 + e33 * e13);
  B[1][2] = -lam * e32 * e13 - mu * e33 * e12;
  B[2][0] = -lam * e33 * e11 - mu * e31 * e13;
  B[2][1] = -lam * e33 * e12 - mu * e32 * e13;
  B[2][2] = -l2m * e33 * e13 - mu * (e31 * e11 + e32 * e12);
  C[0][0] = -l2m * e31 * e21 - mu * (e32 * e22 + e33 * e23);
  C[0][1] = -lam * e31 * e22 - mu * e32 * e21;
  C[0][2] = -lam * e31 * e23 - mu * e33 * e21;
  C[1][0] = -lam * e32 * e21 - mu * e31 * e22;
  C[1][1] = -l2m * e32 * e22 - mu * (e31 * e21 + e33 * e23);
  C[1][2] = -lam * e32 * e23 - mu * e33 * e22;
  C[2][0] = -lam * e33 * e21 - mu * e31 * e23;
  C[2][1] = -lam * e33 * e22 - mu * e32 * e23;
  C[2][2] = -l2m * e33 * e23 - mu * (e31 * e21 + e32 * e22);
  float D[3][3] = {{(yet * e33 - zet * e32) * e_nm, (zet * e31 - xet * e33) * e_nm,
                    (xet * e32 - yet * e31) * e_nm},
                   {xet * e_n, yet * e_n, zet * e_n},
                   {e31 * e_m, e32 * e_m, e33 * e_m}};
  long long ij = (i + (long long)j * g.nx) * 9;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      float ab = 0.f, ac = 0.f;
      for (int k = 0; k < 3; k++) {
        ab += A[r][k] * B[k][c];
        ac += A[r][k] * C[k][c];
      }
      mVx[ij + r * 3 + c] = ab;
      mVy[ij + r * 3 + c] = ac;
      mD[ij + r * 3 + c] = D[r][c];
    }
}

/* visco-elastic free surface after the last stage: the surface stress is
 * rotated into the local frame D, its components on the surface normal are
 * dropped and it is rotated back, T <- D^T P(D T D^T) D
 * (forward/sv_curv_col_vis_iso.c:509-623); surface plane of the end level */
__global__ void k_vis_free(DevGrid g, float *w, const float *__restrict__ mD)
{
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  long long q = (i + g.xoff) + (long long)j * g.px + (long long)g.nk2 * g.sl;
  const long long v = g.vol;
  const float *D = mD + (i + (long long)j * g.nx) * 9;
  float d11 = D[0], d12 = D[1], d13 = D[2], d21 = D[3], d22 = D[4], d23 = D[5];
  float Txx = w[C_TXX * v + q], Tyy = w[C_TYY * v + q], Tzz = w[C_TZZ * v + q];
  float Txy = w[C_TXY * v + q], Txz = w[C_TXZ * v + q], Tyz = w[C_TYZ * v + q];
  float l00 = d11 * d11 * Txx + d12 * d12 * Tyy + d13 * d13 * Tzz +
              2.0f * (d11 * d12 * Txy + d11 * d13 * Txz + d12 * d13 * Tyz);
  float l01 = d11 * d21 * Txx + d12 * d22 * Tyy + d13 * d23 * Tzz +
              (d11 * d22 + d12 * d21) * Txy + (d11 * d23 + d21 * d13) * Txz +
              (d12 * d23 + d22 * d13) * Tyz;
  float l11 = d21 * d21 * Txx + d22 * d22 * Tyy + d23 * d23 * Tzz +
              2.0f * (d21 * d22 * Txy + d21 * d23 * Txz + d22 * d23 * Tyz);
  /* Tg = D^T Tl D with Tl = [[l00, l01, 0], [l01, l11, 0], [0, 0, 0]] */
  float Tg[3][3];
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      float dr0 = D[0 * 3 + r], dr1 = D[1 * 3 + r];
      float dc0 = D[0 * 3 + c], dc1 = D[1 * 3 + c];
      Tg[r][c] = (dr0 * l00 + dr1 * l01) * dc0 + (dr0 * l01 + dr1 * l11) * dc1;
    }
  w[C_TXX * v + q] = Tg[0][0];
  w[C_TYY * v + q] = Tg[1][1];
  w[C_TZZ * v + q] = Tg[2][2];
  w[C_TXY * v + q] = Tg[0][1];
  w[C_TXZ * v + q] = Tg[0][2];
  w[C_TYZ * v + q] = Tg[1][2];
}

/* surface force layers of one stage (forward/src_t.c:153-314): per surface
 * column (i, j) the traction TxSrc..TzSrc and velocity-rate VxSrc..VzSrc
 * sums over the surface forces active at step *d_it, in source order.  A
 * point force adds its value at its column (rate over the Jacobian at the
 * source point), a Gaussian one the surface layer of its weights. */
__global__ void k_surf_layer(DevGrid g, int nsf, const SurfForce *__restrict__ sf,
                             const float *__restrict__ wsurf,
                             const float *__restrict__ jac,
                             const int *__restrict__ it_begin,
                             const int *__restrict__ it_end,
                             const float *__restrict__ Fx, const float *__restrict__ Fy,
                             const float *__restrict__ Fz, const float *__restrict__ Rx,
                             const float *__restrict__ Ry, const float *__restrict__ Rz,
                             int max_nt, int max_stage, int istage,
                             const int *__restrict__ d_it, float *TS, float *VS)
{
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  const int it = *d_it;
  const long long n2 = (long long)g.nx * g.ny, i2 = i + (long long)j * g.nx;
  float t[3] = {0.f, 0.f, 0.f}, v[3] = {0.f, 0.f, 0.f};
  for (int n = 0; n < nsf; n++) {
    const SurfForce f = sf[n];
    if (it < it_begin[f.is] || it > it_end[f.is]) continue;
    const int di = i - f.si, dj = j - f.sj;
    if (di < -f.half || di > f.half || dj < -f.half || dj > f.half) continue;
    const long long tt = ((long long)f.is * max_nt + (it - it_begin[f.is])) * max_stage + istage;
    const long long tr = ((long long)f.n * max_nt + (it - it_begin[f.is])) * max_stage + istage;
    const int k = f.half == 0 ? f.sk : g.nk2;
    const float rj = 1.0f / jac[(i + g.xoff) + (long long)j * g.px + (long long)k * g.sl];
    const float c = f.half == 0 ? 1.0f : wsurf[f.w0 + (dj + f.half) * (2 * f.half + 1) + di + f.half];
    t[0] += Fx[tt] * c; t[1] += Fy[tt] * c; t[2] += Fz[tt] * c;
    v[0] += Rx[tr] * c * rj; v[1] += Ry[tr] * c * rj; v[2] += Rz[tr] * c * rj;
  }
  for (int m = 0; m < 3; m++) {
    TS[m * n2 + i2] = t[m];
    VS[m * n2 + i2] = v[m];
  }
}

/* grid metrics of the physical points from the node coordinates
 * (forward/gd_t.c:238-290): centred 7-point derivatives along i, j, k
 * (forward/fd_t.c:152-176), the Jacobian (x_xi x x_et) . x_zt, and the
 * contravariant metrics as cross products over it.  Grid (ni/32, nj/8, nk). */
__global__ void k_metric(DevGrid g, const float *__restrict__ x,
                         const float *__restrict__ y, const float *__restrict__ z,
                         float *m)
{
  const int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = g.nk1 + blockIdx.z;
  if (i > g.ni2 || j > g.nj2) return;
  const long long q = (i + g.xoff) + (long long)j * g.px + (long long)k * g.sl;
  const float fc[7] = {-0.02084f, 0.1667f, -0.7709f, 0.0f, 0.7709f, -0.1667f, 0.02084f};
  const float *X[3] = {x, y, z};
  const long long st[3] = {1, g.px, g.sl};
  float d[3][3];
#pragma unroll
  for (int ax = 0; ax < 3; ax++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float v = 0.f;
#pragma unroll
      for (int n = 0; n < 7; n++) v += fc[n] * X[c][q + (n - 3) * st[ax]];
      d[ax][c] = v;
    }
  auto cross = [](const float *A, const float *B, float *C) {
    C[0] = A[1] * B[2] - A[2] * B[1];
    C[1] = A[2] * B[0] - A[0] * B[2];
    C[2] = A[0] * B[1] - A[1] * B[0];
  };
  float gv[3];
  cross(d[0], d[1], gv);
  const float jac = gv[0] * d[2][0] + gv[1] * d[2][1] + gv[2] * d[2][2];
  const long long v = g.vol;
  m[q] = jac;
  const int pa[3] = {1, 2, 0}, pb[3] = {2, 0, 1};
#pragma unroll
  for (int r = 0; r < 3; r++) {
    cross(d[pa[r]], d[pb[r]], gv);
#pragma unroll
    for (int c = 0; c < 3; c++) m[(1 + 3 * r + c) * v + q] = gv[c] / jac;
  }
}

/* ghost layers of the metrics: mirrored about the physical boundary along
 * x, then y, then z (forward/gd_t.c:291-401) -- a ghost point takes the
 * value of the physical point whose index is mirrored in every direction */
__global__ void k_metric_ghost(DevGrid g, float *m)
{
  const long long n = (long long)g.nx * g.ny * g.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.nx), j = (int)((t / g.nx) % g.ny), k = (int)(t / ((long long)g.nx * g.ny));
    const int mi = i < g.ni1 ? 2 * g.ni1 - 1 - i : (i > g.ni2 ? 2 * g.ni2 + 1 - i : i);
    const int mj = j < g.nj1 ? 2 * g.nj1 - 1 - j : (j > g.nj2 ? 2 * g.nj2 + 1 - j : j);
    const int mk = k < g.nk1 ? 2 * g.nk1 - 1 - k : (k > g.nk2 ? 2 * g.nk2 + 1 - k : k);
    if (mi == i && mj == j && mk == k) continue;
    const long long q = (i + g.xoff) + (long long)j * g.px + (long long)k * g.sl;
    const long long s = (mi + g.xoff) + (long long)mj * g.px + (long long)mk * g.sl;
    for (int c = 0; c < 10; c++) m[c * g.vol + q] = m[c * g.vol + s];
  }
}

/* source weights at their points: force coef*slw/jac, moment coef/jac
 * (forward/sv_curv_col_el.c:381-470) from the device media and metrics */
__global__ void k_src_weights(DevGrid g, SrcEntry *ent, int n,
                              const float *__restrict__ slw,
                              const float *__restrict__ jac)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float j = jac[ent[e].q], c = ent[e].coef;
  ent[e].vf = c * slw[ent[e].q] / j;
  ent[e].rjac = c / j;
}

/* receivers and lines after a step; one block; advances the step counter.
 * Trilinear weights as forward/io_funcs.c:1595-1612, which uses corner 5
 * twice and corner 4 never (harmless for receivers on a grid plane). */
__global__ void k_recv(const float *__restrict__ w, long long vol, int ncmp,
                       int nrecv, int recv_ncmp, int recv_max_nt,
                       const float *__restrict__ dijk,
                       const int *__restrict__ idx8, float *seismo,
                       int nline, int line_max_nt,
                       const int *__restrict__ line_iptr, float *line_seismo,
                       int *d_it)
{
  int it = *d_it;
  for (int t = threadIdx.x; t < nrecv * recv_ncmp; t += blockDim.x) {
    int n = t / recv_ncmp, c = t % recv_ncmp;
    const int *x = idx8 + 8 * n;
    float Lx2 = dijk[3 * n], Ly2 = dijk[3 * n + 1], Lz2 = dijk[3 * n + 2];
    float Lx1 = 1.0f - Lx2, Ly1 = 1.0f - Ly2, Lz1 = 1.0f - Lz2;
    const float *v = w + c * vol;
    seismo[((long long)n * recv_ncmp + c) * recv_max_nt + it] =
        v[x[0]] * Lx1 * Ly1 * Lz1 + v[x[1]] * Lx2 * Ly1 * Lz1 +
        v[x[2]] * Lx1 * Ly2 * Lz1 + v[x[3]] * Lx2 * Ly2 * Lz1 +
        v[x[5]] * Lx1 * Ly1 * Lz2 + v[x[5]] * Lx2 * Ly1 * Lz2 +
        v[x[6]] * Lx1 * Ly2 * Lz2 + v[x[7]] * Lx2 * Ly2 * Lz2;
  }
  for (int t = threadIdx.x; t < nline * ncmp; t += blockDim.x) {
    int n = t / ncmp, c = t % ncmp;
    line_seismo[((long long)n * ncmp + c) * line_max_nt + it] =
        w[c * vol + line_iptr[n]];
  }
  __syncthreads();
  if (threadIdx.x == 0) *d_it = it + 1;
}

/* surface peak ground motion after a step (forward/wav_t.c:379-455):
 * running maxima of |V|, |A| = |dV/dt| and |D| (D integrated with the
 * trapezoid rule), 15 maps of nx*ny in the order PGV, PGVh, PGVx, PGVy,
 * PGVz, PGA, PGAh, PGAx..z, PGD, PGDh, PGDx..z; Dis holds Dx, Dy, Dz */
__global__ void k_pg(DevGrid g, const float *__restrict__ w1,
                     const float *__restrict__ w0, float *PG, float *Dis, float dt)
{
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  long long q = (i + g.xoff) + (long long)j * g.px + (long long)g.nk2 * g.sl;
  long long s2 = (long long)g.nx * g.ny;
  long long q2 = i + (long long)j * g.nx;
  float vx1 = w1[q], vy1 = w1[g.vol + q], vz1 = w1[2 * g.vol + q];
  float vx0 = w0[q], vy0 = w0[g.vol + q], vz0 = w0[2 * g.vol + q];
  float Ax = fabsf((vx1 - vx0) / dt), Ay = fabsf((vy1 - vy0) / dt),
        Az = fabsf((vz1 - vz0) / dt);
  float Dx = Dis[q2] + 0.5f * (vx1 + vx0) * dt;
  float Dy = Dis[s2 + q2] + 0.5f * (vy1 + vy0) * dt;
  float Dz = Dis[2 * s2 + q2] + 0.5f * (vz1 + vz0) * dt;
  Dis[q2] = Dx; Dis[s2 + q2] = Dy; Dis[2 * s2 + q2] = Dz;
  float V = sqrtf(vx1 * vx1 + vy1 * vy1 + vz1 * vz1);
  float Vh = sqrtf(vx1 * vx1 + vy1 * vy1);
  float A = sqrtf(Ax * Ax + Ay * Ay + Az * Az);
  float Ah = sqrtf(Ax * Ax + Ay * Ay);
  float D = sqrtf(Dx * Dx + Dy * Dy + Dz * Dz);
  float Dh = sqrtf(Dx * Dx + Dy * Dy);
  float v[15] = {V, Vh, fabsf(vx1), fabsf(vy1), fabsf(vz1), A, Ah, Ax, Ay, Az,
                 D, Dh, fabsf(Dx), fabsf(Dy), fabsf(Dz)};
#pragma unroll
  for (int m = 0; m < 15; m++) {
    float *p = PG + m * s2 + q2;
    if (*p < v[m]) *p = v[m];
  }
}

__global__ void k_nonfinite(const float *__restrict__ w, long long n, int *flag)
{
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long stride = (long long)gridDim.x * blockDim.x;
  int bad = 0;
  for (; t < n; t += stride) bad |= !isfinite(w[t]);
  if (bad) atomicOr(flag, 1);
}

/* Gathers output boxes of one wavefield level into a packed buffer: box
 * after box, component, k, j, i (i fastest).  off[] holds each box's first
 * packed index (ascending), total the packed length. */
__global__ void k_pack_boxes(const float *__restrict__ w, long long cvol, DevGrid g,
                             const cgfd_box_t *__restrict__ box,
                             const long long *__restrict__ off, int nbox,
                             long long total, float *__restrict__ out)
{
  long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (; t < total; t += stride) {
    int lo = 0, hi = nbox - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (off[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const cgfd_box_t b = box[lo];
    long long r = t - off[lo];
    const int a = (int)(r % b.ni); r /= b.ni;
    const int bj = (int)(r % b.nj); r /= b.nj;
    const int ck = (int)(r % b.nk);
    const int c = b.c1 + (int)(r / b.nk);
    const long long i = b.i1 + (long long)a * b.di + g.xoff;
    const long long j = b.j1 + (long long)bj * b.dj;
    const long long k = b.k1 + (long long)ck * b.dk;
    out[t] = w[c * cvol + i + j * g.px + k * g.sl];
  }
}

/* ------------------------------------------------------------------------ */
/* host-side source preprocessing                                            */
/* ------------------------------------------------------------------------ */

/* Gaussian weights normalised over the points at or below the surface
 * (forward/src_t.c:2111-2151 with fun_gauss src_t.c:2179-2184), evaluated
 * with the same float/double steps as the reference. */
static float gauss1(float t, float a)
{
  float tt = t - 0.0f;
  float e = (-tt) * tt / (a * a);
  float den = sqrtf((float)3.14159265358979323846) * a;
  return (float)(std::exp((double)e) / (double)den);
}

static void gauss_weights(std::vector<float> &delt, float x0, float y0,
                          float z0, float r, int half, int half_z2)
{
  int n1 = 2 * half + 1;
  delt.assign((size_t)n1 * n1 * n1, 0.f);
  int idx = 0;
  for (int k = -half; k <= half; k++)
    for (int j = -half; j <= half; j++)
      for (int i = -half; i <= half; i++)
        delt[idx++] = gauss1(i - x0, r) * gauss1(j - y0, r) * gauss1(k - z0, r);
  float sum = 0.f;
  idx = 0;
  for (int k = -half; k <= half_z2; k++)
    for (int j = -half; j <= half; j++)
      for (int i = -half; i <= half; i++) sum += delt[idx++];
  for (size_t m = 0; m < delt.size(); m++) delt[m] /= sum;
}

struct HostEntry {
  int col;
  SrcEntry e;
};

/* Source contributions per (i,j) column, sorted by k then source index. */
static int build_source_entries(const cgfd_problem_t *p, std::vector<int> &col,
                                std::vector<SrcEntry> &ent)
{
  size_t ln = p->nx, sl = (size_t)p->nx * p->ny;
  std::vector<HostEntry> all;
  for (int is = 0; is < p->src_n; is++) {
    int si = p->src_si[is], sj = p->src_sj[is], sk = p->src_sk[is];
    if (p->src_spatial == CGFD_SRC_POINT) {
      if (si < p->ni1 || si > p->ni2 || sj < p->nj1 || sj > p->nj2 ||
          sk < p->nk1 || sk > p->nk2)
        continue;
      size_t q = si + sj * ln + (size_t)sk * sl;
      HostEntry h;
      h.col = (si - p->ni1) + (sj - p->nj1) * p->ni;
      h.e.k = sk;
      h.e.is = is;
      h.e.coef = 1.0f;
      h.e.q = q;                   /* host index; vf, rjac on the device */
      h.e.vf = 0.f;
      h.e.rjac = 0.f;
      h.e.force_on = (p->src_surface_strict == 0 || sk < p->nk2);
      all.push_back(h);
    } else {
      int half = p->src_ext_half;
      int kz2 = (sk + half < p->nk2) ? half : p->nk2 - sk;
      std::vector<float> w;
      gauss_weights(w, p->src_si_inc[is], p->src_sj_inc[is],
                    p->src_sk_inc[is], p->src_ext_coef, half, kz2);
      int idx = 0;
      for (int kk = -half; kk <= kz2; kk++)
        for (int jj = -half; jj <= half; jj++)
          for (int ii = -half; ii <= half; ii++, idx++) {
            int i = si + ii, j = sj + jj, k = sk + kk;
            if (i < p->ni1 || i > p->ni2 || j < p->nj1 || j > p->nj2 ||
                k < p->nk1 || k > p->nk2)
              continue;
            size_t q = i + j * ln + (size_t)k * sl;
            float c = w[idx];
            HostEntry h;
            h.col = (i - p->ni1) + (j - p->nj1) * p->ni;
            h.e.k = k;
            h.e.is = is;
            h.e.coef = c;
            h.e.q = q;
            h.e.vf = 0.f;
            h.e.rjac = 0.f;
            h.e.force_on = (p->src_surface_strict == 0 || k < p->nk2);
            all.push_back(h);
          }
    }
  }
  /* stable ordering: column, then k, then source index (the reference adds
   * the sources in index order at every point) */
  std::stable_sort(all.begin(), all.end(), [](const HostEntry &a, const HostEntry &b) {
    if (a.col != b.col) return a.col < b.col;
    if (a.e.k != b.e.k) return a.e.k < b.e.k;
    return a.e.is < b.e.is;
  });
  size_t ncol = (size_t)p->ni * p->nj;
  col.assign(ncol + 1, 0);
  for (auto &h : all) col[h.col + 1]++;
  for (size_t c = 0; c < ncol; c++) col[c + 1] += col[c];
  ent.resize(all.size());
  for (size_t n = 0; n < all.size(); n++) ent[n] = all[n].e;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* solver                                                                    */
/* ------------------------------------------------------------------------ */

/* The enabled blocks of the exponential sponge and their point counts. */
struct AblexpBlocks {
  int n;
  int box[6][6];                /* ni1, ni2, nj1, nj2, nk1, nk2 */
  long long first[7];           /* prefix sums of the blocks' point counts */
};

/* Exponential sponge after a step (forward/bdry_t.c:841-890): the points of
 * the blocks times min(Ex[i], Ey[j], Ez[k]), every component. */
__global__ void k_ablexp(DevGrid g, float *w, int ncmp, AblexpBlocks B,
                         const float *__restrict__ Ex, const float *__restrict__ Ey,
                         const float *__restrict__ Ez)
{
  const long long total = B.first[B.n];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    int b = 0;
    while (b + 1 < B.n && t >= B.first[b + 1]) b++;
    const int *x = B.box[b];
    const int ni = x[1] - x[0] + 1, nj = x[3] - x[2] + 1;
    long long r = t - B.first[b];
    const int i = x[0] + (int)(r % ni);
    r /= ni;
    const int j = x[2] + (int)(r % nj);
    const int k = x[4] + (int)(r / nj);
    float mask = Ex[i] < Ey[j] ? Ex[i] : Ey[j];
    if (mask > Ez[k]) mask = Ez[k];
    const long long q = (long long)(i + g.xoff) + (long long)j * g.px + (long long)k * g.sl;
    for (int c = 0; c < ncmp; c++) w[c * g.vol + q] *= mask;
  }
}

/* Graves Q factors in place over a pitched volume holding Qs */
__global__ void k_qatt(float *v, long long n, float coef)
{
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    v[t] = expf(coef / v[t]);
}

/* One output slot: a set of boxes (slices, snapshots) packed on the device
 * and copied to pinned host memory behind the queued steps. */
struct OutSlot {
  std::vector<cgfd_box_t> boxes;
  cgfd_box_t *d_box, *h_box;    /* box table, device / pinned host */
  long long *d_off, *h_off;     /* each box's first packed index */
  int cap;
  float *d_pack, *h_pack;       /* packed floats, device / pinned host */
  size_t pack_cap, n;
  int *h_err;                   /* pinned copy of the device error flag */
  cudaEvent_t ev;
  int pending;
};

struct cgfd_solver {
  const cgfd_problem_t *p;
  DevGrid g;
  cudaStream_t stream;
  int med;                      /* MED_ISO / MED_VTI / MED_VIS / MED_ANI */
  int ncmp;                     /* wavefield components per level */
  int nmed;                     /* media components */
  float *wav;                   /* 4 levels x ncmp x vol */
  float *metric;                /* 10 x vol */
  float *media;                 /* nmed x vol (cgfd_media.cuh) */
  float *mats;                  /* 3 (4 for visco) x nx*ny*9 */
  float *aux[CGFD_NFACE];       /* 4 levels each */
  DevFace face[CGFD_NFACE];
  int face_src[CGFD_NFACE][2];  /* idim, iside */
  int *src_col, *src_it_begin, *src_it_end;
  SrcEntry *src_ent;
  float *stf;                   /* 9 tables */
  int nsf;                      /* surface force sources */
  SurfForce *sf;                /* their descriptors */
  float *sf_w;                  /* their surface-layer Gaussian weights */
  float *frate;                 /* 3 force-rate tables */
  float *surf;                  /* 6 x nx*ny: TxSrc..TzSrc, VxSrc..VzSrc */
  float *recv_dijk, *recv_seismo, *line_seismo;
  int *recv_idx, *line_iptr;
  int *d_it;
  int *d_flag;
  int step;
  int pre_lev, end_lev;         /* level of pre/end in wav (0 or 3) */
  int nsrc_ent;
  size_t bytes;
  size_t h2d_bytes, d2h_bytes;
  cudaEvent_t ev0, ev1;
  std::vector<cudaEvent_t> kev;   /* per-launch timing events */
  float t_stage_ms, t_other_ms, t_total_ms, t_pml_ms;
  int n_pml;
  int n_stage, n_other;
  int timing;
  cudaGraphExec_t graph8;
  int graph_pre_lev;
  int *d_err;
  int wait_limit;               /* stage-kernel wait polls (0: the default) */
  int test_skip_plane;          /* test hook of cgfd_solver_set_wait_test, -1 off */
  float *pg, *dis;              /* surface peak-motion maps (free top) */
  float *staging;               /* upload staging volume (set-up only) */
  OutSlot out[CGFD_OUT_SLOTS + 1];   /* output boxes; the last: blocking calls */
  float *qatt;                  /* Graves Q factors (pitched volume), or null */
  int *dd_col;                  /* dd sources: per-column entry offsets */
  SrcEntry *dd_ent;
  float *dd_tab;                /* dd_vi then dd_mij */
  float *abl;                   /* sponge masks Ex | Ey | Ez, or null */
  AblexpBlocks abx;             /* sponge blocks */
  StageMaps maps;               /* tensor maps of the stage kernel */
  int kernel;                   /* 2: TMA z-marching (default), 1: direct */
  int ty;                       /* tile rows of the medium's stage kernel */
  int pml_fused;                /* 1: CFS-PML inside the stage kernel */
  int l2_ahead;                 /* L2 prefetch distance of the stage kernel */
  int kchunk;
};

static size_t level_floats(const cgfd_solver_t *s) { return (size_t)s->ncmp * s->g.vol; }

static int medium_of(int medium_type)
{
  return medium_type == CGFD_MEDIUM_ELASTIC_ANISO ? MED_ANI
       : medium_type == CGFD_MEDIUM_ELASTIC_VTI ? MED_VTI
       : medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO ? MED_VIS : MED_ISO;
}

static int pitch_for(int ni) { return 32 * ((ni + 31) / 32 + 2); }
#define XOFF 29

extern "C" size_t cgfd_device_bytes(const cgfd_problem_t *p)
{
  size_t vol = (size_t)pitch_for(p->ni) * p->ny * p->nz;
  int med = medium_of(p->medium_type);
  int nmw = med == MED_VIS ? p->nmaxwell : 0;
  size_t b = (size_t)(4 * (9 + 6 * nmw) + 10 + med_ncomp(med, nmw) + (p->graves_qs ? 1 : 0)) *
             vol * sizeof(float);
  if (p->free_top) b += (med == MED_VIS ? 4 : 3) * (size_t)p->nx * p->ny * 9 * sizeof(float);
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      const cgfd_pml_face_t *f = &p->pml[d][s];
      if (!f->enabled) continue;
      size_t av = (size_t)(f->ni2 - f->ni1 + 1) * (f->nj2 - f->nj1 + 1) *
                  (f->nk2 - f->nk1 + 1);
      b += 4 * 9 * av * sizeof(float);
    }
  return b;
}

static int validate(const cgfd_problem_t *p)
{
  if (p->medium_type != CGFD_MEDIUM_ELASTIC_ISO &&
      p->medium_type != CGFD_MEDIUM_ELASTIC_VTI &&
      p->medium_type != CGFD_MEDIUM_ELASTIC_ANISO &&
      p->medium_type != CGFD_MEDIUM_VISCOELASTIC_ISO)
    return set_err(CGFD_EINVAL, "medium_type %d not supported (elastic_iso 2, "
                   "elastic_vti 3, elastic_aniso 4, viscoelastic_iso 5)", p->medium_type);
  if (p->medium_type == CGFD_MEDIUM_ELASTIC_ANISO) {
    const float *c[21] = {p->c11, p->c12, p->c13, p->c14, p->c15, p->c16, p->c22,
                          p->c23, p->c24, p->c25, p->c26, p->c33, p->c34, p->c35,
                          p->c36, p->c44, p->c45, p->c46, p->c55, p->c56, p->c66};
    for (int n = 0; n < 21; n++)
      if (!c[n]) return set_err(CGFD_EINVAL, "anisotropic medium: constant %d missing", n);
  }
  int ncmp_want = 9;
  if (p->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO) {
    if (p->nmaxwell < 1 || p->nmaxwell > CGFD_VIS_NMW_MAX)
      return set_err(CGFD_EINVAL, "nmaxwell=%d: the GPU visco-elastic path holds "
                     "1..%d Maxwell bodies", p->nmaxwell, CGFD_VIS_NMW_MAX);
    if (!p->wl || !p->lambda || !p->mu)
      return set_err(CGFD_EINVAL, "visco-elastic medium arrays missing");
    for (int n = 0; n < p->nmaxwell; n++)
      if (!p->Ylam[n] || !p->Ymu[n])
        return set_err(CGFD_EINVAL, "Ylam/Ymu[%d] missing", n);
    if (p->free_top && (!p->x3d || !p->y3d || !p->z3d))
      return set_err(CGFD_EINVAL, "visco-elastic free surface needs x3d/y3d/z3d");
    ncmp_want += 6 * p->nmaxwell;
  }
  if (p->medium_type == CGFD_MEDIUM_ELASTIC_VTI &&
      (!p->c11 || !p->c13 || !p->c33 || !p->c55 || !p->c66))
    return set_err(CGFD_EINVAL, "VTI medium arrays missing");
  if (p->ncmp != ncmp_want || p->nlevel != 4)
    return set_err(CGFD_EINVAL, "ncmp=%d nlevel=%d (need %d, 4)", p->ncmp,
                   p->nlevel, ncmp_want);
  if (p->nx != p->ni + 6 || p->ny != p->nj + 6 || p->nz != p->nk + 6 ||
      p->ni1 != 3 || p->nj1 != 3 || p->nk1 != 3 || p->ni2 != p->ni + 2 ||
      p->nj2 != p->nj + 2 || p->nk2 != p->nk + 2)
    return set_err(CGFD_EINVAL, "grid indices are not the 3-ghost layout");
  if (p->ni < 8 || p->nj < 8 || p->nk < 8)
    return set_err(CGFD_EINVAL, "grid too small (ni,nj,nk >= 8 required)");
  if (p->src_n > 0 && p->src_n_surface_force > 0) {
    if (!p->src_force || !p->src_force_rate_indx || !p->Fx_rate || !p->Fy_rate ||
        !p->Fz_rate)
      return set_err(CGFD_EINVAL, "surface force sources need the force and "
                     "force-rate tables");
    if (!p->free_top)
      return set_err(CGFD_EINVAL, "surface force sources need a free surface");
    for (int n = 0; n < p->src_n_surface_force; n++)
      if (p->src_force_rate_indx[n] < 0 || p->src_force_rate_indx[n] >= p->src_n)
        return set_err(CGFD_EINVAL, "surface force %d: bad source index", n);
  }
  if (!p->slw || !p->wav) return set_err(CGFD_EINVAL, "missing input array");
  if (p->jac) {
    const float *mh[10] = {p->jac, p->xi_x, p->xi_y, p->xi_z, p->eta_x,
                           p->eta_y, p->eta_z, p->zeta_x, p->zeta_y, p->zeta_z};
    for (int m = 0; m < 10; m++)
      if (!mh[m]) return set_err(CGFD_EINVAL, "metric array %d missing", m);
  } else if (!p->x3d || !p->y3d || !p->z3d) {
    return set_err(CGFD_EINVAL, "neither metrics nor grid coordinates given");
  }
  if (p->medium_type != CGFD_MEDIUM_ELASTIC_VTI &&
      p->medium_type != CGFD_MEDIUM_ELASTIC_ANISO && (!p->lambda || !p->mu))
    return set_err(CGFD_EINVAL, "missing lambda/mu");
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      const cgfd_pml_face_t *f = &p->pml[d][s];
      if (!f->enabled) continue;
      if (f->ni1 < p->ni1 || f->ni2 > p->ni2 || f->nj1 < p->nj1 ||
          f->nj2 > p->nj2 || f->nk1 < p->nk1 || f->nk2 > p->nk2 ||
          f->ni1 > f->ni2 || f->nj1 > f->nj2 || f->nk1 > f->nk2)
        return set_err(CGFD_EINVAL, "PML face %d/%d box outside the grid", d, s);
      if (!f->A || !f->B || !f->D || !f->aux)
        return set_err(CGFD_EINVAL, "PML face %d/%d arrays missing", d, s);
      /* a face box is the physical box cut down along its normal only
       * (forward/bdry_t.c:160-186); the stage kernel relies on it */
      int lo[3] = {f->ni1, f->nj1, f->nk1}, hi[3] = {f->ni2, f->nj2, f->nk2};
      int glo[3] = {p->ni1, p->nj1, p->nk1}, ghi[3] = {p->ni2, p->nj2, p->nk2};
      for (int e = 0; e < 3; e++) {
        if (e == d) {
          if ((s == 0 && lo[e] != glo[e]) || (s == 1 && hi[e] != ghi[e]))
            return set_err(CGFD_EINVAL, "PML face %d/%d does not start at its side", d, s);
        } else if (lo[e] != glo[e] || hi[e] != ghi[e]) {
          return set_err(CGFD_EINVAL, "PML face %d/%d does not span the grid across "
                         "its normal", d, s);
        }
      }
    }
  if (p->dd_n > 0) {
    if (!p->dd_si || !p->dd_sj || !p->dd_sk || p->dd_max_nt < 0 ||
        (!p->dd_vi && !p->dd_mij))
      return set_err(CGFD_EINVAL, "dd sources: indices or tables missing");
    for (int n = 0; n < p->dd_n; n++)
      if (p->dd_si[n] < p->ni1 || p->dd_si[n] > p->ni2 || p->dd_sj[n] < p->nj1 ||
          p->dd_sj[n] > p->nj2 || p->dd_sk[n] < p->nk1 || p->dd_sk[n] > p->nk2)
        return set_err(CGFD_EINVAL, "dd source %d outside the physical points", n);
  }
  if (p->graves_qs) {
    if (!p->Qs) return set_err(CGFD_EINVAL, "Graves Q: Qs missing");
    if (p->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO)
      return set_err(CGFD_EINVAL, "Graves Q and GMB attenuation are exclusive");
  }
  if (p->ablexp) {
    if (!p->ablexp_Ex || !p->ablexp_Ey || !p->ablexp_Ez)
      return set_err(CGFD_EINVAL, "sponge masks missing");
    for (int n = 0; n < 6; n++) {
      const int *b = p->ablexp_blk[n];
      if (b[0] != 1) continue;
      if (b[1] < 0 || b[2] >= p->nx || b[3] < 0 || b[4] >= p->ny || b[5] < 0 ||
          b[6] >= p->nz || b[2] < b[1] || b[4] < b[3] || b[6] < b[5])
        return set_err(CGFD_EINVAL, "sponge block %d outside the grid", n);
    }
  }
  if (p->recv_n > 0 && (!p->recv_dijk || !p->recv_indx1d || !p->recv_seismo))
    return set_err(CGFD_EINVAL, "receiver arrays missing");
  if (p->recv_n > 0 && p->recv_max_nt < p->nt_total)
    return set_err(CGFD_EINVAL, "receiver max_nt < nt_total");
  if (p->line_n > 0 && p->line_max_nt < p->nt_total)
    return set_err(CGFD_EINVAL, "line max_nt < nt_total");
  long long vol = (long long)p->nx * p->ny * p->nz;
  for (int n = 0; n < 8 * p->recv_n; n++)
    if (p->recv_indx1d[n] < 0 || p->recv_indx1d[n] >= vol)
      return set_err(CGFD_EINVAL, "receiver index out of the volume");
  if (p->line_n > 0 && (!p->line_iptr || !p->line_seismo))
    return set_err(CGFD_EINVAL, "line arrays missing");
  for (int n = 0; n < p->line_n; n++)
    if (p->line_iptr[n] < 0 || p->line_iptr[n] >= vol)
      return set_err(CGFD_EINVAL, "line receiver index out of the volume");
  if (p->src_n > 0) {
    if (!p->src_si || !p->src_sj || !p->src_sk || !p->src_it_begin ||
        !p->src_it_end || p->src_max_nt < 1 || p->src_max_stage != 4)
      return set_err(CGFD_EINVAL, "source description incomplete");
    if (p->src_spatial != CGFD_SRC_POINT &&
        (!p->src_si_inc || p->src_ext_half < 0 || p->src_ext_half > 8))
      return set_err(CGFD_EINVAL, "Gaussian source description incomplete");
    if ((p->src_force && (!p->Fx || !p->Fy || !p->Fz)) ||
        (p->src_moment && (!p->Mxx || !p->Myy || !p->Mzz || !p->Mxz ||
                           !p->Myz || !p->Mxy)))
      return set_err(CGFD_EINVAL, "source time-function tables missing");
    for (int is = 0; is < p->src_n; is++)
      if (p->src_it_end[is] - p->src_it_begin[is] + 1 > p->src_max_nt)
        return set_err(CGFD_EINVAL, "source %d time window exceeds max_nt", is);
  }
  return 0;
}

/* host index of the reference layout -> device (pitched) index */
static long long dev_index(const DevGrid &g, long long h)
{
  long long i = h % g.nx, j = (h / g.nx) % g.ny, k = h / ((long long)g.nx * g.ny);
  return (i + g.xoff) + j * g.px + k * g.sl;
}

static cudaError_t upload_volume(cgfd_solver_t *s, float *dst, const float *src);
static int make_tmap(cgfd_solver_t *s);

template <typename T>
static int dalloc(cgfd_solver_t *s, T **ptr, size_t n)
{
  *ptr = nullptr;
  if (n == 0) return 0;
  cudaError_t e = cudaMalloc((void **)ptr, n * sizeof(T));
  if (e != cudaSuccess)
    return set_err(CGFD_ENOMEM, "cudaMalloc(%zu bytes): %s", n * sizeof(T),
                   cudaGetErrorString(e));
  s->bytes += n * sizeof(T);
  return 0;
}

/* reference layout (nx*ny*nz, contiguous) -> pitched device layout */
__global__ void k_repitch(DevGrid g, const float *__restrict__ src, float *dst)
{
  const int rows = g.ny * g.nz;                 /* row r = j + k*ny */
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const float *a = src + (long long)r * g.nx;
    float *b = dst + g.xoff + (long long)r * g.px;
    for (int i = threadIdx.x; i < g.nx; i += blockDim.x) b[i] = a[i];
  }
}

/* One host volume into the pitched device layout: a contiguous copy into a
 * device staging buffer, then a re-pitch kernel (a strided host-to-device
 * copy with rows of nx floats measured ~35 GB/s on GB300; the contiguous
 * copy runs at the link's rate).  The staging buffer lives until
 * release_staging(). */
static cudaError_t upload_volume(cgfd_solver_t *s, float *dst, const float *src)
{
  const DevGrid &g = s->g;
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  s->h2d_bytes += n * sizeof(float);
  if (!s->staging) {
    cudaError_t e = cudaMalloc((void **)&s->staging, n * sizeof(float));
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = cudaMemcpyAsync(s->staging, src, n * sizeof(float),
                                  cudaMemcpyHostToDevice, s->stream);
  if (e != cudaSuccess) return e;
  k_repitch<<<152 * 8, 256, 0, s->stream>>>(g, s->staging, dst);
  return cudaGetLastError();
}

/* metrics (10 volumes, device layout) from host grid coordinates */
static int device_metrics(cgfd_solver_t *s, const float *x3d, const float *y3d,
                          const float *z3d, float *metric)
{
  const DevGrid &g = s->g;
  float *xyz = nullptr;
  CK(cudaMalloc((void **)&xyz, 3 * (size_t)g.vol * sizeof(float)));
  cudaError_t e = cudaMemsetAsync(xyz, 0, 3 * (size_t)g.vol * sizeof(float), s->stream);
  const float *src[3] = {x3d, y3d, z3d};
  for (int c = 0; c < 3 && e == cudaSuccess; c++)
    e = upload_volume(s, xyz + c * g.vol, src[c]);
  if (e == cudaSuccess) {
    dim3 b(32, 8), gr((g.ni + 31) / 32, (g.nj + 7) / 8, g.nk);
    k_metric<<<gr, b, 0, s->stream>>>(g, xyz, xyz + g.vol, xyz + 2 * g.vol, metric);
    k_metric_ghost<<<152 * 8, 256, 0, s->stream>>>(g, metric);
    e = cudaGetLastError();
  }
  cudaError_t e2 = cudaStreamSynchronize(s->stream);
  cudaFree(xyz);
  CK(e);
  CK(e2);
  return 0;
}

static void release_staging(cgfd_solver_t *s)
{
  if (s->staging) {
    cudaStreamSynchronize(s->stream);
    cudaFree(s->staging);
    s->staging = nullptr;
  }
}

static cudaError_t download_volume(cgfd_solver_t *s, float *dst, const float *src)
{
  const DevGrid &g = s->g;
  s->d2h_bytes += (size_t)g.nx * g.ny * g.nz * sizeof(float);
  return cudaMemcpy2DAsync(dst, (size_t)g.nx * sizeof(float), src + g.xoff,
                           (size_t)g.px * sizeof(float), (size_t)g.nx * sizeof(float),
                           (size_t)g.ny * g.nz, cudaMemcpyDeviceToHost, s->stream);
}

typedef CUresult (*encode_tiled_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t,
                                    void *, const cuuint64_t *, const cuuint64_t *,
                                    const cuuint32_t *, const cuuint32_t *,
                                    CUtensorMapInterleave, CUtensorMapSwizzle,
                                    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

/* 5-D tensor map (x, y, z, component, level) over the wavefield block */
static int make_tmap(cgfd_solver_t *s)
{
  static encode_tiled_fn fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void *ptr = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr,
                                                     12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !ptr)
      return set_err(CGFD_ECUDA, "cuTensorMapEncodeTiled unavailable");
    fn = (encode_tiled_fn)ptr;
  }
  const DevGrid &g = s->g;
  StageMaps &M = s->maps;
  /* components 0..8 of every level; the level stride spans all ncmp */
  cuuint64_t dims[5] = {(cuuint64_t)g.px, (cuuint64_t)g.ny, (cuuint64_t)g.nz, 9, 4};
  cuuint64_t strides[4] = {(cuuint64_t)g.px * 4, (cuuint64_t)g.sl * 4,
                           (cuuint64_t)g.vol * 4, (cuuint64_t)g.vol * s->ncmp * 4};
  cuuint32_t box[5] = {s2::BW, (cuuint32_t)(s->ty + 4), 1, 9, 1};
  cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(&M.wav, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, s->wav, dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(CGFD_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  /* per-point tiles (no halo) for L2 prefetch of the streams */
  cuuint32_t boxp[5] = {s2::TX, (cuuint32_t)s->ty, 1, 9, 1};
  r = fn(&M.pt, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, s->wav, dims, strides,
         boxp, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(CGFD_ECUDA, "tensor map (points) failed (%d)", (int)r);
  cuuint64_t dm[4] = {(cuuint64_t)g.px, (cuuint64_t)g.ny, (cuuint64_t)g.nz, 10};
  cuuint64_t sm_[3] = {(cuuint64_t)g.px * 4, (cuuint64_t)g.sl * 4, (cuuint64_t)g.vol * 4};
  cuuint32_t bm[4] = {s2::TX, (cuuint32_t)s->ty, 1, 9};   /* xi_x..zeta_z */
  r = fn(&M.met, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, s->metric, dm, sm_, bm, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(CGFD_ECUDA, "tensor map (metrics) failed (%d)", (int)r);
  dm[3] = (cuuint64_t)s->nmed;
  bm[3] = (cuuint32_t)s->nmed;
  r = fn(&M.med, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, s->media, dm, sm_, bm, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(CGFD_ECUDA, "tensor map (media) failed (%d)", (int)r);
  /* memory variables (components 9 .. ncmp-1) of the visco-elastic medium */
  M.j = M.pt;
  if (s->ncmp > 9) {
    cuuint64_t dj[5] = {(cuuint64_t)g.px, (cuuint64_t)g.ny, (cuuint64_t)g.nz,
                        (cuuint64_t)s->ncmp, 4};
    cuuint32_t bj[5] = {s2::TX, (cuuint32_t)s->ty, 1, (cuuint32_t)(s->ncmp - 9), 1};
    r = fn(&M.j, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, s->wav, dj, strides, bj, estr,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
      return set_err(CGFD_ECUDA, "tensor map (memory variables) failed (%d)", (int)r);
  }
  return 0;
}

extern "C" void cgfd_solver_destroy(cgfd_solver_t *s)
{
  if (!s) return;
  if (s->graph8) cudaGraphExecDestroy(s->graph8);
  void *ptrs[] = {s->wav, s->metric, s->media, s->mats, s->src_col,
                  s->src_it_begin, s->src_it_end, s->src_ent, s->stf,
                  s->recv_dijk, s->recv_seismo, s->line_seismo, s->recv_idx,
                  s->line_iptr, s->d_it, s->d_flag, s->d_err, s->pg, s->dis,
                  s->sf, s->sf_w, s->frate, s->surf, s->staging, s->qatt, s->abl,
                  s->dd_col, s->dd_ent, s->dd_tab};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  for (OutSlot &o : s->out) {
    if (o.d_box) cudaFree(o.d_box);
    if (o.d_off) cudaFree(o.d_off);
    if (o.h_box) cudaFreeHost(o.h_box);
    if (o.h_off) cudaFreeHost(o.h_off);
    if (o.d_pack) cudaFree(o.d_pack);
    if (o.h_pack) cudaFreeHost(o.h_pack);
    if (o.h_err) cudaFreeHost(o.h_err);
    if (o.ev) cudaEventDestroy(o.ev);
  }
  for (int f = 0; f < CGFD_NFACE; f++)
    if (s->aux[f]) cudaFree(s->aux[f]);
  for (int f = 0; f < CGFD_NFACE; f++) {
    if (s->face[f].A) cudaFree((void *)s->face[f].A);
  }
  for (cudaEvent_t e : s->kev) cudaEventDestroy(e);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

extern "C" int cgfd_solver_create(const cgfd_problem_t *p, cgfd_solver_t **out)
{
  *out = nullptr;
  int rc = validate(p);
  if (rc) return rc;
  cgfd_solver_t *s = new cgfd_solver_t();
  s->p = p;
  s->med = medium_of(p->medium_type);
  s->ncmp = p->ncmp;
  s->nmed = med_ncomp(s->med, s->med == MED_VIS ? p->nmaxwell : 0);
  s->ty = s->med == MED_VTI ? cgfd_stage_rows_vti()
        : s->med == MED_VIS ? cgfd_stage_rows_vis()
        : s->med == MED_ANI ? cgfd_stage_rows_ani() : cgfd_stage_rows_iso();
  DevGrid &g = s->g;
  g.ni = p->ni; g.nj = p->nj; g.nk = p->nk;
  g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
  g.ni1 = p->ni1; g.ni2 = p->ni2; g.nj1 = p->nj1; g.nj2 = p->nj2;
  g.nk1 = p->nk1; g.nk2 = p->nk2;
  g.xoff = XOFF;
  g.px = pitch_for(p->ni);
  g.sl = (long long)g.px * p->ny;
  g.vol = g.sl * p->nz;
#define TRY(x) do { int r_ = (x); if (r_) { cgfd_solver_destroy(s); return r_; } } while (0)
#define TRYC(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { set_err(CGFD_ECUDA, "%s: %s", #x, cudaGetErrorString(e_)); cgfd_solver_destroy(s); return CGFD_ECUDA; } } while (0)
  TRYC(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  TRYC(cudaEventCreate(&s->ev0));
  TRYC(cudaEventCreate(&s->ev1));
  size_t vol = g.vol, L = level_floats(s);
  size_t hvol = (size_t)p->nx * p->ny * p->nz;
  cudaStream_t st = s->stream;
  /* wavefield: level 0 of the input copied into all four levels, so that
   * ghost values stay what the caller passed (they never change in the
   * reference either: rhs ghosts are zero) */
  SetupTrace tr;
  tr.start(st);
  TRY(dalloc(s, &s->wav, 4 * L));
  tr.mark("allocate wavefield");
  TRYC(cudaMemsetAsync(s->wav, 0, L * sizeof(float), st));
  for (int c = 0; c < s->ncmp; c++)
    TRYC(upload_volume(s, s->wav + c * vol, p->wav + (size_t)c * hvol));
  for (int l = 1; l < 4; l++)
    TRYC(cudaMemcpyAsync(s->wav + l * L, s->wav, L * sizeof(float),
                         cudaMemcpyDeviceToDevice, st));

  s->pre_lev = 0;
  s->end_lev = 3;
  tr.mark("upload wavefield");
  TRY(dalloc(s, &s->metric, 10 * vol));
  TRYC(cudaMemsetAsync(s->metric, 0, 10 * vol * sizeof(float), st));
  if (p->jac) {
    const float *mh[10] = {p->jac, p->xi_x, p->xi_y, p->xi_z, p->eta_x,
                           p->eta_y, p->eta_z, p->zeta_x, p->zeta_y, p->zeta_z};
    for (int m = 0; m < 10; m++)
      TRYC(upload_volume(s, s->metric + m * vol, mh[m]));
  } else {
    /* no metrics given: computed here from the grid coordinates */
    TRY(device_metrics(s, p->x3d, p->y3d, p->z3d, s->metric));
  }
  tr.mark("metrics");
  TRY(dalloc(s, &s->media, (size_t)s->nmed * vol));
  TRYC(cudaMemsetAsync(s->media, 0, (size_t)s->nmed * vol * sizeof(float), st));
  {
    const float *md[22 + 2 * CGFD_VIS_NMW_MAX];
    int nm = 0;
    md[nm++] = p->slw;
    if (s->med == MED_ANI) {
      const float *c[21] = {p->c11, p->c12, p->c13, p->c14, p->c15, p->c16, p->c22,
                            p->c23, p->c24, p->c25, p->c26, p->c33, p->c34, p->c35,
                            p->c36, p->c44, p->c45, p->c46, p->c55, p->c56, p->c66};
      for (int n = 0; n < 21; n++) md[nm++] = c[n];
    } else if (s->med == MED_VTI) {
      md[nm++] = p->c11; md[nm++] = p->c13; md[nm++] = p->c33;
      md[nm++] = p->c55; md[nm++] = p->c66;
    } else {
      md[nm++] = p->lambda; md[nm++] = p->mu;
      if (s->med == MED_VIS) {
        for (int n = 0; n < p->nmaxwell; n++) md[nm++] = p->Ylam[n];
        for (int n = 0; n < p->nmaxwell; n++) md[nm++] = p->Ymu[n];
      }
    }
    for (int m = 0; m < nm; m++)
      TRYC(upload_volume(s, s->media + m * vol, md[m]));
  }
  if (p->graves_qs) {
    /* Graves Q factors, forward/sv_curv_col_el.c:642 and :656:
     * coef = -PI * freq * dt evaluated in double, stored as float */
    TRY(dalloc(s, &s->qatt, vol));
    TRYC(cudaMemsetAsync(s->qatt, 0, vol * sizeof(float), st));
    TRYC(upload_volume(s, s->qatt, p->Qs));
    const float coef = (float)(-3.14159265358979323846 * (double)p->qs_freq * (double)p->dt);
    k_qatt<<<152 * 8, 256, 0, st>>>(s->qatt, (long long)vol, coef);
    TRYC(cudaGetLastError());
  }
  if (p->ablexp) {
    TRY(dalloc(s, &s->abl, (size_t)p->nx + p->ny + p->nz));
    TRYC(cudaMemcpyAsync(s->abl, p->ablexp_Ex, p->nx * sizeof(float), cudaMemcpyHostToDevice, st));
    TRYC(cudaMemcpyAsync(s->abl + p->nx, p->ablexp_Ey, p->ny * sizeof(float),
                         cudaMemcpyHostToDevice, st));
    TRYC(cudaMemcpyAsync(s->abl + p->nx + p->ny, p->ablexp_Ez, p->nz * sizeof(float),
                         cudaMemcpyHostToDevice, st));
    s->abx.n = 0;
    s->abx.first[0] = 0;
    for (int n = 0; n < 6; n++) {
      const int *b = p->ablexp_blk[n];
      if (b[0] != 1) continue;
      int *x = s->abx.box[s->abx.n];
      for (int e = 0; e < 6; e++) x[e] = b[1 + e];
      s->abx.first[s->abx.n + 1] = s->abx.first[s->abx.n] +
          (long long)(x[1] - x[0] + 1) * (x[3] - x[2] + 1) * (x[5] - x[4] + 1);
      s->abx.n++;
    }
    if (s->abx.n == 0) {      /* no enabled block: nothing to apply */
      cudaFree(s->abl);
      s->abl = nullptr;
    }
  }
  tr.mark("media");
  /* PML faces */
  int nf = 0;
  for (int d = 0; d < 3; d++)
    for (int sd = 0; sd < 2; sd++) {
      const cgfd_pml_face_t *f = &p->pml[d][sd];
      int fi = d * 2 + sd;
      DevFace &F = s->face[fi];
      F.on = f->enabled ? 1 : 0;
      F.dim = d;
      if (!F.on) continue;
      nf++;
      F.i1 = f->ni1; F.i2 = f->ni2; F.j1 = f->nj1; F.j2 = f->nj2;
      F.k1 = f->nk1; F.k2 = f->nk2;
      F.bx = f->ni2 - f->ni1 + 1;
      F.by = f->nj2 - f->nj1 + 1;
      F.avol = (long long)F.bx * F.by * (f->nk2 - f->nk1 + 1);
      int np = d == 0 ? F.bx : (d == 1 ? F.by : f->nk2 - f->nk1 + 1);
      float *coef;
      TRYC(cudaMalloc((void **)&coef, 3 * np * sizeof(float)));
      s->bytes += 3 * np * sizeof(float);
      TRYC(cudaMemcpyAsync(coef, f->A, np * 4, cudaMemcpyHostToDevice, st));
      TRYC(cudaMemcpyAsync(coef + np, f->B, np * 4, cudaMemcpyHostToDevice, st));
      TRYC(cudaMemcpyAsync(coef + 2 * np, f->D, np * 4, cudaMemcpyHostToDevice, st));
      F.A = coef; F.B = coef + np; F.D = coef + 2 * np;
      /* device: the 9 components the PML updates; the host layout holds
       * ncmp per level (forward/bdry_t.c:300-306), its memory-variable
       * components never change */
      size_t al = 9 * (size_t)F.avol;
      TRY(dalloc(s, &s->aux[fi], 4 * al));
      TRYC(cudaMemcpyAsync(s->aux[fi], f->aux, al * sizeof(float),
                           cudaMemcpyHostToDevice, st));
      for (int l = 1; l < 4; l++)
        TRYC(cudaMemcpyAsync(s->aux[fi] + l * al, s->aux[fi], al * sizeof(float),
                             cudaMemcpyDeviceToDevice, st));
      s->h2d_bytes += al * sizeof(float) + 3 * np * sizeof(float);
    }
  (void)nf;
  tr.mark("PML faces");
  /* free surface matrices, computed on the device */
  if (p->free_top) {
    size_t n2 = (size_t)g.nx * g.ny * 9;
    int nmat = s->med == MED_VIS ? 4 : 3;
    TRY(dalloc(s, &s->mats, nmat * n2));
    TRYC(cudaMemsetAsync(s->mats, 0, nmat * n2 * sizeof(float), st));
    dim3 b(32, 8), gr((g.ni + 31) / 32, (g.nj + 7) / 8);
    const float *M = s->metric;
    if (s->med == MED_ISO) {
      k_dvh2dvz_iso<<<gr, b, 0, st>>>(g, M + vol, M + 2 * vol, M + 3 * vol,
                                      M + 4 * vol, M + 5 * vol, M + 6 * vol,
                                      M + 7 * vol, M + 8 * vol, M + 9 * vol,
                                      s->media + vol, s->media + 2 * vol,
                                      s->mats, s->mats + n2, s->mats + 2 * n2);
    } else if (s->med == MED_VTI) {
      k_dvh2dvz_vti<<<gr, b, 0, st>>>(g, M, s->media, s->mats, s->mats + n2);
    } else if (s->med == MED_ANI) {
      k_dvh2dvz_ani<<<gr, b, 0, st>>>(g, M, s->media, s->mats, s->mats + n2);
    } else {
      /* the surface plane of the grid coordinates (rows j-3..j+3 are read) */
      size_t s2n = (size_t)g.nx * g.ny;
      size_t off = (size_t)p->nk2 * s2n;
      float *xyz = nullptr;
      TRYC(cudaMalloc((void **)&xyz, 3 * s2n * sizeof(float)));
      cudaError_t e1 = cudaMemcpyAsync(xyz, p->x3d + off, s2n * 4, cudaMemcpyHostToDevice, st);
      cudaError_t e2 = cudaMemcpyAsync(xyz + s2n, p->y3d + off, s2n * 4, cudaMemcpyHostToDevice, st);
      cudaError_t e3 = cudaMemcpyAsync(xyz + 2 * s2n, p->z3d + off, s2n * 4, cudaMemcpyHostToDevice, st);
      if (e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess)
        k_dvh2dvz_vis<<<gr, b, 0, st>>>(g, M, s->media, xyz, xyz + s2n, xyz + 2 * s2n,
                                        s->mats, s->mats + n2, s->mats + 3 * n2);
      cudaError_t e4 = cudaStreamSynchronize(st);
      cudaFree(xyz);
      s->h2d_bytes += 3 * s2n * 4;
      TRYC(e1); TRYC(e2); TRYC(e3); TRYC(e4);
    }
    TRYC(cudaGetLastError());
  }
  tr.mark("surface matrices");
  /* sources */
  if (p->src_n > 0) {
    std::vector<int> col;
    std::vector<SrcEntry> ent;
    build_source_entries(p, col, ent);
    for (SrcEntry &e : ent) e.q = dev_index(g, e.q);
    s->nsrc_ent = (int)ent.size();
    TRY(dalloc(s, &s->src_col, col.size()));
    TRYC(cudaMemcpyAsync(s->src_col, col.data(), col.size() * 4, cudaMemcpyHostToDevice, st));
    TRY(dalloc(s, &s->src_ent, ent.size() > 0 ? ent.size() : 1));
    if (!ent.empty())
      TRYC(cudaMemcpyAsync(s->src_ent, ent.data(), ent.size() * sizeof(SrcEntry),
                           cudaMemcpyHostToDevice, st));
    if (!ent.empty()) {
      /* weights coef*slw/jac and coef/jac from the device media and metrics */
      k_src_weights<<<(unsigned)((ent.size() + 127) / 128), 128, 0, st>>>(
          g, s->src_ent, (int)ent.size(), s->media, s->metric);
      TRYC(cudaGetLastError());
    }
    TRY(dalloc(s, &s->src_it_begin, p->src_n));
    TRY(dalloc(s, &s->src_it_end, p->src_n));
    TRYC(cudaMemcpyAsync(s->src_it_begin, p->src_it_begin, p->src_n * 4, cudaMemcpyHostToDevice, st));
    TRYC(cudaMemcpyAsync(s->src_it_end, p->src_it_end, p->src_n * 4, cudaMemcpyHostToDevice, st));
    size_t nstf = (size_t)p->src_n * p->src_max_nt * p->src_max_stage;
    TRY(dalloc(s, &s->stf, 9 * nstf));
    TRYC(cudaMemsetAsync(s->stf, 0, 9 * nstf * sizeof(float), st));
    const float *tabs[9] = {p->Fx, p->Fy, p->Fz, p->Mxx, p->Myy, p->Mzz, p->Mxz, p->Myz, p->Mxy};
    int use[9] = {p->src_force, p->src_force, p->src_force, p->src_moment, p->src_moment,
                  p->src_moment, p->src_moment, p->src_moment, p->src_moment};
    for (int t = 0; t < 9; t++)
      if (use[t] && tabs[t])
        TRYC(cudaMemcpyAsync(s->stf + t * nstf, tabs[t], nstf * 4, cudaMemcpyHostToDevice, st));
    if (p->src_n_surface_force > 0) {
      /* surface forces: descriptors, surface-layer weights, rate tables */
      int nsf = p->src_n_surface_force;
      std::vector<SurfForce> sfv(nsf);
      std::vector<float> wv;
      for (int n = 0; n < nsf; n++) {
        int is = p->src_force_rate_indx[n];
        SurfForce &f = sfv[n];
        f.is = is; f.n = n;
        f.si = p->src_si[is]; f.sj = p->src_sj[is]; f.sk = p->src_sk[is];
        f.half = p->src_spatial == CGFD_SRC_POINT ? 0 : p->src_ext_half;
        f.w0 = (int)wv.size();
        f.pad = 0;
        if (f.half > 0) {
          int half = f.half, len = 2 * half + 1;
          int kx = p->nk2 - f.sk;
          std::vector<float> w3;
          gauss_weights(w3, p->src_si_inc[is], p->src_sj_inc[is], p->src_sk_inc[is],
                        p->src_ext_coef, half, kx);
          size_t off = (size_t)(kx + half) * len * len;
          if (kx < -half || kx > half) {
            set_err(CGFD_EINVAL, "surface force %d does not reach the surface", n);
            cgfd_solver_destroy(s);
            return CGFD_EINVAL;
          }
          wv.insert(wv.end(), w3.begin() + off, w3.begin() + off + len * len);
        }
      }
      s->nsf = nsf;
      TRY(dalloc(s, &s->sf, nsf));
      TRYC(cudaMemcpyAsync(s->sf, sfv.data(), nsf * sizeof(SurfForce), cudaMemcpyHostToDevice, st));
      TRY(dalloc(s, &s->sf_w, wv.empty() ? 1 : wv.size()));
      if (!wv.empty())
        TRYC(cudaMemcpyAsync(s->sf_w, wv.data(), wv.size() * 4, cudaMemcpyHostToDevice, st));
      size_t nr = (size_t)nsf * p->src_max_nt * p->src_max_stage;
      TRY(dalloc(s, &s->frate, 3 * nr));
      const float *rt[3] = {p->Fx_rate, p->Fy_rate, p->Fz_rate};
      for (int m = 0; m < 3; m++)
        TRYC(cudaMemcpyAsync(s->frate + m * nr, rt[m], nr * 4, cudaMemcpyHostToDevice, st));
      TRY(dalloc(s, &s->surf, 6 * (size_t)g.nx * g.ny));
      TRYC(cudaMemsetAsync(s->surf, 0, 6 * (size_t)g.nx * g.ny * sizeof(float), st));
      cudaStreamSynchronize(st);       /* host vectors go out of scope */
    }
  }
  if (p->dd_n > 0) {
    /* distributed sources: point entries per column, sorted by k then point
     * (added in point order, as sv_curv_col_el_rhs_srcdd loops them) */
    size_t ln = p->nx, sl = (size_t)p->nx * p->ny;
    std::vector<HostEntry> all(p->dd_n);
    for (int n = 0; n < p->dd_n; n++) {
      HostEntry &h = all[n];
      h.col = (p->dd_si[n] - p->ni1) + (p->dd_sj[n] - p->nj1) * p->ni;
      h.e.k = p->dd_sk[n];
      h.e.is = n;
      h.e.coef = 1.0f;
      h.e.q = dev_index(g, p->dd_si[n] + p->dd_sj[n] * ln + (size_t)p->dd_sk[n] * sl);
      h.e.vf = h.e.rjac = 0.f;
      h.e.force_on = 1;
    }
    std::stable_sort(all.begin(), all.end(), [](const HostEntry &x, const HostEntry &y) {
      if (x.col != y.col) return x.col < y.col;
      if (x.e.k != y.e.k) return x.e.k < y.e.k;
      return x.e.is < y.e.is;
    });
    std::vector<int> col((size_t)p->ni * p->nj + 1, 0);
    std::vector<SrcEntry> ent;
    for (auto &h : all) { col[h.col + 1]++; ent.push_back(h.e); }
    for (size_t c = 1; c < col.size(); c++) col[c] += col[c - 1];
    TRY(dalloc(s, &s->dd_col, col.size()));
    TRY(dalloc(s, &s->dd_ent, ent.size()));
    TRYC(cudaMemcpyAsync(s->dd_col, col.data(), col.size() * 4, cudaMemcpyHostToDevice, st));
    TRYC(cudaMemcpyAsync(s->dd_ent, ent.data(), ent.size() * sizeof(SrcEntry),
                         cudaMemcpyHostToDevice, st));
    k_src_weights<<<(unsigned)((ent.size() + 127) / 128), 128, 0, st>>>(
        g, s->dd_ent, (int)ent.size(), s->media, s->metric);
    TRYC(cudaGetLastError());
    size_t nt = (size_t)p->dd_max_nt * 4 * p->dd_n;
    TRY(dalloc(s, &s->dd_tab, 9 * nt + 1));
    if (p->dd_vi && nt)
      TRYC(cudaMemcpyAsync(s->dd_tab, p->dd_vi, 3 * nt * 4, cudaMemcpyHostToDevice, st));
    if (p->dd_mij && nt)
      TRYC(cudaMemcpyAsync(s->dd_tab + 3 * nt, p->dd_mij, 6 * nt * 4, cudaMemcpyHostToDevice,
                           st));
    s->h2d_bytes += 9 * nt * 4;
  }
  tr.mark("sources");
  /* receivers and lines */
  if (p->recv_n > 0) {
    TRY(dalloc(s, &s->recv_dijk, 3 * (size_t)p->recv_n));
    TRY(dalloc(s, &s->recv_idx, 8 * (size_t)p->recv_n));
    size_t ns = (size_t)p->recv_n * p->recv_ncmp * p->recv_max_nt;
    TRY(dalloc(s, &s->recv_seismo, ns));
    TRYC(cudaMemcpyAsync(s->recv_dijk, p->recv_dijk, 3 * p->recv_n * 4, cudaMemcpyHostToDevice, st));
    std::vector<int> di(8 * (size_t)p->recv_n);
    for (size_t n = 0; n < di.size(); n++) di[n] = (int)dev_index(g, p->recv_indx1d[n]);
    TRYC(cudaMemcpy(s->recv_idx, di.data(), di.size() * 4, cudaMemcpyHostToDevice));
    TRYC(cudaMemsetAsync(s->recv_seismo, 0, ns * 4, st));
  }
  if (p->line_n > 0) {
    TRY(dalloc(s, &s->line_iptr, p->line_n));
    size_t ns = (size_t)p->line_n * p->ncmp * p->line_max_nt;
    TRY(dalloc(s, &s->line_seismo, ns));
    std::vector<int> di(p->line_n);
    for (int n = 0; n < p->line_n; n++) di[n] = (int)dev_index(g, p->line_iptr[n]);
    TRYC(cudaMemcpy(s->line_iptr, di.data(), di.size() * 4, cudaMemcpyHostToDevice));
    TRYC(cudaMemsetAsync(s->line_seismo, 0, ns * 4, st));
  }
  if (p->free_top) {
    size_t s2 = (size_t)p->nx * p->ny;
    TRY(dalloc(s, &s->pg, 15 * s2));
    TRY(dalloc(s, &s->dis, 3 * s2));
    TRYC(cudaMemsetAsync(s->pg, 0, 15 * s2 * 4, st));
    TRYC(cudaMemsetAsync(s->dis, 0, 3 * s2 * 4, st));
  }
  TRY(dalloc(s, &s->d_it, 1));
  TRYC(cudaMemsetAsync(s->d_it, 0, 4, st));
  TRY(dalloc(s, &s->d_flag, 1));
  TRY(dalloc(s, &s->d_err, 1));
  TRYC(cudaMemsetAsync(s->d_err, 0, 4, st));
  s->kernel = 2;
  /* the direct-load A/B kernel (cgfd_stage.cuh) covers isotropic media only */
  if (const char *e = getenv("CGFD_STAGE_KERNEL"))
    s->kernel = (atoi(e) == 1 && s->med == MED_ISO && s->nsf == 0) ? 1 : 2;
  /* CFS-PML inside the stage kernel (default: measured faster on GB300 for
   * every medium, the face kernels re-read the wavefield, metrics and media
   * and read-modify-write tmp/end) or by the per-face kernels after it.
   * CGFD_PML_SPLIT=1 / 0 forces either form. */
  s->pml_fused = 1;
  if (const char *e = getenv("CGFD_PML_SPLIT")) s->pml_fused = atoi(e) == 1 ? 0 : 1;
  /* planes the producer prefetches into L2 beyond its rings (CGFD_L2_AHEAD):
   * measured on GB300, one plane gains ~1 % for isotropic/VTI media, any
   * prefetch loses for the visco-elastic kernel (8-row tiles, larger slots) */
  s->l2_ahead = s->med == MED_VIS ? 0 : 1;
  s->wait_limit = 0;
  s->test_skip_plane = -1;
  if (const char *e = getenv("CGFD_L2_AHEAD")) s->l2_ahead = std::max(0, std::min(8, atoi(e)));
  {
    /* k planes per CTA: chunks of at most 20 planes, split evenly (measured
     * on GB300: 400x400x200 iso 16-30 planes within 1 %, 67 planes 11 %
     * slower; 300x300x150 VTI and visco best at 16-20 -- short chunks
     * spread the PML planes of the bottom face over many CTAs and leave a
     * short tail), more chunks when the grid has few tiles, so that there
     * are at least ~8 waves of CTAs */
    int tiles = ((g.ni + s2::TX - 1) / s2::TX) * ((g.nj + s->ty - 1) / s->ty);
    int nch = std::max(1, (g.nk + 19) / 20);
    while (tiles * nch < 8 * 152 && (g.nk + nch) / (nch + 1) >= 8) nch++;
    s->kchunk = (g.nk + nch - 1) / nch;
    if (const char *e = getenv("CGFD_KCHUNK")) s->kchunk = std::max(4, atoi(e));
  }
  tr.mark("receivers, counters");
  TRY(make_tmap(s));
  TRYC(cudaStreamSynchronize(st));
  release_staging(s);
  tr.mark("tensor maps");
  *out = s;
  return 0;
#undef TRY
#undef TRYC
}

/* level roles of the four device levels for one stage */
static void stage_levels(cgfd_solver_t *s, int istage, float **cur, float **pre,
                         float **tmp_out, float **end)
{
  size_t L = level_floats(s);
  float *base = s->wav;
  int tA = 1, tB = 2;
  *pre = base + s->pre_lev * L;
  *end = base + s->end_lev * L;
  if (istage == 0) { *cur = *pre; *tmp_out = base + tA * L; }
  else if (istage == 1) { *cur = base + tA * L; *tmp_out = base + tB * L; }
  else if (istage == 2) { *cur = base + tB * L; *tmp_out = base + tA * L; }
  else { *cur = base + tA * L; *tmp_out = nullptr; }
}

/* direct-load A/B kernel (isotropic media only) */
template <int BX, int BY, int BZ>
static void launch_v1(cgfd_solver_t *s, int kind, cudaStream_t st, const StageArgs &a)
{
  dim3 b(V1_TX, V1_TY);
  dim3 gr((s->g.ni + V1_TX - 1) / V1_TX, (s->g.nj + V1_TY - 1) / V1_TY,
          (s->g.nk + V1_KCHUNK - 1) / V1_KCHUNK);
  if (kind == 0) k_stage<BX, BY, BZ, 0><<<gr, b, 0, st>>>(a);
  else if (kind == 1) k_stage<BX, BY, BZ, 1><<<gr, b, 0, st>>>(a);
  else k_stage<BX, BY, BZ, 2><<<gr, b, 0, st>>>(a);
}

static void launch_stage(cgfd_solver_t *s, int code, int kind, cudaStream_t st,
                         const StageArgs &a)
{
  if (s->kernel == 1) {
    switch (code) {
      case 0: launch_v1<0, 0, 0>(s, kind, st, a); break;
      case 1: launch_v1<0, 0, 1>(s, kind, st, a); break;
      case 2: launch_v1<0, 1, 0>(s, kind, st, a); break;
      case 3: launch_v1<0, 1, 1>(s, kind, st, a); break;
      case 4: launch_v1<1, 0, 0>(s, kind, st, a); break;
      case 5: launch_v1<1, 0, 1>(s, kind, st, a); break;
      case 6: launch_v1<1, 1, 0>(s, kind, st, a); break;
      default: launch_v1<1, 1, 1>(s, kind, st, a); break;
    }
    return;
  }
  dim3 gr((s->g.ni + s2::TX - 1) / s2::TX, (s->g.nj + s->ty - 1) / s->ty,
          (s->g.nk + s->kchunk - 1) / s->kchunk);
  if (s->med == MED_VTI) cgfd_launch_stage_vti(code, kind, gr, st, a, s->maps);
  else if (s->med == MED_VIS) cgfd_launch_stage_vis(code, kind, gr, st, a, s->maps);
  else if (s->med == MED_ANI) cgfd_launch_stage_ani(code, kind, gr, st, a, s->maps);
  else cgfd_launch_stage_iso(code, kind, gr, st, a, s->maps);
}

/* CFS-PML corrections, faces in the reference order (after the stage kernel) */
static void launch_pml_faces(cgfd_solver_t *s, int kind, int bx, int by, int bz,
                             cudaStream_t st, const StageArgs &a)
{
  for (int f = 0; f < CGFD_NFACE; f++) {
    const DevFace &F = s->face[f];
    if (!F.on) continue;
    int dim = F.dim, b = dim == 0 ? bx : (dim == 1 ? by : bz);
    if (s->med == MED_VTI) cgfd_launch_pml_vti(dim, b, kind, f, F.avol, st, a);
    else if (s->med == MED_VIS) cgfd_launch_pml_vis(dim, b, kind, f, F.avol, st, a);
    else if (s->med == MED_ANI) cgfd_launch_pml_ani(dim, b, kind, f, F.avol, st, a);
    else cgfd_launch_pml_iso(dim, b, kind, f, F.avol, st, a);
  }
}

static const int PAIR_FLAGS[8][3] = {{0, 0, 0}, {1, 1, 0}, {1, 1, 1}, {0, 0, 1},
                                     {0, 1, 0}, {1, 0, 0}, {1, 0, 1}, {0, 1, 1}};
static const float RK_A[3] = {0.5f, 0.5f, 1.0f};
static const float RK_B[4] = {(float)(1.0 / 6.0), (float)(1.0 / 3.0),
                              (float)(1.0 / 3.0), (float)(1.0 / 6.0)};

static void fill_args(cgfd_solver_t *s, StageArgs &a, int istage)
{
  const cgfd_problem_t *p = s->p;
  memset(&a, 0, sizeof(a));
  a.g = s->g;
  size_t vol = s->g.vol;
  const float *M = s->metric;
  a.jac = M; a.xix = M + vol; a.xiy = M + 2 * vol; a.xiz = M + 3 * vol;
  a.etx = M + 4 * vol; a.ety = M + 5 * vol; a.etz = M + 6 * vol;
  a.ztx = M + 7 * vol; a.zty = M + 8 * vol; a.ztz = M + 9 * vol;
  a.slw = s->media; a.lam = s->media + vol; a.mu = s->media + 2 * vol;
  a.med = s->media;
  a.ncmp = s->ncmp;
  a.nmw = s->med == MED_VIS ? p->nmaxwell : 0;
  for (int n = 0; n < a.nmw; n++) a.wl[n] = p->wl[n];
  float *cur, *pre, *tmp, *end;
  stage_levels(s, istage, &cur, &pre, &tmp, &end);
  a.cur = cur; a.pre = pre; a.tmp_out = tmp; a.end = end;
  a.ca = istage < 3 ? RK_A[istage] * p->dt : 0.f;
  a.cb = RK_B[istage] * p->dt;
  for (int f = 0; f < CGFD_NFACE; f++) {
    a.face[f] = s->face[f];
    if (!s->face[f].on) continue;
    size_t al = 9 * (size_t)s->face[f].avol;
    float *b = s->aux[f];
    float *apre = b + s->pre_lev * al, *aend = b + s->end_lev * al;
    float *tA = b + 1 * al, *tB = b + 2 * al;
    a.apre[f] = apre;
    a.aend[f] = aend;
    if (istage == 0) { a.acur[f] = apre; a.atmp_out[f] = tA; }
    else if (istage == 1) { a.acur[f] = tA; a.atmp_out[f] = tB; }
    else if (istage == 2) { a.acur[f] = tB; a.atmp_out[f] = tA; }
    else { a.acur[f] = tA; a.atmp_out[f] = nullptr; }
  }
  a.qatt = s->qatt;
  a.free_top = p->free_top;
  if (p->free_top) {
    size_t n2 = (size_t)s->g.nx * s->g.ny * 9;
    a.mVx = s->mats; a.mVy = s->mats + n2; a.mF = s->mats + 2 * n2;
    a.mD = s->med == MED_VIS ? s->mats + 3 * n2 : nullptr;
    if (s->surf) {
      size_t s2n = (size_t)s->g.nx * s->g.ny;
      a.TS = s->surf;
      a.VS = s->surf + 3 * s2n;
    }
  }
  if (p->src_n > 0) {
    a.src_n = p->src_n;
    a.src_max_nt = p->src_max_nt;
    a.src_max_stage = p->src_max_stage;
    a.src_force = p->src_force;
    a.src_moment = p->src_moment;
    a.src_col = s->src_col;
    a.src_ent = s->src_ent;
    a.src_it_begin = s->src_it_begin;
    a.src_it_end = s->src_it_end;
    size_t nstf = (size_t)p->src_n * p->src_max_nt * p->src_max_stage;
    a.Fx = s->stf; a.Fy = s->stf + nstf; a.Fz = s->stf + 2 * nstf;
    a.Mxx = s->stf + 3 * nstf; a.Myy = s->stf + 4 * nstf; a.Mzz = s->stf + 5 * nstf;
    a.Mxz = s->stf + 6 * nstf; a.Myz = s->stf + 7 * nstf; a.Mxy = s->stf + 8 * nstf;
  }
  if (p->dd_n > 0) {
    a.dd_n = p->dd_n;
    a.dd_max_nt = p->dd_max_nt;
    a.dd_col = s->dd_col;
    a.dd_ent = s->dd_ent;
    size_t nt = (size_t)p->dd_max_nt * 4 * p->dd_n;
    a.dd_vi = p->dd_vi ? s->dd_tab : nullptr;
    a.dd_mij = p->dd_mij ? s->dd_tab + 3 * nt : nullptr;
  }
  a.d_it = s->d_it;
  a.istage = istage;
  a.err = s->d_err;
  a.wait_limit = s->wait_limit;
  a.test_skip_plane = s->test_skip_plane;
  a.kchunk = s->kchunk;
  a.pml_fused = s->pml_fused;
  a.l2_ahead = s->l2_ahead;
  size_t L = level_floats(s);
  a.cur_level = (int)((cur - s->wav) / (long long)L);
  a.pre_level = (int)((pre - s->wav) / (long long)L);
  a.end_level = (int)((end - s->wav) / (long long)L);
}

/* enqueue one step (4 stages + receivers) for step index `it` */
static int enqueue_step(cgfd_solver_t *s, int it, int *ev_next)
{
  const cgfd_problem_t *p = s->p;
  cudaStream_t st = s->stream;
  int ipair = it % 8;
  for (int is = 0; is < 4; is++) {
    StageArgs a;
    fill_args(s, a, is);
    int bx = (PAIR_FLAGS[ipair][0] + is) % 2;
    int by = (PAIR_FLAGS[ipair][1] + is) % 2;
    int bz = (PAIR_FLAGS[ipair][2] + is) % 2;
    int kind = is == 0 ? 0 : (is < 3 ? 1 : 2);
    int code = bx * 4 + by * 2 + bz;
    if (s->nsf > 0) {
      /* surface force layers of this stage (drv_rk_curv_col.c:230) */
      dim3 b2(32, 8), g2((s->g.ni + 31) / 32, (s->g.nj + 7) / 8);
      size_t nstf = (size_t)p->src_n * p->src_max_nt * p->src_max_stage;
      size_t nr = (size_t)s->nsf * p->src_max_nt * p->src_max_stage;
      size_t s2n = (size_t)s->g.nx * s->g.ny;
      k_surf_layer<<<g2, b2, 0, st>>>(s->g, s->nsf, s->sf, s->sf_w, s->metric,
                                      s->src_it_begin, s->src_it_end, s->stf,
                                      s->stf + nstf, s->stf + 2 * nstf, s->frate,
                                      s->frate + nr, s->frate + 2 * nr,
                                      p->src_max_nt, p->src_max_stage, is, s->d_it,
                                      s->surf, s->surf + 3 * s2n);
    }
    if (ev_next) cudaEventRecord(s->kev[(*ev_next)++], st);
    launch_stage(s, code, kind, st, a);
    if (ev_next) cudaEventRecord(s->kev[(*ev_next)++], st);
    if (s->kernel == 2 && !s->pml_fused) launch_pml_faces(s, kind, bx, by, bz, st, a);
    if (ev_next) cudaEventRecord(s->kev[(*ev_next)++], st);
  }
  size_t L = level_floats(s);
  if (s->med == MED_VIS && p->free_top) {
    /* surface stress rotation after the last stage (drv_rk_curv_col.c:440-445) */
    dim3 b(32, 8), gr((s->g.ni + 31) / 32, (s->g.nj + 7) / 8);
    size_t n2 = (size_t)s->g.nx * s->g.ny * 9;
    k_vis_free<<<gr, b, 0, st>>>(s->g, s->wav + s->end_lev * L, s->mats + 3 * n2);
  }
  if (s->abl) {
    /* exponential sponge (forward/drv_rk_curv_col.c:484-486) */
    long long nb = (s->abx.first[s->abx.n] + 255) / 256;
    k_ablexp<<<(int)(nb < 152 * 8 ? nb : 152 * 8), 256, 0, st>>>(
        s->g, s->wav + s->end_lev * L, s->ncmp, s->abx, s->abl, s->abl + s->g.nx,
        s->abl + s->g.nx + s->g.ny);
  }
  if (s->pg) {
    dim3 b(32, 8), gr((s->g.ni + 31) / 32, (s->g.nj + 7) / 8);
    k_pg<<<gr, b, 0, st>>>(s->g, s->wav + s->end_lev * L, s->wav + s->pre_lev * L,
                           s->pg, s->dis, p->dt);
  }
  k_recv<<<1, 256, 0, st>>>(s->wav + s->end_lev * L, s->g.vol, s->ncmp,
                            p->recv_n, p->recv_ncmp, p->recv_max_nt, s->recv_dijk,
                            s->recv_idx, s->recv_seismo, p->line_n, p->line_max_nt,
                            s->line_iptr, s->line_seismo, s->d_it);
  /* swap pre and end (forward/drv_rk_curv_col.c:530-542) */
  int t = s->pre_lev; s->pre_lev = s->end_lev; s->end_lev = t;
  return 0;
}

extern "C" int cgfd_solver_run(cgfd_solver_t *s, int nsteps)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (nsteps < 0 || s->step + nsteps > s->p->nt_total)
    return set_err(CGFD_EINVAL, "run(%d) past nt_total=%d (at step %d)", nsteps,
                   s->p->nt_total, s->step);
  int nev = s->timing ? 12 * nsteps : 0;
  while ((int)s->kev.size() < nev) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    s->kev.push_back(e);
  }
  int ev = 0;
  CK(cudaEventRecord(s->ev0, s->stream));
  for (int n = 0; n < nsteps; n++) {
    enqueue_step(s, s->step, s->timing ? &ev : nullptr);
    s->step++;
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(s->ev1, s->stream));
  CK(cudaEventSynchronize(s->ev1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
  s->t_total_ms = ms;
  s->t_stage_ms = 0.f;
  s->t_pml_ms = 0.f;
  if (s->timing) {
    for (int e = 0; e < ev; e += 3) {
      float t = 0.f, t2 = 0.f;
      CK(cudaEventElapsedTime(&t, s->kev[e], s->kev[e + 1]));
      CK(cudaEventElapsedTime(&t2, s->kev[e + 1], s->kev[e + 2]));
      s->t_stage_ms += t;
      s->t_pml_ms += t2;
    }
  }
  int nfaces = 0;
  for (int f = 0; f < CGFD_NFACE; f++) nfaces += s->face[f].on;
  s->t_other_ms = s->timing ? ms - s->t_stage_ms : 0.f;
  s->n_stage = 4 * nsteps;
  s->n_pml = (s->kernel == 2 && !s->pml_fused) ? 4 * nfaces * nsteps : 0;
  s->n_other = nsteps * (1 + (s->pg ? 1 : 0) + (s->med == MED_VIS && s->p->free_top ? 1 : 0) +
                         (s->nsf > 0 ? 4 : 0));
  int herr = 0;
  CK(cudaMemcpy(&herr, s->d_err, 4, cudaMemcpyDeviceToHost));
  if (herr) return set_err(CGFD_ECUDA, "device wait timed out (code %d)", herr);
  return 0;
}

extern "C" int cgfd_solver_run_async(cgfd_solver_t *s, int nsteps)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (nsteps < 0 || s->step + nsteps > s->p->nt_total)
    return set_err(CGFD_EINVAL, "run(%d) past nt_total=%d (at step %d)", nsteps,
                   s->p->nt_total, s->step);
  for (int n = 0; n < nsteps; n++) {
    enqueue_step(s, s->step, nullptr);
    s->step++;
  }
  CK(cudaGetLastError());
  return 0;
}

extern "C" int cgfd_solver_step(const cgfd_solver_t *s) { return s ? s->step : -1; }

extern "C" int cgfd_solver_kernel_times(const cgfd_solver_t *s, float out[3], int count[3])
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  out[0] = s->t_stage_ms; out[1] = s->t_total_ms; out[2] = s->t_pml_ms;
  count[0] = s->n_stage; count[1] = s->n_stage + s->n_pml + s->n_other;
  count[2] = s->n_pml;
  return 0;
}

extern "C" int cgfd_solver_set_wait_test(cgfd_solver_t *s, int wait_limit, int skip_plane)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (wait_limit < 0 || skip_plane < -1)
    return set_err(CGFD_EINVAL, "wait test: limit %d, plane %d", wait_limit, skip_plane);
  s->wait_limit = wait_limit;
  s->test_skip_plane = skip_plane;
  return 0;
}

extern "C" int cgfd_solver_set_timing(cgfd_solver_t *s, int on)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  s->timing = on ? 1 : 0;
  return 0;
}

extern "C" int cgfd_solver_transfer_bytes(const cgfd_solver_t *s, size_t *h2d, size_t *d2h)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  *h2d = s->h2d_bytes;
  *d2h = s->d2h_bytes;
  return 0;
}

extern "C" int cgfd_solver_fetch(cgfd_solver_t *s)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  const cgfd_problem_t *p = s->p;
  size_t L = level_floats(s);
  int host_lev = (s->step % 2 == 1) ? 3 : 0;
  size_t hvol = (size_t)p->nx * p->ny * p->nz;
  SetupTrace tr;
  tr.start(s->stream);
  for (int c = 0; c < s->ncmp; c++)
    CK(download_volume(s, p->wav + (size_t)host_lev * s->ncmp * hvol + c * hvol,
                       s->wav + s->pre_lev * L + c * s->g.vol));
  tr.mark("fetch wavefield");
  for (int d = 0; d < 3; d++)
    for (int sd = 0; sd < 2; sd++) {
      int f = d * 2 + sd;
      if (!s->face[f].on) continue;
      size_t av = (size_t)s->face[f].avol;
      size_t al = 9 * av;
      float *hl = p->pml[d][sd].aux + (size_t)host_lev * s->ncmp * av;
      CK(cudaMemcpyAsync(hl, s->aux[f] + s->pre_lev * al, al * sizeof(float),
                         cudaMemcpyDeviceToHost, s->stream));
      s->d2h_bytes += al * sizeof(float);
      /* memory-variable components of the aux: never updated by the PML,
       * every level keeps the input values (rhs stays 0 in the reference) */
      if (s->ncmp > 9 && host_lev != 0)
        memcpy(hl + al, p->pml[d][sd].aux + al, (size_t)(s->ncmp - 9) * av * sizeof(float));
    }
  if (p->recv_n > 0) {
    size_t nb = (size_t)p->recv_n * p->recv_ncmp * p->recv_max_nt * 4;
    CK(cudaMemcpyAsync(p->recv_seismo, s->recv_seismo, nb,
                       cudaMemcpyDeviceToHost, s->stream));
    s->d2h_bytes += nb;
  }
  if (p->line_n > 0) {
    size_t nb = (size_t)p->line_n * p->ncmp * p->line_max_nt * 4;
    CK(cudaMemcpyAsync(p->line_seismo, s->line_seismo, nb,
                       cudaMemcpyDeviceToHost, s->stream));
    s->d2h_bytes += nb;
  }
  CK(cudaStreamSynchronize(s->stream));
  tr.mark("fetch PML, seismograms");
  return 0;
}

extern "C" int cgfd_solver_fetch_seismograms(cgfd_solver_t *s)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  const cgfd_problem_t *p = s->p;
  if (p->recv_n > 0) {
    size_t nb = (size_t)p->recv_n * p->recv_ncmp * p->recv_max_nt * 4;
    CK(cudaMemcpyAsync(p->recv_seismo, s->recv_seismo, nb, cudaMemcpyDeviceToHost, s->stream));
    s->d2h_bytes += nb;
  }
  if (p->line_n > 0) {
    size_t nb = (size_t)p->line_n * p->ncmp * p->line_max_nt * 4;
    CK(cudaMemcpyAsync(p->line_seismo, s->line_seismo, nb, cudaMemcpyDeviceToHost, s->stream));
    s->d2h_bytes += nb;
  }
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

extern "C" int cgfd_solver_fetch_surface_matrices(cgfd_solver_t *s, float *mVx,
                                                  float *mVy, float *mF)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (!s->mats) return set_err(CGFD_EINVAL, "no free surface");
  size_t n2 = (size_t)s->g.nx * s->g.ny * 9;
  float *dst[3] = {mVx, mVy, mF};
  for (int m = 0; m < 3; m++)
    if (dst[m]) CK(cudaMemcpy(dst[m], s->mats + m * n2, n2 * 4, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int cgfd_solver_fetch_surface_rotation(cgfd_solver_t *s, float *mD)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (!s->mats || s->med != MED_VIS)
    return set_err(CGFD_EINVAL, "no visco-elastic free surface");
  size_t n2 = (size_t)s->g.nx * s->g.ny * 9;
  CK(cudaMemcpy(mD, s->mats + 3 * n2, n2 * 4, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int cgfd_solver_fetch_pg(cgfd_solver_t *s, float *pg)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (!s->pg) return set_err(CGFD_EINVAL, "no free surface, no peak-motion maps");
  size_t n = 15 * (size_t)s->g.nx * s->g.ny;
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemcpy(pg, s->pg, n * 4, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int cgfd_solver_fetch_state(cgfd_solver_t *s, float *w)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  size_t hvol = (size_t)s->g.nx * s->g.ny * s->g.nz;
  size_t L = level_floats(s);
  for (int c = 0; c < s->ncmp; c++)
    CK(download_volume(s, w + c * hvol, s->wav + s->pre_lev * L + c * s->g.vol));
  CK(cudaStreamSynchronize(s->stream));
  return 0;
}

static size_t box_floats(const cgfd_box_t &b)
{
  if (b.c2 < b.c1 || b.ni < 1 || b.nj < 1 || b.nk < 1 || b.di < 1 || b.dj < 1 ||
      b.dk < 1)
    return 0;
  return (size_t)(b.c2 - b.c1 + 1) * b.ni * b.nj * b.nk;
}

extern "C" size_t cgfd_box_floats(const cgfd_box_t *box, int nbox)
{
  if (!box || nbox < 1) return 0;
  size_t n = 0;
  for (int m = 0; m < nbox; m++) {
    size_t f = box_floats(box[m]);
    if (!f) return 0;
    n += f;
  }
  return n;
}

/* Writes packed boxes into w (ncmp x nx*ny*nz) at their positions.  One
 * task per (box, component); an x slice scatters one float per grid row,
 * bound by cache and TLB misses rather than bandwidth, so large sets are
 * split over a few host threads. */
static void scatter_boxes(const DevGrid &g, const std::vector<cgfd_box_t> &boxes,
                          const float *packed, float *w)
{
  struct Task { const cgfd_box_t *b; int c; const float *src; };
  std::vector<Task> task;
  const float *q = packed;
  size_t total = 0;
  for (const cgfd_box_t &b : boxes) {
    const size_t per = (size_t)b.ni * b.nj * b.nk;
    for (int c = b.c1; c <= b.c2; c++, q += per) task.push_back({&b, c, q});
    total += per * (b.c2 - b.c1 + 1);
  }
  const size_t nx = g.nx, sl = nx * g.ny, hvol = sl * g.nz;
  auto run = [&](size_t t0, size_t step) {
    for (size_t t = t0; t < task.size(); t += step) {
      const cgfd_box_t &b = *task[t].b;
      const float *src = task[t].src;
      for (int kk = 0; kk < b.nk; kk++)
        for (int jj = 0; jj < b.nj; jj++) {
          float *row = w + task[t].c * hvol + (size_t)(b.k1 + kk * b.dk) * sl +
                       (size_t)(b.j1 + jj * b.dj) * nx + b.i1;
          if (b.di == 1) {
            memcpy(row, src, b.ni * sizeof(float));
            src += b.ni;
          } else {
            for (int ii = 0; ii < b.ni; ii++) row[(size_t)ii * b.di] = *src++;
          }
        }
    }
  };
  unsigned hw = std::thread::hardware_concurrency();
  size_t nth = total < (1u << 18) ? 1 : std::min<size_t>({task.size(), 8, hw ? hw : 1});
  if (nth <= 1) {
    run(0, 1);
    return;
  }
  std::vector<std::thread> th;
  for (size_t t = 1; t < nth; t++) th.emplace_back(run, t, nth);
  run(0, nth);
  for (std::thread &t : th) t.join();
}

/* Queues the packing of boxes of the current state into slot o: box table
 * upload, gather kernel, copy to pinned host memory and the device error
 * flag behind it, then the slot's event.  Returns without waiting. */
static int pack_enqueue(cgfd_solver_t *s, OutSlot &o, const cgfd_box_t *box, int nbox)
{
  if (!box || nbox < 1) return set_err(CGFD_EINVAL, "no output boxes");
  if (o.pending) return set_err(CGFD_EINVAL, "output slot still holds uncollected boxes");
  const DevGrid &g = s->g;
  std::vector<long long> off(nbox);
  size_t total = 0;
  for (int m = 0; m < nbox; m++) {
    const cgfd_box_t &b = box[m];
    size_t f = box_floats(b);
    if (!f) return set_err(CGFD_EINVAL, "output box %d: empty count, stride or component range", m);
    if (b.c1 < 0 || b.c2 >= s->ncmp)
      return set_err(CGFD_EINVAL, "output box %d: components %d..%d outside 0..%d", m,
                     b.c1, b.c2, s->ncmp - 1);
    if (b.i1 < 0 || b.j1 < 0 || b.k1 < 0 ||
        b.i1 + (long long)(b.ni - 1) * b.di >= g.nx ||
        b.j1 + (long long)(b.nj - 1) * b.dj >= g.ny ||
        b.k1 + (long long)(b.nk - 1) * b.dk >= g.nz)
      return set_err(CGFD_EINVAL, "output box %d outside the padded grid", m);
    off[m] = (long long)total;
    total += f;
  }
  if (!o.ev) {
    CK(cudaEventCreateWithFlags(&o.ev, cudaEventDisableTiming));
    CK(cudaMallocHost((void **)&o.h_err, sizeof(int)));
  }
  if (nbox > o.cap) {
    if (o.d_box) cudaFree(o.d_box);
    if (o.d_off) cudaFree(o.d_off);
    if (o.h_box) cudaFreeHost(o.h_box);
    if (o.h_off) cudaFreeHost(o.h_off);
    o.d_box = nullptr; o.d_off = nullptr; o.h_box = nullptr; o.h_off = nullptr;
    o.cap = 0;
    CK(cudaMalloc((void **)&o.d_box, nbox * sizeof(cgfd_box_t)));
    CK(cudaMalloc((void **)&o.d_off, nbox * sizeof(long long)));
    CK(cudaMallocHost((void **)&o.h_box, nbox * sizeof(cgfd_box_t)));
    CK(cudaMallocHost((void **)&o.h_off, nbox * sizeof(long long)));
    o.cap = nbox;
  }
  if (total > o.pack_cap) {
    if (o.d_pack) cudaFree(o.d_pack);
    if (o.h_pack) cudaFreeHost(o.h_pack);
    o.d_pack = nullptr; o.h_pack = nullptr; o.pack_cap = 0;
    CK(cudaMalloc((void **)&o.d_pack, total * sizeof(float)));
    CK(cudaMallocHost((void **)&o.h_pack, total * sizeof(float)));
    o.pack_cap = total;
  }
  /* the table goes through the slot's pinned copy: a copy from pageable
   * memory may wait for the stream, which would end the overlap */
  memcpy(o.h_box, box, nbox * sizeof(cgfd_box_t));
  memcpy(o.h_off, off.data(), nbox * sizeof(long long));
  CK(cudaMemcpyAsync(o.d_box, o.h_box, nbox * sizeof(cgfd_box_t), cudaMemcpyHostToDevice,
                     s->stream));
  CK(cudaMemcpyAsync(o.d_off, o.h_off, nbox * sizeof(long long), cudaMemcpyHostToDevice,
                     s->stream));
  long long nblk = ((long long)total + 255) / 256;
  if (nblk > 152 * 8) nblk = 152 * 8;
  k_pack_boxes<<<(int)nblk, 256, 0, s->stream>>>(s->wav + s->pre_lev * level_floats(s),
                                                  g.vol, g, o.d_box, o.d_off, nbox,
                                                  (long long)total, o.d_pack);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(o.h_pack, o.d_pack, total * sizeof(float), cudaMemcpyDeviceToHost,
                     s->stream));
  CK(cudaMemcpyAsync(o.h_err, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaEventRecord(o.ev, s->stream));
  s->d2h_bytes += total * sizeof(float);
  o.boxes.assign(box, box + nbox);
  o.n = total;
  o.pending = 1;
  return 0;
}

/* Waits for slot o and hands its boxes out: scattered into w (reference
 * layout) and/or packed into out; either may be null. */
static int pack_collect(cgfd_solver_t *s, OutSlot &o, float *w, float *out)
{
  if (!o.pending) return set_err(CGFD_EINVAL, "output slot holds no boxes");
  o.pending = 0;
  CK(cudaEventSynchronize(o.ev));
  if (*o.h_err) return set_err(CGFD_ECUDA, "device wait timed out (code %d)", *o.h_err);
  if (out) memcpy(out, o.h_pack, o.n * sizeof(float));
  if (w) scatter_boxes(s->g, o.boxes, o.h_pack, w);
  return 0;
}

extern "C" int cgfd_solver_pack_boxes(cgfd_solver_t *s, const cgfd_box_t *box, int nbox,
                                      float *out)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  OutSlot &o = s->out[CGFD_OUT_SLOTS];
  int rc = pack_enqueue(s, o, box, nbox);
  return rc ? rc : pack_collect(s, o, nullptr, out);
}

extern "C" int cgfd_solver_fetch_boxes(cgfd_solver_t *s, const cgfd_box_t *box, int nbox,
                                       float *w)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  OutSlot &o = s->out[CGFD_OUT_SLOTS];
  int rc = pack_enqueue(s, o, box, nbox);
  return rc ? rc : pack_collect(s, o, w, nullptr);
}

extern "C" int cgfd_solver_pack_boxes_async(cgfd_solver_t *s, const cgfd_box_t *box,
                                            int nbox, int slot)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (slot < 0 || slot >= CGFD_OUT_SLOTS)
    return set_err(CGFD_EINVAL, "output slot %d outside 0..%d", slot, CGFD_OUT_SLOTS - 1);
  return pack_enqueue(s, s->out[slot], box, nbox);
}

extern "C" int cgfd_solver_collect_boxes(cgfd_solver_t *s, int slot, float *w, float *out)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  if (slot < 0 || slot >= CGFD_OUT_SLOTS)
    return set_err(CGFD_EINVAL, "output slot %d outside 0..%d", slot, CGFD_OUT_SLOTS - 1);
  return pack_collect(s, s->out[slot], w, out);
}

extern "C" int cgfd_solver_check_finite(cgfd_solver_t *s)
{
  if (!s) return set_err(CGFD_EINVAL, "null solver");
  size_t L = level_floats(s);
  CK(cudaMemsetAsync(s->d_flag, 0, 4, s->stream));
  k_nonfinite<<<152 * 4, 256, 0, s->stream>>>(s->wav + s->pre_lev * L, L, s->d_flag);
  CK(cudaGetLastError());
  int h = 0;
  CK(cudaMemcpyAsync(&h, s->d_flag, 4, cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  return h ? set_err(CGFD_ENONFINITE, "wavefield holds NaN/Inf at step %d", s->step) : 0;
}

extern "C" int cgfd_allstep(const cgfd_problem_t *p)
{
  cgfd_solver_t *s = nullptr;
  int rc = cgfd_solver_create(p, &s);
  if (rc) return rc;
  rc = cgfd_solver_run(s, p->nt_total);
  if (!rc) rc = cgfd_solver_fetch(s);
  cgfd_solver_destroy(s);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* reset (used by the batch autotuner)                                       */
/* ------------------------------------------------------------------------ */

/* Puts a solver back at step 0 with the problem's host inputs: wavefield
 * level 0 and PML auxiliary level 0 into all four levels, seismograms,
 * peak-motion maps and the step counter zeroed. */
static int solver_reset(cgfd_solver_t *s)
{
  const cgfd_problem_t *p = s->p;
  const DevGrid &g = s->g;
  cudaStream_t st = s->stream;
  size_t vol = g.vol, L = level_floats(s);
  size_t hvol = (size_t)p->nx * p->ny * p->nz;
  for (int c = 0; c < s->ncmp; c++) CK(upload_volume(s, s->wav + c * vol, p->wav + c * hvol));
  for (int l = 1; l < 4; l++)
    CK(cudaMemcpyAsync(s->wav + l * L, s->wav, L * sizeof(float), cudaMemcpyDeviceToDevice, st));
  for (int d = 0; d < 3; d++)
    for (int sd = 0; sd < 2; sd++) {
      int f = d * 2 + sd;
      if (!s->face[f].on) continue;
      size_t al = 9 * (size_t)s->face[f].avol;
      CK(cudaMemcpyAsync(s->aux[f], p->pml[d][sd].aux, al * sizeof(float),
                         cudaMemcpyHostToDevice, st));
      for (int l = 1; l < 4; l++)
        CK(cudaMemcpyAsync(s->aux[f] + l * al, s->aux[f], al * sizeof(float),
                           cudaMemcpyDeviceToDevice, st));
    }
  if (s->recv_seismo)
    CK(cudaMemsetAsync(s->recv_seismo, 0,
                       (size_t)p->recv_n * p->recv_ncmp * p->recv_max_nt * 4, st));
  if (s->line_seismo)
    CK(cudaMemsetAsync(s->line_seismo, 0, (size_t)p->line_n * p->ncmp * p->line_max_nt * 4, st));
  if (s->pg) {
    size_t s2n = (size_t)p->nx * p->ny;
    CK(cudaMemsetAsync(s->pg, 0, 15 * s2n * 4, st));
    CK(cudaMemsetAsync(s->dis, 0, 3 * s2n * 4, st));
  }
  CK(cudaMemsetAsync(s->d_it, 0, 4, st));
  CK(cudaStreamSynchronize(st));
  release_staging(s);
  s->step = 0;
  s->pre_lev = 0;
  s->end_lev = 3;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* batched shots                                                             */
/* ------------------------------------------------------------------------ */

/* receivers / lines of one shot after a step (arguments of k_recv) */
struct RecvJob {
  const float *w;
  long long vol;
  int ncmp, nrecv, recv_ncmp, recv_max_nt;
  const float *dijk;
  const int *idx8;
  float *seismo;
  int nline, line_max_nt;
  const int *line_iptr;
  float *line_seismo;
  int *d_it;
};

/* peak-motion maps of one shot after a step (arguments of k_pg) */
struct PgJob {
  DevGrid g;
  const float *w1, *w0;
  float *pg, *dis;
  float dt;
  int on;
};

/* k_recv for every shot of a batch: one block per shot */
__global__ void k_recv_batch(const RecvJob *__restrict__ jobs)
{
  const RecvJob &J = jobs[blockIdx.x];
  const int it = *J.d_it;
  for (int t = threadIdx.x; t < J.nrecv * J.recv_ncmp; t += blockDim.x) {
    int n = t / J.recv_ncmp, c = t % J.recv_ncmp;
    const int *x = J.idx8 + 8 * n;
    float Lx2 = J.dijk[3 * n], Ly2 = J.dijk[3 * n + 1], Lz2 = J.dijk[3 * n + 2];
    float Lx1 = 1.0f - Lx2, Ly1 = 1.0f - Ly2, Lz1 = 1.0f - Lz2;
    const float *v = J.w + c * J.vol;
    J.seismo[((long long)n * J.recv_ncmp + c) * J.recv_max_nt + it] =
        v[x[0]] * Lx1 * Ly1 * Lz1 + v[x[1]] * Lx2 * Ly1 * Lz1 +
        v[x[2]] * Lx1 * Ly2 * Lz1 + v[x[3]] * Lx2 * Ly2 * Lz1 +
        v[x[5]] * Lx1 * Ly1 * Lz2 + v[x[5]] * Lx2 * Ly1 * Lz2 +
        v[x[6]] * Lx1 * Ly2 * Lz2 + v[x[7]] * Lx2 * Ly2 * Lz2;
  }
  for (int t = threadIdx.x; t < J.nline * J.ncmp; t += blockDim.x) {
    int n = t / J.ncmp, c = t % J.ncmp;
    J.line_seismo[((long long)n * J.ncmp + c) * J.line_max_nt + it] =
        J.w[c * J.vol + J.line_iptr[n]];
  }
  __syncthreads();
  if (threadIdx.x == 0) *J.d_it = it + 1;
}

/* k_pg for every shot of a batch: blockIdx.z is the shot */
__global__ void k_pg_batch(const PgJob *__restrict__ jobs)
{
  const PgJob &J = jobs[blockIdx.z];
  if (!J.on) return;
  const DevGrid &g = J.g;
  int i = g.ni1 + blockIdx.x * blockDim.x + threadIdx.x;
  int j = g.nj1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (i > g.ni2 || j > g.nj2) return;
  long long q = (i + g.xoff) + (long long)j * g.px + (long long)g.nk2 * g.sl;
  long long s2 = (long long)g.nx * g.ny;
  long long q2 = i + (long long)j * g.nx;
  const float dt = J.dt;
  float vx1 = J.w1[q], vy1 = J.w1[g.vol + q], vz1 = J.w1[2 * g.vol + q];
  float vx0 = J.w0[q], vy0 = J.w0[g.vol + q], vz0 = J.w0[2 * g.vol + q];
  float Ax = fabsf((vx1 - vx0) / dt), Ay = fabsf((vy1 - vy0) / dt),
        Az = fabsf((vz1 - vz0) / dt);
  float Dx = J.dis[q2] + 0.5f * (vx1 + vx0) * dt;
  float Dy = J.dis[s2 + q2] + 0.5f * (vy1 + vy0) * dt;
  float Dz = J.dis[2 * s2 + q2] + 0.5f * (vz1 + vz0) * dt;
  J.dis[q2] = Dx; J.dis[s2 + q2] = Dy; J.dis[2 * s2 + q2] = Dz;
  float v[15] = {sqrtf(vx1 * vx1 + vy1 * vy1 + vz1 * vz1), sqrtf(vx1 * vx1 + vy1 * vy1),
                 fabsf(vx1), fabsf(vy1), fabsf(vz1),
                 sqrtf(Ax * Ax + Ay * Ay + Az * Az), sqrtf(Ax * Ax + Ay * Ay), Ax, Ay, Az,
                 sqrtf(Dx * Dx + Dy * Dy + Dz * Dz), sqrtf(Dx * Dx + Dy * Dy),
                 fabsf(Dx), fabsf(Dy), fabsf(Dz)};
#pragma unroll
  for (int m = 0; m < 15; m++) {
    float *p = J.pg + m * s2 + q2;
    if (*p < v[m]) *p = v[m];
  }
}

struct cgfd_batch {
  std::vector<cgfd_solver_t *> sv;
  int n = 0;
  int med = MED_ISO;
  int kchunk = 16;
  int step = 0;
  int par = 0;                    /* level parity: 0 pre=0/end=3, 1 swapped */
  int nt_total = 0;
  cudaStream_t stream = nullptr;
  StageArgs *d_args = nullptr;    /* [parity][stage][shot] */
  s3::ShotGeo *d_geo = nullptr;   /* [shot] */
  RecvJob *d_recv = nullptr;      /* [parity][shot] */
  PgJob *d_pg = nullptr;          /* [parity][shot] */
  int nctas = 0, pg_any = 0, max_ni = 0, max_nj = 0;
  /* schedule of the stage launches: 0 one CTA per (shot, tile, k chunk)
   * item, 1 persistent CTAs (one per SM) taking the items largest first */
  int persistent = 0, pgrid = 0;
  int *d_order = nullptr;         /* items, largest first */
  int *d_next = nullptr;          /* the persistent launches' item counter */
  cudaError_t enq_err = cudaSuccess;   /* first error of an enqueue call */
  cudaGraphExec_t graph = nullptr;
  int graph_par = -1;
  int use_graph = 1;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float t_ms = 0.f;
  int launches = 0;
};

static void batch_free_tables(cgfd_batch_t *b)
{
  void *ptrs[] = {b->d_args, b->d_geo, b->d_recv, b->d_pg, b->d_order, b->d_next};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  b->d_args = nullptr; b->d_geo = nullptr; b->d_recv = nullptr; b->d_pg = nullptr;
  b->d_order = nullptr; b->d_next = nullptr;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  b->graph_par = -1;
}

/* device tables of the batch for its current kchunk */
static int batch_tables(cgfd_batch_t *b)
{
  batch_free_tables(b);
  const int n = b->n;
  std::vector<StageArgs> args((size_t)8 * n);
  std::vector<s3::ShotGeo> geo(n);
  std::vector<RecvJob> rj((size_t)2 * n);
  std::vector<PgJob> pj((size_t)2 * n);
  int cta = 0;
  b->pg_any = 0; b->max_ni = 0; b->max_nj = 0;
  for (int k = 0; k < n; k++) {
    cgfd_solver_t *s = b->sv[k];
    s->kchunk = b->kchunk;
    const int pre0 = s->pre_lev, end0 = s->end_lev;
    for (int par = 0; par < 2; par++) {
      s->pre_lev = par == 0 ? 0 : 3;
      s->end_lev = par == 0 ? 3 : 0;
      for (int is = 0; is < 4; is++) fill_args(s, args[(size_t)(par * 4 + is) * n + k], is);
      size_t L = level_floats(s);
      RecvJob &r = rj[(size_t)par * n + k];
      const cgfd_problem_t *p = s->p;
      r.w = s->wav + s->end_lev * L; r.vol = s->g.vol; r.ncmp = s->ncmp;
      r.nrecv = p->recv_n; r.recv_ncmp = p->recv_ncmp; r.recv_max_nt = p->recv_max_nt;
      r.dijk = s->recv_dijk; r.idx8 = s->recv_idx; r.seismo = s->recv_seismo;
      r.nline = p->line_n; r.line_max_nt = p->line_max_nt; r.line_iptr = s->line_iptr;
      r.line_seismo = s->line_seismo; r.d_it = s->d_it;
      PgJob &g = pj[(size_t)par * n + k];
      g.g = s->g; g.w1 = s->wav + s->end_lev * L; g.w0 = s->wav + s->pre_lev * L;
      g.pg = s->pg; g.dis = s->dis; g.dt = p->dt; g.on = s->pg != nullptr;
    }
    s->pre_lev = pre0; s->end_lev = end0;
    s3::ShotGeo &G = geo[k];
    memset(&G, 0, sizeof(G));
    G.wav = s->maps.wav; G.met = s->maps.met; G.med = s->maps.med;
    G.pt = s->maps.pt; G.j = s->maps.j;
    G.tiles_x = (s->g.ni + s2::TX - 1) / s2::TX;
    G.tiles_y = (s->g.nj + s->ty - 1) / s->ty;
    G.nchunk = (s->g.nk + b->kchunk - 1) / b->kchunk;
    G.cta0 = cta;
    cta += G.tiles_x * G.tiles_y * G.nchunk;
    b->pg_any |= s->pg != nullptr;
    b->max_ni = std::max(b->max_ni, s->g.ni);
    b->max_nj = std::max(b->max_nj, s->g.nj);
  }
  b->nctas = cta;
  /* the persistent schedule's item order: most points x planes first, so
   * that the short edge tiles and chunks fill the end of the launch */
  std::vector<int> order(cta);
  std::vector<long long> cost(cta);
  for (int k = 0; k < n; k++) {
    const cgfd_solver_t *s = b->sv[k];
    const s3::ShotGeo &G = geo[k];
    const int nitem = G.tiles_x * G.tiles_y * G.nchunk;
    for (int c = 0; c < nitem; c++) {
      const int bx = c % G.tiles_x, by = (c / G.tiles_x) % G.tiles_y,
                bz = c / (G.tiles_x * G.tiles_y);
      const long long wi = std::min(s2::TX, s->g.ni - bx * s2::TX);
      const long long wj = std::min(s->ty, s->g.nj - by * s->ty);
      const long long wk = std::min(b->kchunk, s->g.nk - bz * b->kchunk);
      cost[G.cta0 + c] = wi * wj * wk;
    }
  }
  for (int c = 0; c < cta; c++) order[c] = c;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return cost[x] > cost[y]; });
  CK(cudaMalloc((void **)&b->d_order, (size_t)cta * sizeof(int)));
  CK(cudaMalloc((void **)&b->d_next, sizeof(int)));
  CK(cudaMemcpy(b->d_order, order.data(), (size_t)cta * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMalloc((void **)&b->d_args, args.size() * sizeof(StageArgs)));
  CK(cudaMalloc((void **)&b->d_geo, geo.size() * sizeof(s3::ShotGeo)));
  CK(cudaMalloc((void **)&b->d_recv, rj.size() * sizeof(RecvJob)));
  CK(cudaMalloc((void **)&b->d_pg, pj.size() * sizeof(PgJob)));
  CK(cudaMemcpy(b->d_args, args.data(), args.size() * sizeof(StageArgs), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_geo, geo.data(), geo.size() * sizeof(s3::ShotGeo), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_recv, rj.data(), rj.size() * sizeof(RecvJob), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_pg, pj.data(), pj.size() * sizeof(PgJob), cudaMemcpyHostToDevice));
  return 0;
}

extern "C" void cgfd_batch_destroy(cgfd_batch_t *b)
{
  if (!b) return;
  batch_free_tables(b);
  for (cgfd_solver_t *s : b->sv) cgfd_solver_destroy(s);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

extern "C" int cgfd_batch_create(const cgfd_problem_t *const *shots, int nshot,
                                 int kchunk, cgfd_batch_t **out)
{
  *out = nullptr;
  if (!shots || nshot < 1) return set_err(CGFD_EINVAL, "empty batch");
  for (int k = 0; k < nshot; k++) {
    const cgfd_problem_t *p = shots[k];
    if (!p) return set_err(CGFD_EINVAL, "shot %d: null problem", k);
    if (p->medium_type != shots[0]->medium_type)
      return set_err(CGFD_EINVAL, "shot %d: every shot of a batch has the same medium", k);
    if (p->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO ||
        p->medium_type == CGFD_MEDIUM_ELASTIC_ANISO)
      return set_err(CGFD_EINVAL, "batched shots: isotropic and VTI elastic media only");
    if (p->src_n > 0 && p->src_n_surface_force > 0)
      return set_err(CGFD_EINVAL, "shot %d: surface force sources are not batched", k);
    if (p->ablexp)
      return set_err(CGFD_EINVAL, "shot %d: the exponential sponge is not batched "
                     "(CFS-PML is)", k);
    if (p->dd_n > 0)
      return set_err(CGFD_EINVAL, "shot %d: distributed sources are not batched", k);
    if (p->nt_total != shots[0]->nt_total || p->dt != shots[0]->dt)
      return set_err(CGFD_EINVAL, "shot %d: every shot steps with the same dt and nt_total", k);
  }
  {
    /* the batched kernel reuses each shot's tensor maps: its tile rows must
     * be the single kernel's */
    const int med = medium_of(shots[0]->medium_type);
    const int rows_single = med == MED_VTI ? cgfd_stage_rows_vti() : cgfd_stage_rows_iso();
    const int rows_batch = med == MED_VTI ? cgfd_stage_rows_batch_vti()
                                          : cgfd_stage_rows_batch_iso();
    if (rows_single != rows_batch)
      return set_err(CGFD_EINVAL, "batched stage kernel built with %d tile rows, the "
                     "single-shot kernel with %d", rows_batch, rows_single);
  }
  cgfd_batch_t *b = new cgfd_batch_t();
  b->n = nshot;
  b->nt_total = shots[0]->nt_total;
  b->med = medium_of(shots[0]->medium_type);
  b->kchunk = kchunk > 0 ? kchunk : 16;
  if (const char *e = getenv("CGFD_BATCH_GRAPH")) b->use_graph = atoi(e) != 0;
#define BTRY(x) do { int r_ = (x); if (r_) { cgfd_batch_destroy(b); return r_; } } while (0)
#define BTRYC(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { set_err(CGFD_ECUDA, "%s: %s", #x, cudaGetErrorString(e_)); cgfd_batch_destroy(b); return CGFD_ECUDA; } } while (0)
  BTRYC(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BTRYC(cudaEventCreate(&b->ev0));
  BTRYC(cudaEventCreate(&b->ev1));
  for (int k = 0; k < nshot; k++) {
    cgfd_solver_t *s = nullptr;
    int rc = cgfd_solver_create(shots[k], &s);
    if (rc) {
      std::string m = g_err;
      cgfd_batch_destroy(b);
      return set_err(rc, "shot %d: %s", k, m.c_str());
    }
    s->pml_fused = 1;
    s->kernel = 2;
    b->sv.push_back(s);
  }
  /* shared-memory attribute of every batched stage form (graph capture
   * must not be the first use) */
  const BatchSched none = {nullptr, 0, nullptr};
  for (int code = 0; code < 8; code++)
    for (int kind = 0; kind < 3; kind++) {
      if (b->med == MED_VTI) cgfd_launch_stage_batch_vti(code, kind, 0, b->stream, nullptr, nullptr, 0, none);
      else cgfd_launch_stage_batch_iso(code, kind, 0, b->stream, nullptr, nullptr, 0, none);
    }
  {
    /* one persistent CTA per SM (the stage kernel's shared memory allows no
     * more); CGFD_BATCH_PERSISTENT=1 makes it the schedule from the start */
    int dev = 0, nsm = 0;
    BTRYC(cudaGetDevice(&dev));
    BTRYC(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    b->pgrid = nsm;
    if (const char *e = getenv("CGFD_BATCH_PERSISTENT")) b->persistent = atoi(e) != 0;
  }
  BTRYC(cudaGetLastError());
  BTRY(batch_tables(b));
  *out = b;
  return 0;
#undef BTRY
#undef BTRYC
}

static void batch_enqueue_step(cgfd_batch_t *b, int it)
{
  const int n = b->n, ipair = it % 8, par = b->par;
  for (int is = 0; is < 4; is++) {
    int bx = (PAIR_FLAGS[ipair][0] + is) % 2;
    int by = (PAIR_FLAGS[ipair][1] + is) % 2;
    int bz = (PAIR_FLAGS[ipair][2] + is) % 2;
    int kind = is == 0 ? 0 : (is < 3 ? 1 : 2);
    int code = bx * 4 + by * 2 + bz;
    const StageArgs *args = b->d_args + (size_t)(par * 4 + is) * n;
    int grid = b->nctas;
    BatchSched w = {nullptr, b->nctas, nullptr};
    if (b->persistent) {
      const cudaError_t e = cudaMemsetAsync(b->d_next, 0, sizeof(int), b->stream);
      if (e != cudaSuccess && b->enq_err == cudaSuccess) b->enq_err = e;
      grid = std::min(b->pgrid, b->nctas);
      w.order = b->d_order;
      w.next = b->d_next;
    }
    if (b->med == MED_VTI)
      cgfd_launch_stage_batch_vti(code, kind, grid, b->stream, args, b->d_geo, n, w);
    else
      cgfd_launch_stage_batch_iso(code, kind, grid, b->stream, args, b->d_geo, n, w);
  }
  if (b->pg_any) {
    dim3 bl(32, 8), gr((b->max_ni + 31) / 32, (b->max_nj + 7) / 8, n);
    k_pg_batch<<<gr, bl, 0, b->stream>>>(b->d_pg + (size_t)par * n);
  }
  k_recv_batch<<<n, 256, 0, b->stream>>>(b->d_recv + (size_t)par * n);
  b->par ^= 1;
}

/* advance the per-shot bookkeeping of the solvers by nsteps */
static void batch_sync_solvers(cgfd_batch_t *b, int nsteps)
{
  for (cgfd_solver_t *s : b->sv) {
    s->step += nsteps;
    if (nsteps % 2) std::swap(s->pre_lev, s->end_lev);
  }
}

extern "C" int cgfd_batch_run(cgfd_batch_t *b, int nsteps)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  if (nsteps < 0 || b->step + nsteps > b->nt_total)
    return set_err(CGFD_EINVAL, "run(%d) past nt_total=%d (at step %d)", nsteps,
                   b->nt_total, b->step);
  CK(cudaEventRecord(b->ev0, b->stream));
  int it = b->step, end = b->step + nsteps;
  int launches = 0;
  const int per_step = 4 + (b->pg_any ? 1 : 0) + 1;
  /* whole 8-step pair cycles (starting at a multiple of 8) are replayed
   * from one CUDA graph; the steps before and after run eagerly */
  while (it < end) {
    if (!(b->use_graph && it % 8 == 0 && end - it >= 8)) {
      batch_enqueue_step(b, it++);
      launches += per_step;
      continue;
    }
    if (!b->graph || b->graph_par != b->par) {
      if (b->graph) cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
      const int par0 = b->par;
      cudaGraph_t gph = nullptr;
      CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      for (int m = 0; m < 8; m++) batch_enqueue_step(b, m);
      CK(cudaStreamEndCapture(b->stream, &gph));
      cudaError_t e = cudaGraphInstantiate(&b->graph, gph, 0);
      cudaGraphDestroy(gph);
      CK(e);
      b->graph_par = par0;
      b->par = par0;              /* capture recorded, nothing ran */
    }
    CK(cudaGraphLaunch(b->graph, b->stream));
    it += 8;
    launches += 8 * per_step;
  }
  CK(cudaGetLastError());
  {
    const cudaError_t e = b->enq_err;
    b->enq_err = cudaSuccess;
    CK(e);
  }
  CK(cudaEventRecord(b->ev1, b->stream));
  CK(cudaEventSynchronize(b->ev1));
  CK(cudaEventElapsedTime(&b->t_ms, b->ev0, b->ev1));
  b->launches = launches;
  batch_sync_solvers(b, nsteps);
  b->step = end;
  for (cgfd_solver_t *s : b->sv) {
    int herr = 0;
    CK(cudaMemcpy(&herr, s->d_err, 4, cudaMemcpyDeviceToHost));
    if (herr) return set_err(CGFD_ECUDA, "device wait timed out (code %d)", herr);
  }
  return 0;
}

extern "C" int cgfd_batch_times(const cgfd_batch_t *b, float *ms, int *launches)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  *ms = b->t_ms;
  *launches = b->launches;
  return 0;
}

extern "C" int cgfd_batch_fetch(cgfd_batch_t *b)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  for (cgfd_solver_t *s : b->sv) {
    int rc = cgfd_solver_fetch(s);
    if (rc) return rc;
  }
  return 0;
}

extern "C" int cgfd_batch_fetch_seismograms(cgfd_batch_t *b)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  for (cgfd_solver_t *s : b->sv) {
    int rc = cgfd_solver_fetch_seismograms(s);
    if (rc) return rc;
  }
  return 0;
}

extern "C" int cgfd_batch_reset(cgfd_batch_t *b)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  for (cgfd_solver_t *s : b->sv) {
    int rc = solver_reset(s);
    if (rc) return rc;
  }
  b->step = 0;
  b->par = 0;
  return 0;
}

extern "C" int cgfd_batch_set_kchunk(cgfd_batch_t *b, int kchunk)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  if (kchunk < 4 || kchunk > 4096) return set_err(CGFD_EINVAL, "kchunk %d out of 4..4096", kchunk);
  b->kchunk = kchunk;
  return batch_tables(b);
}

extern "C" int cgfd_batch_set_schedule(cgfd_batch_t *b, int persistent)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  b->persistent = persistent ? 1 : 0;
  if (b->graph) cudaGraphExecDestroy(b->graph);   /* captured with the old schedule */
  b->graph = nullptr;
  b->graph_par = -1;
  return 0;
}

extern "C" int cgfd_batch_schedule(const cgfd_batch_t *b) { return b ? b->persistent : -1; }

extern "C" int cgfd_batch_autotune_schedule(cgfd_batch_t *b, const int *cand, int ncand,
                                            int steps, float *ms_out, int *best_kchunk,
                                            int *best_persistent)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  if (!cand || ncand < 1 || steps < 1 || steps > b->nt_total || !best_kchunk ||
      !best_persistent)
    return set_err(CGFD_EINVAL, "autotune: bad candidates or steps");
  float tbest = 0.f;
  int kbest = b->kchunk, pbest = b->persistent, first = 1;
  for (int sch = 0; sch < 2; sch++)
    for (int c = 0; c < ncand; c++) {
      int rc = cgfd_batch_set_schedule(b, sch);
      if (!rc) rc = cgfd_batch_set_kchunk(b, cand[c]);
      if (!rc) rc = cgfd_batch_run(b, 1);         /* warm-up step */
      if (!rc) rc = cgfd_batch_run(b, steps < b->nt_total ? steps : b->nt_total - 1);
      if (rc) return rc;
      const float t = b->t_ms;
      if (ms_out) ms_out[sch * ncand + c] = t;
      if (first || t < tbest) { tbest = t; kbest = cand[c]; pbest = sch; first = 0; }
      rc = cgfd_batch_reset(b);
      if (rc) return rc;
    }
  *best_kchunk = kbest;
  *best_persistent = pbest;
  int rc = cgfd_batch_set_schedule(b, pbest);
  return rc ? rc : cgfd_batch_set_kchunk(b, kbest);
}

extern "C" int cgfd_batch_autotune(cgfd_batch_t *b, const int *cand, int ncand, int steps,
                                   float *ms_out, int *best)
{
  if (!b) return set_err(CGFD_EINVAL, "null batch");
  if (!cand || ncand < 1 || steps < 1 || steps > b->nt_total)
    return set_err(CGFD_EINVAL, "autotune: bad candidates or steps");
  float tbest = 0.f;
  int kbest = b->kchunk;
  for (int c = 0; c < ncand; c++) {
    int rc = cgfd_batch_set_kchunk(b, cand[c]);
    if (!rc) rc = cgfd_batch_run(b, 1);         /* warm-up step */
    if (!rc) rc = cgfd_batch_run(b, steps < b->nt_total ? steps : b->nt_total - 1);
    if (rc) return rc;
    float t = b->t_ms;
    if (ms_out) ms_out[c] = t;
    if (c == 0 || t < tbest) { tbest = t; kbest = cand[c]; }
    rc = cgfd_batch_reset(b);
    if (rc) return rc;
  }
  *best = kbest;
  return cgfd_batch_set_kchunk(b, kbest);
}

extern "C" cgfd_solver_t *cgfd_batch_shot(cgfd_batch_t *b, int k)
{
  if (!b || k < 0 || k >= b->n) return nullptr;
  return b->sv[k];
}

/* ------------------------------------------------------------------------ */
/* grid metrics on the device (forward/gd_t.c:190-402)                       */
/* ------------------------------------------------------------------------ */

extern "C" int cgfd_metric_calc(int nx, int ny, int nz, int ni1, int ni2, int nj1,
                                int nj2, int nk1, int nk2, const float *x3d,
                                const float *y3d, const float *z3d, float *metric)
{
  if (!x3d || !y3d || !z3d || !metric) return set_err(CGFD_EINVAL, "null array");
  if (ni1 != 3 || nj1 != 3 || nk1 != 3 || nx != ni2 + 4 || ny != nj2 + 4 ||
      nz != nk2 + 4 || ni2 < ni1 || nj2 < nj1 || nk2 < nk1)
    return set_err(CGFD_EINVAL, "grid indices are not the 3-ghost layout");
  cgfd_solver_t tmp{};
  cgfd_solver_t *s = &tmp;
  DevGrid &g = s->g;
  g.nx = nx; g.ny = ny; g.nz = nz;
  g.ni = ni2 - ni1 + 1; g.nj = nj2 - nj1 + 1; g.nk = nk2 - nk1 + 1;
  g.ni1 = ni1; g.ni2 = ni2; g.nj1 = nj1; g.nj2 = nj2; g.nk1 = nk1; g.nk2 = nk2;
  g.xoff = XOFF;
  g.px = pitch_for(g.ni);
  g.sl = (long long)g.px * ny;
  g.vol = g.sl * nz;
  CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  float *m = nullptr;
  int rc = 0;
  cudaError_t e = cudaMalloc((void **)&m, 10 * (size_t)g.vol * sizeof(float));
  if (e != cudaSuccess) rc = set_err(CGFD_ENOMEM, "cudaMalloc: %s", cudaGetErrorString(e));
  if (!rc) {
    e = cudaMemsetAsync(m, 0, 10 * (size_t)g.vol * sizeof(float), s->stream);
    if (e != cudaSuccess) rc = set_err(CGFD_ECUDA, "memset: %s", cudaGetErrorString(e));
  }
  if (!rc) rc = device_metrics(s, x3d, y3d, z3d, m);
  const size_t hvol = (size_t)nx * ny * nz;
  for (int c = 0; c < 10 && !rc; c++) {
    e = download_volume(s, metric + c * hvol, m + c * g.vol);
    if (e != cudaSuccess) rc = set_err(CGFD_ECUDA, "download: %s", cudaGetErrorString(e));
  }
  if (!rc) {
    e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) rc = set_err(CGFD_ECUDA, "sync: %s", cudaGetErrorString(e));
  }
  release_staging(s);
  if (m) cudaFree(m);
  cudaStreamDestroy(s->stream);
  return rc;
}
