/*
 * media_layer2model_gpu.cpp -- drop-in for CGFD3D's discretisation of
 * media on a curvilinear grid: elastic isotropic and elastic VTI layered
 * models, elastic isotropic 3-D grid models, and models given as binary
 * volumes.
 *
 * Built inside the reference tree (its media headers: inter_t,
 * read_interface_file) and linked with -Wl,--wrap= for
 * media_layer2model_el_iso, _el_vti, media_grid2model_el_iso and
 * media_bin2model_el_iso, _vis_iso,
 * so the reference's main (forward/main_curv_col_el_3d.c:328-515)
 * calls the __wrap_ functions below with its unchanged arguments.  A .md3lay
 * file is read by the reference's own reader (media/media_read_file.cpp:
 * 22-240), its arrays are interleaved into the record layout of
 * cgfd_media_layer_* (include/cgfd3d_gpu.h) and the device computes the
 * medium with the requested equivalent-medium method; of binary volumes only
 * the box the grid needs is read, as the reference reads only its crop
 * (cgfd_media_bin_crop; one fread per run of the files' fastest dimension
 * instead of one per sample), and interpolated on the device
 * (cgfd_media_bin_*_box).  Grids other than
 * curvilinear, methods other than loc/har/ari and other media types go to
 * the reference's routine (__real_...), which handles or rejects them as it
 * always did.  Errors print the library's message and exit(1), as the
 * reference does on bad input.
 */
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using std::fabs;   /* the reference's media headers call fabs unqualified */

#include "media_read_file.hpp"
#include "media_utility.hpp"

#include "../../../include/cgfd3d_gpu.h"

extern "C" int __real_media_layer2model_el_iso(float *lam3d, float *mu3d, float *rho3d,
                                               const float *x3d, const float *y3d,
                                               const float *z3d, size_t nx, size_t ny,
                                               size_t nz, int grid_type,
                                               const char *in_3lay_file,
                                               const char *equivalent_medium_method,
                                               int myid);

extern "C" int __real_media_layer2model_el_vti(float *rho, float *c11, float *c33,
                                               float *c55, float *c66, float *c13,
                                               const float *x3d, const float *y3d,
                                               const float *z3d, size_t nx, size_t ny,
                                               size_t nz, int grid_type,
                                               const char *in_3lay_file,
                                               const char *equivalent_medium_method,
                                               int myid);

/* the grid and method this library takes */
static bool lay_ours(int grid_type, const char *m, size_t nx, size_t ny, size_t nz)
{
  return grid_type == GRID_CURV && m &&
         (strcmp(m, "loc") == 0 || strcmp(m, "har") == 0 || strcmp(m, "ari") == 0) &&
         nx <= INT_MAX && ny <= INT_MAX && nz <= INT_MAX;
}

/* [interface][y][x][ncol]: the reader's arrays ([interface][y][x] each)
 * interleaved */
static std::vector<float> lay_interleave(const inter_t &it, const float *const *cols, int ncol)
{
  const size_t n = it.NI * it.NX * it.NY;
  std::vector<float> rec(n * ncol);
  for (size_t q = 0; q < n; q++)
    for (int c = 0; c < ncol; c++) rec[q * ncol + c] = cols[c][q];
  return rec;
}

static void lay_fail(const char *file)
{
  fprintf(stderr, "Error: %s (layered model %s)\n", cgfd_last_error(), file);
  fflush(stderr);
  exit(1);
}

extern "C" int __wrap_media_layer2model_el_iso(float *lam3d, float *mu3d, float *rho3d,
                                               const float *x3d, const float *y3d,
                                               const float *z3d, size_t nx, size_t ny,
                                               size_t nz, int grid_type,
                                               const char *in_3lay_file,
                                               const char *equivalent_medium_method,
                                               int myid)
{
  const char *m = equivalent_medium_method;
  if (!lay_ours(grid_type, m, nx, ny, nz))
    return __real_media_layer2model_el_iso(lam3d, mu3d, rho3d, x3d, y3d, z3d, nx, ny, nz,
                                           grid_type, in_3lay_file, m, myid);
  inter_t it;
  read_interface_file(in_3lay_file, &it);
  if (it.media_type != ELASTIC_ISOTROPIC)
    return __real_media_layer2model_el_iso(lam3d, mu3d, rho3d, x3d, y3d, z3d, nx, ny, nz,
                                           grid_type, in_3lay_file, m, myid);
  /* elevation, then value, gradient and power of rho, vp and vs */
  const float *cols[10] = {it.elevation, it.rho, it.rho_grad, it.rho_pow, it.vp,
                           it.vp_grad,   it.vp_pow, it.vs,     it.vs_grad, it.vs_pow};
  const std::vector<float> rec = lay_interleave(it, cols, 10);
  if (!cgfd_media_layer_pow_ok(10, rec.data(), it.NI * it.NX * it.NY))
    return __real_media_layer2model_el_iso(lam3d, mu3d, rho3d, x3d, y3d, z3d, nx, ny, nz,
                                           grid_type, in_3lay_file, m, myid);
  if (myid == 0)
    fprintf(stdout, "discretising the layered model on the GPU (method %s)\n", m);
  const int rc = cgfd_media_layer_el_iso((int)it.NI, (int)it.NX, (int)it.NY, it.MINX, it.MINY,
                                         it.DX, it.DY, rec.data(), (int)nx, (int)ny, (int)nz,
                                         x3d, y3d, z3d, m, lam3d, mu3d, rho3d);
  if (rc != 0) lay_fail(in_3lay_file);
  return 0;
}

extern "C" int __wrap_media_layer2model_el_vti(float *rho, float *c11, float *c33, float *c55,
                                               float *c66, float *c13, const float *x3d,
                                               const float *y3d, const float *z3d, size_t nx,
                                               size_t ny, size_t nz, int grid_type,
                                               const char *in_3lay_file,
                                               const char *equivalent_medium_method,
                                               int myid)
{
  const char *m = equivalent_medium_method;
  if (!lay_ours(grid_type, m, nx, ny, nz))
    return __real_media_layer2model_el_vti(rho, c11, c33, c55, c66, c13, x3d, y3d, z3d, nx, ny,
                                           nz, grid_type, in_3lay_file, m, myid);
  inter_t it;
  read_interface_file(in_3lay_file, &it);
  /* elevation, then value, gradient and power of the six parameters */
  const float *cols[19];
  cols[0] = it.elevation;
  const float *p[18];
  if (it.media_type == ELASTIC_VTI_PREM) {
    const float *q[18] = {it.rho, it.rho_grad, it.rho_pow, it.vph, it.vph_grad, it.vph_pow,
                          it.vpv, it.vpv_grad, it.vpv_pow, it.vsh, it.vsh_grad, it.vsh_pow,
                          it.vsv, it.vsv_grad, it.vsv_pow, it.eta, it.eta_grad, it.eta_pow};
    memcpy(p, q, sizeof p);
  } else if (it.media_type == ELASTIC_VTI_THOMSEN) {
    const float *q[18] = {it.rho,     it.rho_grad,     it.rho_pow,     it.vp0,
                          it.vp0_grad, it.vp0_pow,     it.vs0,         it.vs0_grad,
                          it.vs0_pow, it.epsilon,      it.epsilon_grad, it.epsilon_pow,
                          it.delta,   it.delta_grad,   it.delta_pow,   it.gamma,
                          it.gamma_grad, it.gamma_pow};
    memcpy(p, q, sizeof p);
  } else if (it.media_type == ELASTIC_VTI_CIJ) {
    const float *q[18] = {it.rho, it.rho_grad, it.rho_pow, it.c11, it.c11_grad, it.c11_pow,
                          it.c33, it.c33_grad, it.c33_pow, it.c55, it.c55_grad, it.c55_pow,
                          it.c66, it.c66_grad, it.c66_pow, it.c13, it.c13_grad, it.c13_pow};
    memcpy(p, q, sizeof p);
  } else {
    return __real_media_layer2model_el_vti(rho, c11, c33, c55, c66, c13, x3d, y3d, z3d, nx, ny,
                                           nz, grid_type, in_3lay_file, m, myid);
  }
  for (int c = 0; c < 18; c++) cols[1 + c] = p[c];
  const std::vector<float> rec = lay_interleave(it, cols, 19);
  if (!cgfd_media_layer_pow_ok(19, rec.data(), it.NI * it.NX * it.NY))
    return __real_media_layer2model_el_vti(rho, c11, c33, c55, c66, c13, x3d, y3d, z3d, nx, ny,
                                           nz, grid_type, in_3lay_file, m, myid);
  if (myid == 0)
    fprintf(stdout, "discretising the layered model on the GPU (method %s)\n", m);
  const int rc = cgfd_media_layer_el_vti(it.media_type, (int)it.NI, (int)it.NX, (int)it.NY,
                                         it.MINX, it.MINY, it.DX, it.DY, rec.data(), (int)nx,
                                         (int)ny, (int)nz, x3d, y3d, z3d, m, c11, c33, c55, c66,
                                         c13, rho);
  if (rc != 0) lay_fail(in_3lay_file);
  return 0;
}

/* the box of a binary volume (file order, count[0] x count[1] x count[2]
 * floats), one read per run of the files' fastest dimension */
static std::vector<float> bin_read_box(const char *file, const int *size,
                                       const cgfd_bin_box_t &box)
{
  const size_t run = (size_t)box.count[0];
  std::vector<float> v(run * box.count[1] * box.count[2]);
  FILE *fp = fopen(file, "rb");
  bool ok = fp != nullptr;
  for (int c2 = 0; ok && c2 < box.count[2]; c2++)
    for (int c1 = 0; ok && c1 < box.count[1]; c1++) {
      const long long off = (((long long)(box.first[2] + c2) * size[1] + box.first[1] + c1) *
                                 size[0] + box.first[0]) * (long long)sizeof(float);
      ok = fseeko(fp, (off_t)off, SEEK_SET) == 0 &&
           fread(v.data() + ((size_t)c2 * box.count[1] + c1) * run, sizeof(float), run, fp) ==
               run;
    }
  if (!ok) {
    fprintf(stderr, "Error: Insufficient data in %s.\n", file);
    fflush(stderr);
    exit(1);
  }
  fclose(fp);
  return v;
}

static cgfd_bin_model_t bin_layout(const int *order, const int *size, const float *spacing,
                                   const float *origin)
{
  cgfd_bin_model_t m;
  for (int d = 0; d < 3; d++) {
    m.order[d] = order[d];
    m.size[d] = size[d];
    m.spacing[d] = spacing[d];
    m.origin[d] = origin[d];
  }
  return m;
}

extern "C" int __real_media_bin2model_el_iso(float *rho3d, float *lam3d, float *mu3d,
                                             const float *x3d, const float *y3d,
                                             const float *z3d, size_t nx, size_t ny, size_t nz,
                                             float xmin, float xmax, float ymin, float ymax,
                                             int grid_type, int *bin_order, int *bin_size,
                                             float *bin_spacing, float *bin_origin,
                                             const char *bin_file_rho, const char *bin_file_vp,
                                             const char *bin_file_vs);

extern "C" int __wrap_media_bin2model_el_iso(float *rho3d, float *lam3d, float *mu3d,
                                             const float *x3d, const float *y3d,
                                             const float *z3d, size_t nx, size_t ny, size_t nz,
                                             float xmin, float xmax, float ymin, float ymax,
                                             int grid_type, int *bin_order, int *bin_size,
                                             float *bin_spacing, float *bin_origin,
                                             const char *bin_file_rho, const char *bin_file_vp,
                                             const char *bin_file_vs)
{
  if (grid_type != GRID_CURV || nx > INT_MAX || ny > INT_MAX || nz > INT_MAX ||
      bin_size[0] < 1 || bin_size[1] < 1 || bin_size[2] < 1)
    return __real_media_bin2model_el_iso(rho3d, lam3d, mu3d, x3d, y3d, z3d, nx, ny, nz, xmin,
                                         xmax, ymin, ymax, grid_type, bin_order, bin_size,
                                         bin_spacing, bin_origin, bin_file_rho, bin_file_vp,
                                         bin_file_vs);
  const cgfd_bin_model_t m = bin_layout(bin_order, bin_size, bin_spacing, bin_origin);
  cgfd_bin_box_t box;
  if (cgfd_media_bin_crop(&m, xmin, xmax, ymin, ymax, (int)nx, (int)ny, (int)nz, z3d, &box))
    lay_fail(bin_file_rho);
  fprintf(stdout, "- reading model files %s, %s, %s\n", bin_file_rho, bin_file_vp, bin_file_vs);
  const std::vector<float> rho = bin_read_box(bin_file_rho, bin_size, box),
                           vp = bin_read_box(bin_file_vp, bin_size, box),
                           vs = bin_read_box(bin_file_vs, bin_size, box);
  fprintf(stdout, "discretising the binary model on the GPU\n");
  if (cgfd_media_bin_el_iso_box(&m, &box, xmin, xmax, ymin, ymax, rho.data(), vp.data(),
                                vs.data(), (int)nx, (int)ny, (int)nz, x3d, y3d, z3d, rho3d,
                                lam3d, mu3d))
    lay_fail(bin_file_rho);
  return 0;
}

extern "C" int __real_media_bin2model_vis_iso(float *Qp3d, float *Qs3d, const float *x3d,
                                              const float *y3d, const float *z3d, size_t nx,
                                              size_t ny, size_t nz, float xmin, float xmax,
                                              float ymin, float ymax, int grid_type,
                                              int *bin_order, int *bin_size, float *bin_spacing,
                                              float *bin_origin, const char *bin_file_Qp,
                                              const char *bin_file_Qs);

extern "C" int __wrap_media_bin2model_vis_iso(float *Qp3d, float *Qs3d, const float *x3d,
                                              const float *y3d, const float *z3d, size_t nx,
                                              size_t ny, size_t nz, float xmin, float xmax,
                                              float ymin, float ymax, int grid_type,
                                              int *bin_order, int *bin_size, float *bin_spacing,
                                              float *bin_origin, const char *bin_file_Qp,
                                              const char *bin_file_Qs)
{
  if (grid_type != GRID_CURV || nx > INT_MAX || ny > INT_MAX || nz > INT_MAX ||
      bin_size[0] < 1 || bin_size[1] < 1 || bin_size[2] < 1)
    return __real_media_bin2model_vis_iso(Qp3d, Qs3d, x3d, y3d, z3d, nx, ny, nz, xmin, xmax,
                                          ymin, ymax, grid_type, bin_order, bin_size,
                                          bin_spacing, bin_origin, bin_file_Qp, bin_file_Qs);
  const cgfd_bin_model_t m = bin_layout(bin_order, bin_size, bin_spacing, bin_origin);
  cgfd_bin_box_t box;
  if (cgfd_media_bin_crop(&m, xmin, xmax, ymin, ymax, (int)nx, (int)ny, (int)nz, z3d, &box))
    lay_fail(bin_file_Qp);
  fprintf(stdout, "- reading model files %s, %s\n", bin_file_Qp, bin_file_Qs);
  const std::vector<float> qp = bin_read_box(bin_file_Qp, bin_size, box),
                           qs = bin_read_box(bin_file_Qs, bin_size, box);
  fprintf(stdout, "discretising the binary model on the GPU\n");
  if (cgfd_media_bin_vis_iso_box(&m, &box, xmin, xmax, ymin, ymax, qp.data(), qs.data(),
                                 (int)nx, (int)ny, (int)nz, x3d, y3d, z3d, Qp3d, Qs3d))
    lay_fail(bin_file_Qp);
  return 0;
}

extern "C" int __real_media_grid2model_el_iso(float *rho3d, float *lam3d, float *mu3d,
                                              const float *x3d, const float *y3d,
                                              const float *z3d, int nx, int ny, int nz,
                                              float Xmin, float Xmax, float Ymin, float Ymax,
                                              int grid_type, const char *in_media_file,
                                              const char *equivalent_medium_method, int myid);

/* a .md3grd model: read (and cropped to the grid's extent) by the reference's
 * reader, discretised on the device */
extern "C" int __wrap_media_grid2model_el_iso(float *rho3d, float *lam3d, float *mu3d,
                                              const float *x3d, const float *y3d,
                                              const float *z3d, int nx, int ny, int nz,
                                              float Xmin, float Xmax, float Ymin, float Ymax,
                                              int grid_type, const char *in_media_file,
                                              const char *equivalent_medium_method, int myid)
{
  const char *m = equivalent_medium_method;
  /* the library takes grid models with "loc" only */
  if (!lay_ours(grid_type, m, nx, ny, nz) || strcmp(m, "loc") != 0)
    return __real_media_grid2model_el_iso(rho3d, lam3d, mu3d, x3d, y3d, z3d, nx, ny, nz, Xmin,
                                          Xmax, Ymin, Ymax, grid_type, in_media_file, m, myid);
  int NL = 0;
  std::vector<int> NGz;
  inter_t it;
  read_grid_file(in_media_file, Xmin, Xmax, Ymin, Ymax, NL, NGz, &it);
  if (it.media_type != ELASTIC_ISOTROPIC)
    return __real_media_grid2model_el_iso(rho3d, lam3d, mu3d, x3d, y3d, z3d, nx, ny, nz, Xmin,
                                          Xmax, Ymin, Ymax, grid_type, in_media_file, m, myid);
  const float *cols[4] = {it.elevation, it.rho, it.vp, it.vs};
  const std::vector<float> rec = lay_interleave(it, cols, 4);
  if (myid == 0)
    fprintf(stdout, "discretising the grid model on the GPU (method %s)\n", m);
  if (cgfd_media_grid_el_iso((int)it.NI, NL, NGz.data(), (int)it.NX, (int)it.NY, it.MINX,
                             it.MINY, it.DX, it.DY, rec.data(), nx, ny, nz, x3d, y3d, z3d, m,
                             rho3d, lam3d, mu3d))
    lay_fail(in_media_file);
  return 0;
}

extern "C" int __real_media_grid2model_el_vti(float *rho, float *c11, float *c33, float *c55,
                                              float *c66, float *c13, const float *x3d,
                                              const float *y3d, const float *z3d, int nx, int ny,
                                              int nz, float Xmin, float Xmax, float Ymin,
                                              float Ymax, int grid_type,
                                              const char *in_media_file,
                                              const char *equivalent_medium_method, int myid);

extern "C" int __wrap_media_grid2model_el_vti(float *rho, float *c11, float *c33, float *c55,
                                              float *c66, float *c13, const float *x3d,
                                              const float *y3d, const float *z3d, int nx, int ny,
                                              int nz, float Xmin, float Xmax, float Ymin,
                                              float Ymax, int grid_type,
                                              const char *in_media_file,
                                              const char *equivalent_medium_method, int myid)
{
  const char *m = equivalent_medium_method;
  if (!lay_ours(grid_type, m, nx, ny, nz) || strcmp(m, "loc") != 0)
    return __real_media_grid2model_el_vti(rho, c11, c33, c55, c66, c13, x3d, y3d, z3d, nx, ny,
                                          nz, Xmin, Xmax, Ymin, Ymax, grid_type, in_media_file,
                                          m, myid);
  int NL = 0;
  std::vector<int> NGz;
  inter_t it;
  read_grid_file(in_media_file, Xmin, Xmax, Ymin, Ymax, NL, NGz, &it);
  const float *cols[7] = {it.elevation};
  if (it.media_type == ELASTIC_VTI_PREM) {
    const float *q[6] = {it.rho, it.vph, it.vpv, it.vsh, it.vsv, it.eta};
    for (int c = 0; c < 6; c++) cols[1 + c] = q[c];
  } else if (it.media_type == ELASTIC_VTI_THOMSEN) {
    const float *q[6] = {it.rho, it.vp0, it.vs0, it.epsilon, it.delta, it.gamma};
    for (int c = 0; c < 6; c++) cols[1 + c] = q[c];
  } else if (it.media_type == ELASTIC_VTI_CIJ) {
    const float *q[6] = {it.rho, it.c11, it.c33, it.c55, it.c66, it.c13};
    for (int c = 0; c < 6; c++) cols[1 + c] = q[c];
  } else {
    return __real_media_grid2model_el_vti(rho, c11, c33, c55, c66, c13, x3d, y3d, z3d, nx, ny,
                                          nz, Xmin, Xmax, Ymin, Ymax, grid_type, in_media_file,
                                          m, myid);
  }
  const std::vector<float> rec = lay_interleave(it, cols, 7);
  if (myid == 0)
    fprintf(stdout, "discretising the grid model on the GPU (method %s)\n", m);
  if (cgfd_media_grid_el_vti(it.media_type, (int)it.NI, NL, NGz.data(), (int)it.NX, (int)it.NY,
                             it.MINX, it.MINY, it.DX, it.DY, rec.data(), nx, ny, nz, x3d, y3d,
                             z3d, m, c11, c33, c55, c66, c13, rho))
    lay_fail(in_media_file);
  return 0;
}

extern "C" int __real_media_layer2model_el_aniso(
    float *rho, float *c11, float *c12, float *c13, float *c14, float *c15, float *c16,
    float *c22, float *c23, float *c24, float *c25, float *c26, float *c33, float *c34, float *c35,
    float *c36, float *c44, float *c45, float *c46, float *c55, float *c56, float *c66,
    const float *x3d, const float *y3d, const float *z3d, size_t nx, size_t ny, size_t nz,
    int grid_type, const char *in_3lay_file, const char *equivalent_medium_method, int myid);

/* media_layer2model_el_aniso for elastic isotropic and VTI layered models
 * (media/media_layer2model.cpp:249-375): the same discretisation on the
 * device, then the reference's spreading into the 21 constants, in its
 * float/double order.  TTI and full-anisotropy models and the "tti" method
 * stay with the reference's routine. */
extern "C" int __wrap_media_layer2model_el_aniso(
    float *rho, float *c11, float *c12, float *c13, float *c14, float *c15, float *c16,
    float *c22, float *c23, float *c24, float *c25, float *c26, float *c33, float *c34, float *c35,
    float *c36, float *c44, float *c45, float *c46, float *c55, float *c56, float *c66,
    const float *x3d, const float *y3d, const float *z3d, size_t nx, size_t ny, size_t nz,
    int grid_type, const char *in_3lay_file, const char *equivalent_medium_method, int myid)
{
  const char *m = equivalent_medium_method;
  if (!lay_ours(grid_type, m, nx, ny, nz))
    return __real_media_layer2model_el_aniso(rho, c11, c12, c13, c14, c15, c16, c22, c23, c24,
                                             c25, c26, c33, c34, c35, c36, c44, c45, c46, c55,
                                             c56, c66, x3d, y3d, z3d, nx, ny, nz, grid_type,
                                             in_3lay_file, m, myid);
  inter_t it;
  read_interface_file(in_3lay_file, &it);
  const int t = it.media_type;
  const size_t vol = nx * ny * nz;
  int rc = -1;
  if (t == ELASTIC_ISOTROPIC) {
    const float *cols[10] = {it.elevation, it.rho, it.rho_grad, it.rho_pow, it.vp,
                             it.vp_grad,   it.vp_pow, it.vs,     it.vs_grad, it.vs_pow};
    const std::vector<float> rec = lay_interleave(it, cols, 10);
    if (cgfd_media_layer_pow_ok(10, rec.data(), it.NI * it.NX * it.NY)) {
      if (myid == 0)
        fprintf(stdout, "discretising the layered model on the GPU (method %s)\n", m);
      /* lambda into c13, mu into c44, as the reference's isotropic branch */
      rc = cgfd_media_layer_el_iso((int)it.NI, (int)it.NX, (int)it.NY, it.MINX, it.MINY, it.DX,
                                   it.DY, rec.data(), (int)nx, (int)ny, (int)nz, x3d, y3d, z3d,
                                   m, c13, c44, rho);
      if (rc != 0) lay_fail(in_3lay_file);
      for (size_t i = 0; i < vol; ++i) {
        c11[i] = c13[i] + 2.0 * c44[i];
        c22[i] = c11[i]; c33[i] = c11[i];
        c12[i] = c13[i]; c23[i] = c13[i];
        c55[i] = c44[i]; c66[i] = c44[i];
      }
    }
  } else if (t == ELASTIC_VTI_PREM || t == ELASTIC_VTI_THOMSEN || t == ELASTIC_VTI_CIJ) {
    const float *cols[19] = {it.elevation};
    const float *p[18];
    if (t == ELASTIC_VTI_PREM) {
      const float *q[18] = {it.rho, it.rho_grad, it.rho_pow, it.vph, it.vph_grad, it.vph_pow,
                            it.vpv, it.vpv_grad, it.vpv_pow, it.vsh, it.vsh_grad, it.vsh_pow,
                            it.vsv, it.vsv_grad, it.vsv_pow, it.eta, it.eta_grad, it.eta_pow};
      memcpy(p, q, sizeof p);
    } else if (t == ELASTIC_VTI_THOMSEN) {
      const float *q[18] = {it.rho,     it.rho_grad,     it.rho_pow,     it.vp0,
                            it.vp0_grad, it.vp0_pow,     it.vs0,         it.vs0_grad,
                            it.vs0_pow, it.epsilon,      it.epsilon_grad, it.epsilon_pow,
                            it.delta,   it.delta_grad,   it.delta_pow,   it.gamma,
                            it.gamma_grad, it.gamma_pow};
      memcpy(p, q, sizeof p);
    } else {
      const float *q[18] = {it.rho, it.rho_grad, it.rho_pow, it.c11, it.c11_grad, it.c11_pow,
                            it.c33, it.c33_grad, it.c33_pow, it.c55, it.c55_grad, it.c55_pow,
                            it.c66, it.c66_grad, it.c66_pow, it.c13, it.c13_grad, it.c13_pow};
      memcpy(p, q, sizeof p);
    }
    for (int c = 0; c < 18; c++) cols[1 + c] = p[c];
    const std::vector<float> rec = lay_interleave(it, cols, 19);
    if (cgfd_media_layer_pow_ok(19, rec.data(), it.NI * it.NX * it.NY)) {
      if (myid == 0)
        fprintf(stdout, "discretising the layered model on the GPU (method %s)\n", m);
      rc = cgfd_media_layer_el_vti(t, (int)it.NI, (int)it.NX, (int)it.NY, it.MINX, it.MINY,
                                   it.DX, it.DY, rec.data(), (int)nx, (int)ny, (int)nz, x3d,
                                   y3d, z3d, m, c11, c33, c55, c66, c13, rho);
      if (rc != 0) lay_fail(in_3lay_file);
      for (size_t i = 0; i < vol; i++) {
        c12[i] = c11[i] - 2.0 * c66[i];
        c22[i] = c11[i];
        c23[i] = c13[i];
        c44[i] = c55[i];
      }
    }
  }
  if (rc != 0)
    return __real_media_layer2model_el_aniso(rho, c11, c12, c13, c14, c15, c16, c22, c23, c24,
                                             c25, c26, c33, c34, c35, c36, c44, c45, c46, c55,
                                             c56, c66, x3d, y3d, z3d, nx, ny, nz, grid_type,
                                             in_3lay_file, m, myid);
  float *zero[12] = {c14, c24, c34, c15, c25, c35, c16, c26, c36, c45, c46, c56};
  for (int n = 0; n < 12; n++)
    for (size_t i = 0; i < vol; i++) zero[n][i] = 0.0;
  return 0;
}

extern "C" int __real_media_grid2model_el_aniso(
    float *rho, float *c11, float *c12, float *c13, float *c14, float *c15, float *c16,
    float *c22, float *c23, float *c24, float *c25, float *c26, float *c33, float *c34, float *c35,
    float *c36, float *c44, float *c45, float *c46, float *c55, float *c56, float *c66,
    const float *x3d, const float *y3d, const float *z3d, int nx, int ny, int nz, float Xmin,
    float Xmax, float Ymin, float Ymax, int grid_type, const char *in_media_file,
    const char *equivalent_medium_method, int myid);

/* media_grid2model_el_aniso for elastic isotropic and VTI grid models with
 * "loc" (media/media_grid2model.cpp:250-395): the device discretisation,
 * then the reference's spreading into the 21 constants. */
extern "C" int __wrap_media_grid2model_el_aniso(
    float *rho, float *c11, float *c12, float *c13, float *c14, float *c15, float *c16,
    float *c22, float *c23, float *c24, float *c25, float *c26, float *c33, float *c34, float *c35,
    float *c36, float *c44, float *c45, float *c46, float *c55, float *c56, float *c66,
    const float *x3d, const float *y3d, const float *z3d, int nx, int ny, int nz, float Xmin,
    float Xmax, float Ymin, float Ymax, int grid_type, const char *in_media_file,
    const char *equivalent_medium_method, int myid)
{
  const char *m = equivalent_medium_method;
  if (!lay_ours(grid_type, m, nx, ny, nz) || strcmp(m, "loc") != 0)
    return __real_media_grid2model_el_aniso(rho, c11, c12, c13, c14, c15, c16, c22, c23, c24,
                                            c25, c26, c33, c34, c35, c36, c44, c45, c46, c55,
                                            c56, c66, x3d, y3d, z3d, nx, ny, nz, Xmin, Xmax,
                                            Ymin, Ymax, grid_type, in_media_file, m, myid);
  int NL = 0;
  std::vector<int> NGz;
  inter_t it;
  read_grid_file(in_media_file, Xmin, Xmax, Ymin, Ymax, NL, NGz, &it);
  const int t = it.media_type;
  const size_t vol = (size_t)nx * ny * nz;
  if (t == ELASTIC_ISOTROPIC) {
    const float *cols[4] = {it.elevation, it.rho, it.vp, it.vs};
    const std::vector<float> rec = lay_interleave(it, cols, 4);
    if (myid == 0) fprintf(stdout, "discretising the grid model on the GPU (method %s)\n", m);
    /* lambda into c13, mu into c44, as the reference's isotropic branch */
    if (cgfd_media_grid_el_iso((int)it.NI, NL, NGz.data(), (int)it.NX, (int)it.NY, it.MINX,
                               it.MINY, it.DX, it.DY, rec.data(), nx, ny, nz, x3d, y3d, z3d, m,
                               rho, c13, c44))
      lay_fail(in_media_file);
    for (size_t i = 0; i < vol; ++i) {
      c11[i] = c13[i] + 2.0 * c44[i];
      c22[i] = c11[i]; c33[i] = c11[i];
      c12[i] = c13[i]; c23[i] = c13[i];
      c55[i] = c44[i]; c66[i] = c44[i];
    }
  } else if (t == ELASTIC_VTI_PREM || t == ELASTIC_VTI_THOMSEN || t == ELASTIC_VTI_CIJ) {
    const float *cols[7] = {it.elevation};
    const float *q[3][6] = {{it.rho, it.vph, it.vpv, it.vsh, it.vsv, it.eta},
                            {it.rho, it.vp0, it.vs0, it.epsilon, it.delta, it.gamma},
                            {it.rho, it.c11, it.c33, it.c55, it.c66, it.c13}};
    const int k = t == ELASTIC_VTI_PREM ? 0 : t == ELASTIC_VTI_THOMSEN ? 1 : 2;
    for (int c = 0; c < 6; c++) cols[1 + c] = q[k][c];
    const std::vector<float> rec = lay_interleave(it, cols, 7);
    if (myid == 0) fprintf(stdout, "discretising the grid model on the GPU (method %s)\n", m);
    if (cgfd_media_grid_el_vti(t, (int)it.NI, NL, NGz.data(), (int)it.NX, (int)it.NY, it.MINX,
                               it.MINY, it.DX, it.DY, rec.data(), nx, ny, nz, x3d, y3d, z3d, m,
                               c11, c33, c55, c66, c13, rho))
      lay_fail(in_media_file);
    for (size_t i = 0; i < vol; i++) {
      c12[i] = c11[i] - 2.0 * c66[i];
      c22[i] = c11[i];
      c23[i] = c13[i];
      c44[i] = c55[i];
    }
  } else {
    return __real_media_grid2model_el_aniso(rho, c11, c12, c13, c14, c15, c16, c22, c23, c24,
                                            c25, c26, c33, c34, c35, c36, c44, c45, c46, c55,
                                            c56, c66, x3d, y3d, z3d, nx, ny, nz, Xmin, Xmax,
                                            Ymin, Ymax, grid_type, in_media_file, m, myid);
  }
  float *zero[12] = {c14, c24, c34, c15, c25, c35, c16, c26, c36, c45, c46, c56};
  for (int n = 0; n < 12; n++)
    for (size_t i = 0; i < vol; i++) zero[n][i] = 0.0;
  return 0;
}
