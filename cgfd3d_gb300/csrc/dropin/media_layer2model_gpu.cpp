/*
 * media_layer2model_gpu.cpp -- drop-in for CGFD3D's discretisation of
 * elastic isotropic layered models on a curvilinear grid.
 *
 * Built inside the reference tree (its media headers: inter_t,
 * read_interface_file) and linked with -Wl,--wrap=media_layer2model_el_iso,
 * so the reference's main (forward/main_curv_col_el_3d.c:328-334) calls
 * __wrap_media_layer2model_el_iso below with its unchanged arguments.  The
 * .md3lay file is read by the reference's own reader
 * (media/media_read_file.cpp:22-240), its arrays are interleaved into the
 * record layout of cgfd_media_layer_el_iso (include/cgfd3d_gpu.h) and the
 * device computes lambda, mu, rho with the requested equivalent-medium
 * method.  Grids other than curvilinear, methods other than loc/har/ari and
 * media other than elastic isotropic go to the reference's routine
 * (__real_media_layer2model_el_iso), which handles or rejects them as it
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

extern "C" int __wrap_media_layer2model_el_iso(float *lam3d, float *mu3d, float *rho3d,
                                               const float *x3d, const float *y3d,
                                               const float *z3d, size_t nx, size_t ny,
                                               size_t nz, int grid_type,
                                               const char *in_3lay_file,
                                               const char *equivalent_medium_method,
                                               int myid)
{
  const char *m = equivalent_medium_method;
  const bool ours = grid_type == GRID_CURV && m &&
                    (strcmp(m, "loc") == 0 || strcmp(m, "har") == 0 || strcmp(m, "ari") == 0) &&
                    nx <= INT_MAX && ny <= INT_MAX && nz <= INT_MAX;
  if (!ours)
    return __real_media_layer2model_el_iso(lam3d, mu3d, rho3d, x3d, y3d, z3d, nx, ny, nz,
                                           grid_type, in_3lay_file, m, myid);
  inter_t it;
  read_interface_file(in_3lay_file, &it);
  if (it.media_type != ELASTIC_ISOTROPIC)
    return __real_media_layer2model_el_iso(lam3d, mu3d, rho3d, x3d, y3d, z3d, nx, ny, nz,
                                           grid_type, in_3lay_file, m, myid);
  /* [interface][y][x][10]: elevation, then value, gradient and power of rho,
   * vp and vs (the reader's arrays are [interface][y][x] each) */
  const size_t n = it.NI * it.NX * it.NY;
  const float *cols[10] = {it.elevation, it.rho, it.rho_grad, it.rho_pow, it.vp,
                           it.vp_grad,   it.vp_pow, it.vs,     it.vs_grad, it.vs_pow};
  std::vector<float> rec(n * 10);
  for (size_t q = 0; q < n; q++)
    for (int c = 0; c < 10; c++) rec[q * 10 + c] = cols[c][q];
  if (myid == 0)
    fprintf(stdout, "discretising the layered model on the GPU (method %s)\n", m);
  const int rc = cgfd_media_layer_el_iso((int)it.NI, (int)it.NX, (int)it.NY, it.MINX, it.MINY,
                                         it.DX, it.DY, rec.data(), (int)nx, (int)ny, (int)nz,
                                         x3d, y3d, z3d, m, lam3d, mu3d, rho3d);
  if (rc != 0) {
    fprintf(stderr, "Error: %s (layered model %s)\n", cgfd_last_error(), in_3lay_file);
    fflush(stderr);
    exit(1);
  }
  return 0;
}
