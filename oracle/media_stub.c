/*
 * media_stub.c -- TEST INFRASTRUCTURE ONLY.  Stands in for the CUDA
 * library's cgfd_media_layer_el_iso, _el_vti and cgfd_media_bin_*
 * (include/cgfd3d_gpu.h) in a CPU-only
 * link of the reference with the media drop-in adapter
 * (cgfd3d_gb300/csrc/dropin/media_layer2model_gpu.cpp), so a test can run
 * the adapter inside the reference's own process and check what it hands
 * over: the values come from the oracle's restatement, which equals the
 * reference bit for bit.  Linked only into oracle/_ref/ref_probe_media
 * (oracle/Makefile); nothing of the product links it.
 */
#include <string.h>

#include "cgfd3d_gpu.h"

int oracle_layer(int kind, int method, int NI, int NX, int NY, float MINX, float MINY,
                 float DX, float DY, const float *rec, int nx, int ny, int nz,
                 const float *x3d, const float *y3d, const float *z3d, float **out);

static const char *stub_msg = "";

int cgfd_media_layer_pow_ok(int nc, const float *rec, size_t nrec)
{
  (void)nc; (void)rec; (void)nrec;
  return 1;
}

static int stub_method(const char *method)
{
  return !method ? -1 : !strcmp(method, "loc") ? 0 : !strcmp(method, "har") ? 1
       : !strcmp(method, "ari") ? 2 : -1;
}

static int stub_run(int kind, int NI, int NX, int NY, float MINX, float MINY, float DX, float DY,
                    const float *rec, int nx, int ny, int nz, const float *x3d,
                    const float *y3d, const float *z3d, const char *method, float **out)
{
  int m = stub_method(method);
  if (m < 0) {
    stub_msg = "layered model: unknown equivalent medium method";
    return CGFD_EINVAL;
  }
  if (oracle_layer(kind, m, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d, z3d,
                   out)) {
    stub_msg = "layered model: a point outside the mesh or vp <= sqrt(2) vs";
    return CGFD_EINVAL;
  }
  return 0;
}

int cgfd_media_layer_el_iso(int NI, int NX, int NY, float MINX, float MINY, float DX,
                            float DY, const float *rec, int nx, int ny, int nz,
                            const float *x3d, const float *y3d, const float *z3d,
                            const char *method, float *lam, float *mu, float *rho)
{
  float *out[3] = {lam, mu, rho};
  return stub_run(21, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d, z3d, method,
                  out);
}

int cgfd_media_layer_el_vti(int media_type, int NI, int NX, int NY, float MINX, float MINY,
                            float DX, float DY, const float *rec, int nx, int ny, int nz,
                            const float *x3d, const float *y3d, const float *z3d,
                            const char *method, float *c11, float *c33, float *c55,
                            float *c66, float *c13, float *rho)
{
  float *out[6] = {c11, c33, c55, c66, c13, rho};
  return stub_run(media_type, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d, z3d,
                  method, out);
}

const char *cgfd_last_error(void) { return stub_msg; }


int oracle_bin(int vis, const int *order, const int *size, const float *spacing,
               const float *origin, const float *ext, const float *const *vols, int nx, int ny,
               int nz, const float *x3d, const float *y3d, const float *z3d, float **out);

static int stub_bin(int vis, const cgfd_bin_model_t *m, float xmin, float xmax, float ymin,
                    float ymax, const float *const *v, int nx, int ny, int nz,
                    const float *x3d, const float *y3d, const float *z3d, float **o)
{
  const float ext[4] = {xmin, xmax, ymin, ymax};
  if (oracle_bin(vis, m->order, m->size, m->spacing, m->origin, ext, v, nx, ny, nz, x3d, y3d,
                 z3d, o)) {
    stub_msg = "binary model: the model does not cover the grid";
    return CGFD_EINVAL;
  }
  return 0;
}

int cgfd_media_bin_el_iso(const cgfd_bin_model_t *model, float xmin, float xmax, float ymin,
                          float ymax, const float *rho_vol, const float *vp_vol,
                          const float *vs_vol, int nx, int ny, int nz, const float *x3d,
                          const float *y3d, const float *z3d, float *rho, float *lam,
                          float *mu)
{
  const float *v[3] = {rho_vol, vp_vol, vs_vol};
  float *o[3] = {rho, lam, mu};
  return stub_bin(0, model, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}

int cgfd_media_bin_vis_iso(const cgfd_bin_model_t *model, float xmin, float xmax, float ymin,
                           float ymax, const float *qp_vol, const float *qs_vol, int nx,
                           int ny, int nz, const float *x3d, const float *y3d,
                           const float *z3d, float *qp, float *qs)
{
  const float *v[2] = {qp_vol, qs_vol};
  float *o[2] = {qp, qs};
  return stub_bin(1, model, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}

int oracle_bin_crop(const int *order, const int *size, const float *spacing,
                    const float *origin, const float *ext, size_t vol, const float *z3d,
                    int *first, int *count);

int cgfd_media_bin_crop(const cgfd_bin_model_t *model, float xmin, float xmax, float ymin,
                        float ymax, int nx, int ny, int nz, const float *z3d,
                        cgfd_bin_box_t *box)
{
  const float ext[4] = {xmin, xmax, ymin, ymax};
  if (oracle_bin_crop(model->order, model->size, model->spacing, model->origin, ext,
                      (size_t)nx * ny * nz, z3d, box->first, box->count)) {
    stub_msg = "binary model: the model does not cover the grid";
    return CGFD_EINVAL;
  }
  return 0;
}

/* box volumes placed in zero-filled whole-file volumes (the crop reads
 * inside the box only), then the whole-file restatement */
static int stub_bin_box(int vis, const cgfd_bin_model_t *m, const cgfd_bin_box_t *box,
                        float xmin, float xmax, float ymin, float ymax, const float *const *bv,
                        int nx, int ny, int nz, const float *x3d, const float *y3d,
                        const float *z3d, float **o)
{
  const int nv = vis ? 2 : 3;
  const size_t whole = (size_t)m->size[0] * m->size[1] * m->size[2];
  float *v[3] = {NULL, NULL, NULL};
  int rc = 0;
  for (int n = 0; n < nv; n++) {
    v[n] = calloc(whole, sizeof(float));
    for (int c2 = 0; c2 < box->count[2]; c2++)
      for (int c1 = 0; c1 < box->count[1]; c1++)
        memcpy(v[n] + ((size_t)(box->first[2] + c2) * m->size[1] + box->first[1] + c1) *
                          m->size[0] + box->first[0],
               bv[n] + ((size_t)c2 * box->count[1] + c1) * box->count[0],
               (size_t)box->count[0] * sizeof(float));
  }
  rc = stub_bin(vis, m, xmin, xmax, ymin, ymax, (const float *const *)v, nx, ny, nz, x3d, y3d,
                z3d, o);
  for (int n = 0; n < nv; n++) free(v[n]);
  return rc;
}

int cgfd_media_bin_el_iso_box(const cgfd_bin_model_t *model, const cgfd_bin_box_t *box,
                              float xmin, float xmax, float ymin, float ymax,
                              const float *rho_box, const float *vp_box, const float *vs_box,
                              int nx, int ny, int nz, const float *x3d, const float *y3d,
                              const float *z3d, float *rho, float *lam, float *mu)
{
  const float *v[3] = {rho_box, vp_box, vs_box};
  float *o[3] = {rho, lam, mu};
  return stub_bin_box(0, model, box, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}

int cgfd_media_bin_vis_iso_box(const cgfd_bin_model_t *model, const cgfd_bin_box_t *box,
                               float xmin, float xmax, float ymin, float ymax,
                               const float *qp_box, const float *qs_box, int nx, int ny, int nz,
                               const float *x3d, const float *y3d, const float *z3d, float *qp,
                               float *qs)
{
  const float *v[2] = {qp_box, qs_box};
  float *o[2] = {qp, qs};
  return stub_bin_box(1, model, box, xmin, xmax, ymin, ymax, v, nx, ny, nz, x3d, y3d, z3d, o);
}

int oracle_grid_el_iso(int method, int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                       float MINY, float DX, float DY, const float *rec, int nx, int ny, int nz,
                       const float *x3d, const float *y3d, const float *z3d, float **out);

int cgfd_media_grid_el_iso(int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                           float MINY, float DX, float DY, const float *rec, int nx, int ny,
                           int nz, const float *x3d, const float *y3d, const float *z3d,
                           const char *method, float *rho, float *lam, float *mu)
{
  int m = stub_method(method);
  float *o[3] = {rho, lam, mu};
  if (m < 0 || oracle_grid_el_iso(m, NI, NL, ngz, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz,
                                  x3d, y3d, z3d, o)) {
    stub_msg = "grid model: bad method, a point outside the mesh or vp <= sqrt(2) vs";
    return CGFD_EINVAL;
  }
  return 0;
}

int oracle_grid_el_vti_loc(int kind, int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                           float MINY, float DX, float DY, const float *rec, int nx, int ny,
                           int nz, const float *x3d, const float *y3d, const float *z3d,
                           float **out);

int cgfd_media_grid_el_vti(int media_type, int NI, int NL, const int *ngz, int NX, int NY,
                           float MINX, float MINY, float DX, float DY, const float *rec, int nx,
                           int ny, int nz, const float *x3d, const float *y3d, const float *z3d,
                           const char *method, float *c11, float *c33, float *c55, float *c66,
                           float *c13, float *rho)
{
  float *o[6] = {c11, c33, c55, c66, c13, rho};
  if (stub_method(method) != 0 ||
      oracle_grid_el_vti_loc(media_type, NI, NL, ngz, NX, NY, MINX, MINY, DX, DY, rec, nx, ny,
                             nz, x3d, y3d, z3d, o)) {
    stub_msg = "grid model: bad method or a point outside the mesh";
    return CGFD_EINVAL;
  }
  return 0;
}
