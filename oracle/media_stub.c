/*
 * media_stub.c -- TEST INFRASTRUCTURE ONLY.  Stands in for the CUDA
 * library's cgfd_media_layer_el_iso, _el_vti and _onecmp
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

int cgfd_media_layer_onecmp(int NI, int NX, int NY, float MINX, float MINY, float DX, float DY,
                            const float *rec, int nx, int ny, int nz, const float *x3d,
                            const float *y3d, const float *z3d, const char *method, float *var)
{
  float *out[1] = {var};
  return stub_run(0, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d, z3d, method,
                  out);
}
