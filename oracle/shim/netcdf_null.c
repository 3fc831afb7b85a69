/*
 * Null NetCDF implementation (see shim/netcdf.h).
 * TEST INFRASTRUCTURE ONLY (reference build for golden vectors).
 *
 * Writers discard their data.  Readers accept one format only: a raw
 * container the golden-fixture scripts write (not NetCDF), holding what the
 * reference's distributed-source reader asks for (forward/src_t.c:1245-1640):
 *   char magic[8] = "CGNCRAW1";
 *   int n_att;  n_att x { char name[32]; int value; }        (global ints)
 *   int n_dim;  n_dim x { char name[32]; long long len; }
 *   int n_var;  n_var x { char name[32]; int ndims; int dimid[4];
 *                         float data[product of the dims' lengths]; }
 * Opened containers get ids from 1000 up; any other file fails to open.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "netcdf.h"

#define RAW_MAX 4
#define RAW_BASE 1000
typedef struct {
  int used;
  int natt, ndim, nvar;
  char (*att_name)[32];
  int *att_val;
  char (*dim_name)[32];
  long long *dim_len;
  char (*var_name)[32];
  int *var_ndims;
  int (*var_dims)[4];
  float **var_data;
} raw_file_t;
static raw_file_t g_raw[RAW_MAX];

static raw_file_t *raw_of(int ncid)
{
  int k = ncid - RAW_BASE;
  return (k >= 0 && k < RAW_MAX && g_raw[k].used) ? &g_raw[k] : NULL;
}

static long long raw_var_len(const raw_file_t *f, int v)
{
  long long n = 1;
  for (int d = 0; d < f->var_ndims[v]; d++) n *= f->dim_len[f->var_dims[v][d]];
  return n;
}

static int raw_open(const char *path, int *ncidp)
{
  FILE *fp = fopen(path, "rb");
  if (!fp) return NC_ENOTFOUND;
  char magic[8];
  int k = 0;
  while (k < RAW_MAX && g_raw[k].used) k++;
  if (k == RAW_MAX || fread(magic, 1, 8, fp) != 8 || memcmp(magic, "CGNCRAW1", 8) != 0) {
    fclose(fp);
    return NC_ENOTFOUND;
  }
  raw_file_t *f = &g_raw[k];
  memset(f, 0, sizeof(*f));
  int ok = fread(&f->natt, 4, 1, fp) == 1;
  f->att_name = calloc(f->natt + 1, 32);
  f->att_val = calloc(f->natt + 1, sizeof(int));
  for (int a = 0; ok && a < f->natt; a++)
    ok = fread(f->att_name[a], 32, 1, fp) == 1 && fread(&f->att_val[a], 4, 1, fp) == 1;
  ok = ok && fread(&f->ndim, 4, 1, fp) == 1;
  f->dim_name = calloc(f->ndim + 1, 32);
  f->dim_len = calloc(f->ndim + 1, sizeof(long long));
  for (int d = 0; ok && d < f->ndim; d++)
    ok = fread(f->dim_name[d], 32, 1, fp) == 1 && fread(&f->dim_len[d], 8, 1, fp) == 1;
  ok = ok && fread(&f->nvar, 4, 1, fp) == 1;
  f->var_name = calloc(f->nvar + 1, 32);
  f->var_ndims = calloc(f->nvar + 1, sizeof(int));
  f->var_dims = calloc(f->nvar + 1, sizeof(int[4]));
  f->var_data = calloc(f->nvar + 1, sizeof(float *));
  for (int v = 0; ok && v < f->nvar; v++) {
    ok = fread(f->var_name[v], 32, 1, fp) == 1 && fread(&f->var_ndims[v], 4, 1, fp) == 1 &&
         fread(f->var_dims[v], 4, 4, fp) == 4;
    if (!ok) break;
    long long n = raw_var_len(f, v);
    f->var_data[v] = malloc((size_t)n * sizeof(float));
    ok = fread(f->var_data[v], sizeof(float), (size_t)n, fp) == (size_t)n;
  }
  fclose(fp);
  if (!ok) return NC_ENOTFOUND;
  f->used = 1;
  *ncidp = RAW_BASE + k;
  return NC_NOERR;
}

static int next_id = 1;

const char *nc_strerror(int ncerr)
{
  return ncerr == NC_NOERR ? "no error"
                           : "NetCDF reading is not available in the null shim";
}
int nc_create(const char *path, int cmode, int *ncidp)
{ (void)path; (void)cmode; *ncidp = next_id++; return NC_NOERR; }
int nc_open(const char *path, int mode, int *ncidp)
{
  (void)mode;
  *ncidp = -1;
  if (raw_open(path, ncidp) == NC_NOERR) return NC_NOERR;
  fprintf(stderr, "netcdf shim: cannot open %s\n", path);
  return NC_ENOTFOUND;
}
int nc_close(int ncid)
{
  raw_file_t *f = raw_of(ncid);
  if (f) {
    for (int v = 0; v < f->nvar; v++) free(f->var_data[v]);
    free(f->att_name); free(f->att_val); free(f->dim_name); free(f->dim_len);
    free(f->var_name); free(f->var_ndims); free(f->var_dims); free(f->var_data);
    f->used = 0;
  }
  return NC_NOERR;
}
int nc_enddef(int ncid) { (void)ncid; return NC_NOERR; }
int nc_def_dim(int ncid, const char *name, size_t len, int *idp)
{ (void)ncid; (void)name; (void)len; *idp = next_id++; return NC_NOERR; }
int nc_def_var(int ncid, const char *name, nc_type xtype, int ndims,
               const int *dimidsp, int *varidp)
{ (void)ncid; (void)name; (void)xtype; (void)ndims; (void)dimidsp; *varidp = next_id++; return NC_NOERR; }
int nc_put_att_int(int ncid, int varid, const char *name, nc_type xtype,
                   size_t len, const int *op)
{ (void)ncid; (void)varid; (void)name; (void)xtype; (void)len; (void)op; return NC_NOERR; }
int nc_get_att_int(int ncid, int varid, const char *name, int *ip)
{
  raw_file_t *f = raw_of(ncid);
  if (!f || varid != NC_GLOBAL) return NC_ENOTFOUND;
  for (int a = 0; a < f->natt; a++)
    if (strncmp(f->att_name[a], name, 32) == 0) { *ip = f->att_val[a]; return NC_NOERR; }
  return NC_ENOTFOUND;
}
int nc_inq_varid(int ncid, const char *name, int *varidp)
{
  raw_file_t *f = raw_of(ncid);
  if (!f) return NC_ENOTFOUND;
  for (int v = 0; v < f->nvar; v++)
    if (strncmp(f->var_name[v], name, 32) == 0) { *varidp = v; return NC_NOERR; }
  return NC_ENOTFOUND;
}
int nc_inq_dimid(int ncid, const char *name, int *idp)
{
  raw_file_t *f = raw_of(ncid);
  if (!f) return NC_ENOTFOUND;
  for (int d = 0; d < f->ndim; d++)
    if (strncmp(f->dim_name[d], name, 32) == 0) { *idp = d; return NC_NOERR; }
  return NC_ENOTFOUND;
}
int nc_inq_dimlen(int ncid, int dimid, size_t *lenp)
{
  raw_file_t *f = raw_of(ncid);
  if (!f || dimid < 0 || dimid >= f->ndim) return NC_ENOTFOUND;
  *lenp = (size_t)f->dim_len[dimid];
  return NC_NOERR;
}
int nc_put_var_float(int ncid, int varid, const float *op)
{ (void)ncid; (void)varid; (void)op; return NC_NOERR; }
int nc_put_var1_float(int ncid, int varid, const size_t *indexp, const float *op)
{ (void)ncid; (void)varid; (void)indexp; (void)op; return NC_NOERR; }
int nc_put_vara_float(int ncid, int varid, const size_t *startp,
                      const size_t *countp, const float *op)
{ (void)ncid; (void)varid; (void)startp; (void)countp; (void)op; return NC_NOERR; }
int nc_get_var_float(int ncid, int varid, float *ip)
{
  raw_file_t *f = raw_of(ncid);
  if (!f || varid < 0 || varid >= f->nvar) return NC_ENOTFOUND;
  memcpy(ip, f->var_data[varid], (size_t)raw_var_len(f, varid) * sizeof(float));
  return NC_NOERR;
}
int nc_get_var(int ncid, int varid, void *ip) { return nc_get_var_float(ncid, varid, (float *)ip); }
int nc_get_vara_float(int ncid, int varid, const size_t *startp,
                      const size_t *countp, float *ip)
{
  raw_file_t *f = raw_of(ncid);
  if (!f || varid < 0 || varid >= f->nvar) return NC_ENOTFOUND;
  const int nd = f->var_ndims[varid];
  long long len[4] = {1, 1, 1, 1}, st[4] = {0, 0, 0, 0}, ct[4] = {1, 1, 1, 1};
  for (int d = 0; d < nd; d++) {
    len[4 - nd + d] = f->dim_len[f->var_dims[varid][d]];
    st[4 - nd + d] = (long long)startp[d];
    ct[4 - nd + d] = (long long)countp[d];
    if (st[4 - nd + d] + ct[4 - nd + d] > len[4 - nd + d]) return NC_ENOTFOUND;
  }
  const float *src = f->var_data[varid];
  size_t o = 0;
  for (long long a = 0; a < ct[0]; a++)
    for (long long b = 0; b < ct[1]; b++)
      for (long long c = 0; c < ct[2]; c++)
        for (long long e = 0; e < ct[3]; e++)
          ip[o++] = src[(((st[0] + a) * len[1] + st[1] + b) * len[2] + st[2] + c) * len[3] +
                        st[3] + e];
  return NC_NOERR;
}
