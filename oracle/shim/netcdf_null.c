/*
 * Null NetCDF implementation (see shim/netcdf.h).
 * TEST INFRASTRUCTURE ONLY (reference build for golden vectors).
 */
#include <stdio.h>
#include "netcdf.h"

static int next_id = 1;

const char *nc_strerror(int ncerr)
{
  return ncerr == NC_NOERR ? "no error"
                           : "NetCDF reading is not available in the null shim";
}
int nc_create(const char *path, int cmode, int *ncidp)
{ (void)path; (void)cmode; *ncidp = next_id++; return NC_NOERR; }
int nc_open(const char *path, int mode, int *ncidp)
{ (void)mode; *ncidp = -1; fprintf(stderr, "netcdf shim: cannot open %s\n", path); return NC_ENOTFOUND; }
int nc_close(int ncid) { (void)ncid; return NC_NOERR; }
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
{ (void)ncid; (void)varid; (void)name; (void)ip; return NC_ENOTFOUND; }
int nc_inq_varid(int ncid, const char *name, int *varidp)
{ (void)ncid; (void)name; (void)varidp; return NC_ENOTFOUND; }
int nc_inq_dimid(int ncid, const char *name, int *idp)
{ (void)ncid; (void)name; (void)idp; return NC_ENOTFOUND; }
int nc_inq_dimlen(int ncid, int dimid, size_t *lenp)
{ (void)ncid; (void)dimid; (void)lenp; return NC_ENOTFOUND; }
int nc_put_var_float(int ncid, int varid, const float *op)
{ (void)ncid; (void)varid; (void)op; return NC_NOERR; }
int nc_put_var1_float(int ncid, int varid, const size_t *indexp, const float *op)
{ (void)ncid; (void)varid; (void)indexp; (void)op; return NC_NOERR; }
int nc_put_vara_float(int ncid, int varid, const size_t *startp,
                      const size_t *countp, const float *op)
{ (void)ncid; (void)varid; (void)startp; (void)countp; (void)op; return NC_NOERR; }
int nc_get_var(int ncid, int varid, void *ip)
{ (void)ncid; (void)varid; (void)ip; return NC_ENOTFOUND; }
int nc_get_var_float(int ncid, int varid, float *ip)
{ (void)ncid; (void)varid; (void)ip; return NC_ENOTFOUND; }
int nc_get_vara_float(int ncid, int varid, const size_t *startp,
                      const size_t *countp, float *ip)
{ (void)ncid; (void)varid; (void)startp; (void)countp; (void)ip; return NC_ENOTFOUND; }
