/*
 * netcdf.h stand-in for compiling the reference's common/utils.c (which
 * includes common/ncw.h) into oracle/_ref/libenkf_ref_utils.so.  TEST
 * INFRASTRUCTURE ONLY.  Declares the handful of names the header and
 * utils.c mention; nothing of NetCDF is called by the functions the tests
 * use (the interpolation and taper routines).
 */
#ifndef ORREF_NETCDF_STUB_H
#define ORREF_NETCDF_STUB_H
#include <stddef.h>
typedef int nc_type;
#define NC_NOERR 0
#define NC_WRITE 1
#define NC_GLOBAL -1
#define NC_MAX_NAME 256
#endif
