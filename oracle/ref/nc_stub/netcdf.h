/*
 * netcdf.h stand-in for compiling the reference's common/utils.c (which
 * includes common/ncw.h) into oracle/_ref/libenkf_ref_utils.so, and
 * update/update.c + common/dasystem.c into libenkf_ref_update.so, and
 * calc/ensobs.c into libenkf_ref_ensobs.so.  TEST
 * INFRASTRUCTURE ONLY.  Declares the handful of names the headers and
 * these files mention; nothing of NetCDF is called by the functions the
 * tests use (interpolation, taper, field update, hybrid ensemble).
 */
#ifndef ORREF_NETCDF_STUB_H
#define ORREF_NETCDF_STUB_H
#include <stddef.h>
typedef int nc_type;
#define NC_NOERR 0
#define NC_WRITE 1
#define NC_GLOBAL -1
#define NC_MAX_NAME 256
#define NC_NOWRITE 0
#define NC_CLOBBER 0
#define NC_NOCLOBBER 4
#define NC_64BIT_OFFSET 0x0200
#define NC_64BIT_DATA 0x0020
#define NC_CLASSIC_MODEL 0x0100
#define NC_NETCDF4 0x1000
#define NC_UNLIMITED 0L
#define NC_BYTE 1
#define NC_CHAR 2
#define NC_SHORT 3
#define NC_INT 4
#define NC_FLOAT 5
#define NC_DOUBLE 6
#define NC_CHUNKED 0
#define NC_CONTIGUOUS 1
#define NC_NOFILL 0x100
#define NC_UINT 9
#define NC_INT64 10
#define NC_UINT64 11
#define NC_UBYTE 7
#define NC_USHORT 8
#endif
