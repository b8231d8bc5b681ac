/*
 * ref_obs_stubs.c -- link glue for oracle/_ref/libenkf_ref_obs.so (the
 * reference's own common/observations.c and common/obstypes.c, compiled
 * unmodified; see ref_obs.c).  TEST INFRASTRUCTURE ONLY.
 *
 * The two files also read and write observation files and parse the
 * obstypes parameter file, which name functions of the model, grid and
 * NetCDF modules; obs_findlocal never reaches them, and they are defined
 * here to abort if reached.  kd_printinfo (a diagnostic print that
 * obs_createkdtrees makes; common/utils.c defines it only for enkf_calc
 * builds) does nothing here.
 */
#include <stdio.h>
#include <stdlib.h>

void kd_printinfo(void* tree, char* offset)
{
    (void) tree;
    (void) offset;
}

static void unreachable(const char* name)
{
    fprintf(stderr, "ref_obs_stubs: %s is not available in this build\n", name);
    abort();
}

#define UNREACHABLE(name) void name(void) { unreachable(#name); }

UNREACHABLE(grid_isgeographic)
UNREACHABLE(model_adddata)
UNREACHABLE(model_getdomainid)
UNREACHABLE(model_getgridbyid)
UNREACHABLE(model_getvargridid)
UNREACHABLE(model_getvargridsize)
UNREACHABLE(model_getvarid)
UNREACHABLE(model_getvarislog)
UNREACHABLE(nc_open)
UNREACHABLE(ncu_getnD)
UNREACHABLE(ncu_readvarfloat)
UNREACHABLE(ncw_check_attlen)
UNREACHABLE(ncw_check_varsize)
UNREACHABLE(ncw_get_att_double)
UNREACHABLE(ncw_get_att_int)
UNREACHABLE(ncw_get_att_text)
UNREACHABLE(ncw_get_var_double)
UNREACHABLE(ncw_get_var_float)
UNREACHABLE(ncw_get_var_int)
UNREACHABLE(ncw_get_var_short)
UNREACHABLE(ncw_inq_att)
UNREACHABLE(ncw_inq_attlen)
UNREACHABLE(ncw_inq_attname)
UNREACHABLE(ncw_inq_dimid)
UNREACHABLE(ncw_inq_dimlen)
UNREACHABLE(ncw_inq_varid)
UNREACHABLE(ncw_inq_varnatts)
UNREACHABLE(ncw_put_var_uchar)
UNREACHABLE(ncw_var_exists)
