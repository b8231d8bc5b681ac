/*
 * ref_gethe_stubs.c -- link glue for oracle/_ref/libenkf_ref_gethe.so (see
 * ref_gethe.c).  TEST INFRASTRUCTURE ONLY: enkf_calc's skip-bad-forecast
 * flag, and the names the rest of calc/ensobs.c, calc/model2obs.c and the
 * observation module use (files, asynchronous observations, footprints,
 * mixed-layer depth, the analysis-observation update), defined to abort if
 * reached.
 */
#include <stdio.h>
#include <stdlib.h>

int skip_bad_fc_obs = 0;

static void unreachable(const char* name)
{
    fprintf(stderr, "ref_gethe_stubs: %s is not available in this build\n", name);
    abort();
}

#define UNREACHABLE(name) void name(void) { unreachable(#name); }

UNREACHABLE(das_calcmld)
UNREACHABLE(das_getbgfname_async)
UNREACHABLE(das_getfname_transforms)
UNREACHABLE(das_getmemberfname_async)
UNREACHABLE(grid_getsize)
UNREACHABLE(grid_getstride)
UNREACHABLE(grid_getvtype)
UNREACHABLE(grid_isperiodic_i)
UNREACHABLE(model_addorreplacedata)
UNREACHABLE(model_adddata)
UNREACHABLE(model_getdomainid)
UNREACHABLE(model_getvarinflation)
UNREACHABLE(model_getvarislog)
UNREACHABLE(nc_open)
UNREACHABLE(ncu_getnD)
UNREACHABLE(ncu_readvarfloat)
UNREACHABLE(ncw_check_attlen)
UNREACHABLE(ncw_check_varsize)
UNREACHABLE(ncw_create)
UNREACHABLE(ncw_def_deflate)
UNREACHABLE(ncw_def_dim)
UNREACHABLE(ncw_def_var)
UNREACHABLE(ncw_del_att)
UNREACHABLE(ncw_enddef)
UNREACHABLE(ncw_get_att_double)
UNREACHABLE(ncw_get_att_int)
UNREACHABLE(ncw_get_att_text)
UNREACHABLE(ncw_get_var_double)
UNREACHABLE(ncw_get_var_float)
UNREACHABLE(ncw_get_var_int)
UNREACHABLE(ncw_get_var_short)
UNREACHABLE(ncw_get_vara_float)
UNREACHABLE(ncw_inq_att)
UNREACHABLE(ncw_inq_attlen)
UNREACHABLE(ncw_inq_attname)
UNREACHABLE(ncw_inq_dimid)
UNREACHABLE(ncw_inq_dimlen)
UNREACHABLE(ncw_inq_vardims)
UNREACHABLE(ncw_inq_varid)
UNREACHABLE(ncw_inq_varnatts)
UNREACHABLE(ncw_put_att_int)
UNREACHABLE(ncw_put_var_double)
UNREACHABLE(ncw_put_var_float)
UNREACHABLE(ncw_put_var_uchar)
UNREACHABLE(ncw_redef)
UNREACHABLE(ncw_rename_var)
UNREACHABLE(ncw_var_exists)
