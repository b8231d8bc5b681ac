/*
 * ref_ensobs_stubs.c -- link glue for oracle/_ref/libenkf_ref_ensobs.so (the
 * reference's own calc/ensobs.c, compiled unmodified; see ref_ensobs.c).
 * TEST INFRASTRUCTURE ONLY.
 *
 * ensobs.c also holds the reference's HE assembly from the model fields and
 * its observation-file output, which name functions of its model, grid,
 * NetCDF, observation and distribution modules.  das_calcinnandspread and
 * das_standardise never reach them (only their error paths print an
 * observation); they are defined here to abort if reached.
 */
#include <stdio.h>
#include <stdlib.h>

/* the distribution module's globals (common/distribute.c) and enkf_calc's
 * skip-bad-forecast flag */
int my_first_iteration = 0;
int my_last_iteration = -1;
int skip_bad_fc_obs = 0;

static void unreachable(const char* name)
{
    fprintf(stderr, "ref_ensobs_stubs: %s is not available in this build\n", name);
    abort();
}

#define UNREACHABLE(name) void name(void) { unreachable(#name); }

UNREACHABLE(das_getbgfname)
UNREACHABLE(das_getbgfname_async)
UNREACHABLE(das_getfname_transforms)
UNREACHABLE(das_getmemberfname)
UNREACHABLE(das_getmemberfname_async)
UNREACHABLE(distribute_iterations)
UNREACHABLE(getH)
UNREACHABLE(grid_destroytreeXYZ)
UNREACHABLE(grid_getsize)
UNREACHABLE(grid_getstride)
UNREACHABLE(grid_gettreeXYZ)
UNREACHABLE(grid_isperiodic_i)
UNREACHABLE(grid_isstructured)
UNREACHABLE(kd_printinfo)
UNREACHABLE(model_getgridbyid)
UNREACHABLE(model_getngrid)
UNREACHABLE(model_getvarinflation)
UNREACHABLE(ncw_create)
UNREACHABLE(ncw_def_deflate)
UNREACHABLE(ncw_def_dim)
UNREACHABLE(ncw_def_var)
UNREACHABLE(ncw_del_att)
UNREACHABLE(ncw_enddef)
UNREACHABLE(ncw_get_att_double)
UNREACHABLE(ncw_get_vara_float)
UNREACHABLE(ncw_inq_dimid)
UNREACHABLE(ncw_inq_dimlen)
UNREACHABLE(ncw_inq_vardims)
UNREACHABLE(ncw_inq_varid)
UNREACHABLE(ncw_put_att_int)
UNREACHABLE(ncw_put_var_double)
UNREACHABLE(ncw_put_var_float)
UNREACHABLE(ncw_redef)
UNREACHABLE(ncw_rename_var)
UNREACHABLE(ncw_var_exists)
UNREACHABLE(obs_calcstats)
UNREACHABLE(obs_find_bytype)
UNREACHABLE(obs_find_bytypeandtime)
UNREACHABLE(obs_inorder)
UNREACHABLE(obs_printob)
UNREACHABLE(orref_sgemv_)
