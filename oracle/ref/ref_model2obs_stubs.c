/*
 * ref_model2obs_stubs.c -- link glue for oracle/_ref/libenkf_ref_model2obs.so
 * (see ref_model2obs.c).  TEST INFRASTRUCTURE ONLY: enkf_calc's
 * skip-bad-forecast flag, and the names the other H functions of
 * calc/model2obs.c use (footprints, mixed-layer depth, bias files, vertical
 * sums), defined to abort if reached.
 */
#include <stdio.h>
#include <stdlib.h>

int skip_bad_fc_obs = 0;

static void unreachable(const char* name)
{
    fprintf(stderr, "ref_model2obs_stubs: %s is not available in this build\n", name);
    abort();
}

#define UNREACHABLE(name) void name(void) { unreachable(#name); }

UNREACHABLE(das_calcmld)
UNREACHABLE(das_getbgfname)
UNREACHABLE(das_getmemberfname)
UNREACHABLE(grid_gettreeXYZ)
UNREACHABLE(grid_getvtype)
UNREACHABLE(kd_findnodeswithinrange)
UNREACHABLE(kd_getnodedata)
UNREACHABLE(model_addorreplacedata)
UNREACHABLE(model_getvarislog)
UNREACHABLE(ncu_getnD)
UNREACHABLE(obs_printob)
