/*
 * ref_update_stubs.c -- link glue for oracle/_ref/libenkf_ref_update.so (the
 * reference's own update/update.c and common/dasystem.c, compiled
 * unmodified; see ref_update.c).  TEST INFRASTRUCTURE ONLY.
 *
 * The two files also hold the reference's file I/O, assembly and MPI
 * distribution code, which name functions of its model, grid, NetCDF,
 * point-log and distribution modules.  The field-update entry points never
 * reach them; they are defined here to abort if reached.  sgemv_ (the only
 * BLAS call of the field update, update/update.c:399) is routed to the
 * OpenBLAS bound at run time by ../or_blas.c.
 */
#include <stdio.h>
#include <stdlib.h>
#include "../or_blas.h"

int orref_sgemv_(char* t, int* m, int* n, float* a, float* A, int* lda, float* x, int* incx, float* b, float* y,
                 int* incy)
{
    if (*incx != 1 || *incy != 1) {
        fprintf(stderr, "ref_update_stubs: sgemv_ with a stride other than 1\n");
        abort();
    }
    or_sgemv(*t, *m, *n, *a, A, *lda, x, *b, y);
    return 0;
}

/* the distribution module's globals (common/distribute.c) */
int my_first_iteration = 0;
int my_last_iteration = -1;

typedef void (*orref_quit_fn) (char* format, ...);
void ncw_set_quitfn(orref_quit_fn f) { (void) f; }
void ncu_set_quitfn(orref_quit_fn f) { (void) f; }

static void unreachable(const char* name)
{
    fprintf(stderr, "ref_update_stubs: %s is not available in this build\n", name);
    abort();
}

#define UNREACHABLE(name) void name(void) { unreachable(#name); }

UNREACHABLE(das_allocatedst)
UNREACHABLE(das_assemble)
UNREACHABLE(das_preassemble)
UNREACHABLE(das_writeinflation)
UNREACHABLE(das_writespread)
UNREACHABLE(distribute_free)
UNREACHABLE(distribute_iterations)
UNREACHABLE(grid_isempty)
UNREACHABLE(grid_isstructured)
UNREACHABLE(model_create)
UNREACHABLE(model_destroy)
UNREACHABLE(model_getgridbyname)
UNREACHABLE(model_getnvar)
UNREACHABLE(model_getvargridid)
UNREACHABLE(model_getvarname)
UNREACHABLE(model_readfield_part)
UNREACHABLE(model_writefield)
UNREACHABLE(ncu_getnlevels)
UNREACHABLE(ncw_att_exists)
UNREACHABLE(ncw_copy_vardef)
UNREACHABLE(ncw_create)
UNREACHABLE(ncw_def_deflate)
UNREACHABLE(ncw_def_dim)
UNREACHABLE(ncw_def_var)
UNREACHABLE(ncw_enddef)
UNREACHABLE(ncw_get_att_double)
UNREACHABLE(ncw_get_var_float)
UNREACHABLE(ncw_put_att_text)
UNREACHABLE(ncw_put_var_float)
UNREACHABLE(ncw_redef)
UNREACHABLE(ncw_var_exists)
UNREACHABLE(plogs_destroy)
UNREACHABLE(plogs_writestatevars)
