/*
 * ref_utils_stubs.c -- link glue for oracle/_ref/libenkf_ref_utils.so, the
 * reference's own common/utils.c, common/global.c and common/version.c
 * compiled unmodified.  TEST INFRASTRUCTURE ONLY: the library pins the
 * oracle's forward-operator restatement (interpolate2d_structured,
 * interpolate3d_structured, taper_gc, ll2xyz) against the reference.
 *
 * utils.c references a few NetCDF wrappers (common/ncw.c, common/ncutils.c)
 * from its file-writing helpers, which the tests never call; they are defined
 * here to abort if reached.
 */
#include <stdio.h>
#include <stdlib.h>

static void unreachable(const char* name)
{
    fprintf(stderr, "ref_utils_stubs: %s is not available in this build\n", name);
    abort();
}

typedef void (*orref_quit_fn) (char* format, ...);

void ncw_set_quitfn(orref_quit_fn f) { (void) f; }
void ncu_set_quitfn(orref_quit_fn f) { (void) f; }
void ncw_open(const char fname[], int mode, int* ncid) { (void) fname; (void) mode; (void) ncid; unreachable("ncw_open"); }
void ncw_close(int ncid) { (void) ncid; unreachable("ncw_close"); }
void ncw_put_att_text(int ncid, int varid, const char attname[], const char v[]) { (void) ncid; (void) varid; (void) attname; (void) v; unreachable("ncw_put_att_text"); }
int ncw_att_exists(int ncid, int varid, const char attname[]) { (void) ncid; (void) varid; (void) attname; unreachable("ncw_att_exists"); return 0; }
