/*
 * ref_model2obs.c -- entry point into the reference's own calc/model2obs.c
 * (compiled unmodified) for oracle/_ref/libenkf_ref_model2obs.so.  TEST
 * INFRASTRUCTURE ONLY: pins the oracle's restatement of the forward
 * operators H_surf_standard and H_subsurf_standard (calc/model2obs.c:
 * 127-181, 256-348, with evaluate_2d_obs and interpolate_3d_obs, 37-124)
 * against the reference itself.
 *
 * What the H functions read outside model2obs.c is supplied in memory: the
 * observations (type, fractional grid position fij and fk, no footprint),
 * one model variable on one structured grid (its size, wet-level counts,
 * periodicity and surface-layer index), the member's field as the model
 * module would read it, and its OFFSET data.  The grid's interpolation
 * entry points are the grid module's one-line dispatch to the reference's
 * interpolate2d_structured / interpolate3d_structured (common/utils.c,
 * compiled into the library).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "ncw.h"
#include "global.h"
#include "utils.h"
#include "observations.h"
#include "dasystem.h"
#include "model2obs.h"

extern int skip_bad_fc_obs;

static struct {
    int ni, nj, nk, ksurf, periodic_i;
    int** numlevels;            /* row pointers [nj][ni] */
    const float* field;         /* [nk][nj][ni] */
    void* offset;               /* row-pointer view for ALLOCTYPE_2D / 3D, plain for 1D; NULL: none */
    int offset_type;
} mo;

static int orref_model_handle;

int model_getvarid(model* m, char* name, int hastosucceed) { (void) m; (void) name; (void) hastosucceed; return 0; }
void* model_getvargrid(model* m, int vid) { (void) m; (void) vid; return &orref_model_handle; }
int model_getvargridid(model* m, int vid) { (void) m; (void) vid; return 0; }
void model_getvargridsize(model* m, int vid, int* ni, int* nj, int* nk)
{
    (void) m;
    (void) vid;
    if (ni != NULL)
        *ni = mo.ni;
    if (nj != NULL)
        *nj = mo.nj;
    if (nk != NULL)
        *nk = mo.nk;
}
int grid_getsurflayerid(grid* g) { (void) g; return mo.ksurf; }
int grid_isstructured(grid* g) { (void) g; return 1; }
int grid_isgeographic(grid* g) { (void) g; return 0; }
int das_isstatic(dasystem* das, int mem) { (void) das; (void) mem; return 0; }

void model_readfield(model* m, char fname[], char varname[], int r, int k, float* v, int ignorelog)
{
    (void) m;
    (void) fname;
    (void) varname;
    (void) r;
    (void) ignorelog;
    memcpy(v, mo.field + (size_t) k * mo.ni * mo.nj, (size_t) mo.ni * mo.nj * sizeof(float));
}

void model_read3dfield(model* m, char fname[], char varname[], int r, float* v, int ignorelog)
{
    (void) m;
    (void) fname;
    (void) varname;
    (void) r;
    (void) ignorelog;
    memcpy(v, mo.field, (size_t) mo.ni * mo.nj * mo.nk * sizeof(float));
}

void* model_getdata(model* m, char tag[]) { (void) m; (void) tag; return mo.offset; }
int model_getdataalloctype(model* m, char tag[]) { (void) m; (void) tag; return mo.offset_type; }

/* grid.c:727-743 and 748-760 for a structured grid */
float grid_interpolate2d(grid* g, double* fij, void* v)
{
    (void) g;
    if (v == NULL)
        return NAN;
    return interpolate2d_structured(fij, mo.ni, mo.nj, (float**) v, mo.numlevels, mo.periodic_i);
}

float grid_interpolate3d(grid* g, double* fij, float fk, void* v)
{
    (void) g;
    if (v == NULL)
        return NAN;
    return interpolate3d_structured(fij, (double) fk, mo.ni, mo.nj, mo.nk, mo.ksurf, (float***) v, mo.numlevels,
                                    mo.periodic_i);
}

/*
 * H_surf_standard (three_d 0: the surface layer ksurf of field) or
 * H_subsurf_standard (three_d 1) for one member: field [nk][nj][ni],
 * numlevels [nj][ni]; offset NULL or [nk] (offset_kind 1, 3-D only),
 * [nj][ni] (2) or [nk][nj][ni] (3, 3-D only); the nids observations ids[]
 * of nobs, at (fi, fj, fk); dst [nobs] receives them (NaN elsewhere).
 * skip_bad: the --skip-bad-forecast-obs flag (without it a bad forecast
 * stops the process, as in the reference).
 */
int ref_H(int three_d, int ni, int nj, int nk, int ksurf, int periodic_i, int* numlevels, const float* offset,
          int offset_kind, const float* field, int nobs, int nids, const int* ids, const double* fi, const double* fj,
          const float* fk, int skip_bad, float* dst)
{
    dasystem das;
    observations obs;
    obstype ot;
    observation* data = calloc(nobs > 0 ? nobs : 1, sizeof(observation));
    char* varnames[1] = { "v" };
    int** nl = malloc(nj * sizeof(int*));
    int* sel = malloc((nids > 0 ? nids : 1) * sizeof(int));
    void* off = NULL;
    int o, j, k;

    for (j = 0; j < nj; ++j)
        nl[j] = numlevels + (size_t) j * ni;
    mo.ni = ni;
    mo.nj = nj;
    mo.nk = nk;
    mo.ksurf = ksurf;
    mo.periodic_i = periodic_i;
    mo.numlevels = nl;
    mo.field = field;
    mo.offset_type = ALLOCTYPE_NONE;
    if (offset != NULL && offset_kind == 1) {
        off = (void*) offset;
        mo.offset_type = ALLOCTYPE_1D;
    } else if (offset != NULL && offset_kind == 2) {
        float** r = malloc(nj * sizeof(float*));

        for (j = 0; j < nj; ++j)
            r[j] = (float*) offset + (size_t) j * ni;
        off = r;
        mo.offset_type = ALLOCTYPE_2D;
    } else if (offset != NULL && offset_kind == 3) {
        float*** r = malloc(nk * sizeof(float**));

        for (k = 0; k < nk; ++k) {
            r[k] = malloc(nj * sizeof(float*));
            for (j = 0; j < nj; ++j)
                r[k][j] = (float*) offset + ((size_t) k * nj + j) * ni;
        }
        off = r;
        mo.offset_type = ALLOCTYPE_3D;
    }
    mo.offset = off;

    memset(&ot, 0, sizeof(ot));
    ot.name = "type0";
    ot.nvar = 1;
    ot.varnames = varnames;
    memset(&obs, 0, sizeof(obs));
    for (o = 0; o < nobs; ++o) {
        data[o].id = o;
        data[o].type = 0;
        data[o].fij[0] = fi[o];
        data[o].fij[1] = fj[o];
        data[o].fij[2] = NAN;
        data[o].fk = fk != NULL ? fk[o] : 0.0f;
        dst[o] = NAN;
    }
    obs.nobstypes = 1;
    obs.obstypes = &ot;
    obs.nobs = nobs;
    obs.data = data;
    memset(&das, 0, sizeof(das));
    das.mode = MODE_ENKF;
    das.obs = &obs;
    das.m = (model*) &orref_model_handle;
    skip_bad_fc_obs = skip_bad;
    memcpy(sel, ids, nids * sizeof(int));
    if (three_d)
        H_subsurf_standard(&das, nids, sel, "member", 0, 1, 0, dst);
    else
        H_surf_standard(&das, nids, sel, "member", 0, 1, 0, dst);

    if (offset_kind == 3 && off != NULL) {
        for (k = 0; k < nk; ++k)
            free(((float***) off)[k]);
        free(off);
    } else if (offset_kind == 2 && off != NULL)
        free(off);
    free(sel);
    free(nl);
    free(data);
    return 0;
}
