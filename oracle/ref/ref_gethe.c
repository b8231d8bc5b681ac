/*
 * ref_gethe.c -- entry point into the reference's own das_getHE
 * (calc/ensobs.c:46-490, compiled unmodified with calc/model2obs.c,
 * calc/allhs.c and the observation module) for
 * oracle/_ref/libenkf_ref_gethe.so.  TEST INFRASTRUCTURE ONLY: pins the
 * oracle's restatement of the whole HE stage -- the forward operators per
 * type and member, the bad-forecast statuses and the EnOI / hybrid
 * treatment at its end -- against the reference itself.
 *
 * Supplied in memory: the members' files (one 3-D variable "v" on one
 * structured grid; the EnOI background after the members), the grid (size,
 * wet levels, periodicity, surface-layer index; its interpolation entry
 * points are the grid module's one-line dispatch to the reference's
 * interpolate2d_structured / interpolate3d_structured), the distribution of
 * all members to this one process, and the observations (type, status,
 * fractional grid position, no footprint).
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
    int ni, nj, nk, ksurf, periodic_i, nmem;
    int** numlevels;
    const float* members;       /* [nmem (+1)][nk][nj][ni] */
} ge;

static int orref_model_handle;

/* the member of a file name made by das_getmemberfname / das_getbgfname */
static const float* member_of(const char* fname)
{
    int e = 0;

    if (strcmp(fname, "bg") == 0)
        e = ge.nmem;
    else if (sscanf(fname, "mem%d", &e) == 1)
        e -= 1;
    else
        enkf_quit("ref_gethe: unknown file %s", fname);
    return ge.members + (size_t) e * ge.nk * ge.nj * ge.ni;
}

void das_getmemberfname(dasystem* das, char varname[], int mem, char fname[])
{
    (void) das;
    (void) varname;
    snprintf(fname, MAXSTRLEN, "mem%03d", mem);
}

void das_getbgfname(dasystem* das, char varname[], char fname[])
{
    (void) das;
    (void) varname;
    snprintf(fname, MAXSTRLEN, "bg");
}

int das_isstatic(dasystem* das, int mem)
{
    return mem > das->nmem_dynamic;     /* common/dasystem.c:826-829 */
}

int model_getvarid(model* m, char* name, int hastosucceed) { (void) m; (void) name; (void) hastosucceed; return 0; }
void* model_getvargrid(model* m, int vid) { (void) m; (void) vid; return &orref_model_handle; }
int model_getvargridid(model* m, int vid) { (void) m; (void) vid; return 0; }
int model_getngrid(model* m) { (void) m; return 1; }
void* model_getgridbyid(model* m, int id) { (void) m; (void) id; return &orref_model_handle; }
void model_getvargridsize(model* m, int vid, int* ni, int* nj, int* nk)
{
    (void) m;
    (void) vid;
    if (ni != NULL)
        *ni = ge.ni;
    if (nj != NULL)
        *nj = ge.nj;
    if (nk != NULL)
        *nk = ge.nk;
}
int grid_getsurflayerid(grid* g) { (void) g; return ge.ksurf; }
int grid_isstructured(grid* g) { (void) g; return 1; }
int grid_isgeographic(grid* g) { (void) g; return 0; }
kdtree* grid_gettreeXYZ(grid* g, int createifnull) { (void) g; (void) createifnull; return NULL; }
void grid_destroytreeXYZ(grid* g) { (void) g; }

void model_readfield(model* m, char fname[], char varname[], int r, int k, float* v, int ignorelog)
{
    (void) m;
    (void) varname;
    (void) r;
    (void) ignorelog;
    memcpy(v, member_of(fname) + (size_t) k * ge.ni * ge.nj, (size_t) ge.ni * ge.nj * sizeof(float));
}

void model_read3dfield(model* m, char fname[], char varname[], int r, float* v, int ignorelog)
{
    (void) m;
    (void) varname;
    (void) r;
    (void) ignorelog;
    memcpy(v, member_of(fname), (size_t) ge.ni * ge.nj * ge.nk * sizeof(float));
}

void* model_getdata(model* m, char tag[]) { (void) m; (void) tag; return NULL; }
int model_getdataalloctype(model* m, char tag[]) { (void) m; (void) tag; return ALLOCTYPE_NONE; }

float grid_interpolate2d(grid* g, double* fij, void* v)
{
    (void) g;
    if (v == NULL)
        return NAN;
    return interpolate2d_structured(fij, ge.ni, ge.nj, (float**) v, ge.numlevels, ge.periodic_i);
}

float grid_interpolate3d(grid* g, double* fij, float fk, void* v)
{
    (void) g;
    if (v == NULL)
        return NAN;
    return interpolate3d_structured(fij, (double) fk, ge.ni, ge.nj, ge.nk, ge.ksurf, (float***) v, ge.numlevels,
                                    ge.periodic_i);
}

/* all iterations (members) to this process */
int my_number_of_iterations = 0;
int my_first_iteration = 0;
int my_last_iteration = -1;
int* number_of_iterations = NULL;
int* first_iteration = NULL;
int* last_iteration = NULL;

void distribute_iterations(int i1, int i2, int nslot, char prefix[])
{
    (void) nslot;
    (void) prefix;
    my_first_iteration = i1;
    my_last_iteration = i2;
    my_number_of_iterations = i2 - i1 + 1;
}

/* a diagnostic print (common/utils.c has it only in enkf_calc builds) */
void kd_printinfo(kdtree* tree, char* offset)
{
    (void) tree;
    (void) offset;
}

/*
 * das_getHE for mode (the reference's codes: MODE_ENKF 1, ENOI 2, HYBRID 3)
 * on members [nmem (+1: the EnOI background)][nk][nj][ni] of one variable;
 * observations of ntypes types (issurface[t]: H_surf_standard, else
 * H_subsurf_standard) with status (in and out: the bad-forecast statuses
 * come back), fi, fj, fk.  HE [nmem (+1)][nobs] receives das->S.
 */
int ref_getHE(int mode, int nmem, int nmem_dynamic, double gamma, int skip_bad, int ni, int nj, int nk, int ksurf,
              int periodic_i, int* numlevels, const float* members, int nobs, const short* type, short* status,
              const double* fi, const double* fj, const float* fk, int ntypes, const int* issurface, float* HE)
{
    dasystem das;
    observations obs;
    obstype* types = calloc(ntypes > 0 ? ntypes : 1, sizeof(obstype));
    observation* data = calloc(nobs > 0 ? nobs : 1, sizeof(observation));
    char* varnames[1] = { "v" };
    int** nl = malloc(nj * sizeof(int*));
    const int nrows = (mode == MODE_ENOI) ? nmem + 1 : nmem;
    int o, j, t;

    for (j = 0; j < nj; ++j)
        nl[j] = numlevels + (size_t) j * ni;
    ge.ni = ni;
    ge.nj = nj;
    ge.nk = nk;
    ge.ksurf = ksurf;
    ge.periodic_i = periodic_i;
    ge.nmem = nmem;
    ge.numlevels = nl;
    ge.members = members;
    for (t = 0; t < ntypes; ++t) {
        char name[32];

        snprintf(name, sizeof(name), "type%d", t);
        types[t].id = t;
        types[t].name = strdup(name);
        types[t].issurface = issurface[t];
        types[t].hfunction = "standard";
        types[t].nvar = 1;
        types[t].varnames = varnames;
        types[t].alias = "v";
    }
    for (o = 0; o < nobs; ++o) {
        data[o].id = o;
        data[o].type = type[o];
        data[o].status = status[o];
        data[o].fij[0] = fi[o];
        data[o].fij[1] = fj[o];
        data[o].fij[2] = NAN;
        data[o].fk = fk[o];
        types[type[o]].nobs++;
    }
    memset(&obs, 0, sizeof(obs));
    obs.nobstypes = ntypes;
    obs.obstypes = types;
    obs.nobs = nobs;
    obs.data = data;
    memset(&das, 0, sizeof(das));
    das.mode = mode;
    das.nmem = nmem;
    das.nmem_dynamic = nmem_dynamic;
    das.nmem_static = nmem - nmem_dynamic;
    das.gamma = gamma;
    das.obs = &obs;
    das.m = (model*) &orref_model_handle;
    skip_bad_fc_obs = skip_bad;
    enkf_verbose = 0;
    das_getHE(&das);
    memcpy(HE, das.S[0], (size_t) nrows * nobs * sizeof(float));
    for (o = 0; o < nobs; ++o)
        status[o] = data[o].status;
    free(das.S);
    for (t = 0; t < ntypes; ++t)
        free(types[t].name);
    free(types);
    free(data);
    free(nl);
    return 0;
}
