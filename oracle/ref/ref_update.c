/*
 * ref_update.c -- the reference's own update/update.c, compiled unmodified
 * inside this translation unit, with in-memory stand-ins for what its field
 * update reads from the model, grid and transforms file.  TEST
 * INFRASTRUCTURE ONLY: oracle/_ref/libenkf_ref_update.so pins the oracle's
 * restatement of das_updatefields and das_updatebg (update/update.c:92-814)
 * and of das_sethybridensemble (common/dasystem.c:775-819, compiled
 * unmodified into the same library) against the reference itself.
 *
 * das_updatefields and das_updatebg are static in update.c, so update.c is
 * included here and the entry points below call them directly.  What they
 * reach outside update.c is supplied in memory:
 *   - the model: one variable on one grid (its log flag, inflation,
 *     inflation ratio, and its deflation and sigma: NaN unless
 *     ref_set_noise gave them, in which case das_updatefields ends with
 *     addnoise, drawing its normals with get_normalpair from utils.c);
 *   - the grid: size, stride, surface layer id, periodic flag, numlevels;
 *   - the transforms file (transforms.nc, read through ncw_*): T
 *     [nj][ni][m_dyn][m] and w [nj][ni][m] arrays and the stride attribute.
 * update.c also calls MPI_Barrier outside its `#if defined(MPI)` guards (in
 * functions these entry points never reach); it is declared here as a
 * no-op so that the file compiles without MPI.
 */
#define MPI_COMM_WORLD 0
int MPI_Barrier(int comm);

#include "update.c"

int MPI_Barrier(int comm)
{
    (void) comm;
    return 0;
}

/* ---- the in-memory model, grid and transforms file ---- */

typedef struct {
    int id;
    int stride;
    int mni, mnj;
    int surfk;
    int periodic_i;
    int** numlevels;            /* row pointers [mnj][mni] */
} orref_grid;

typedef struct {
    orref_grid* g;
    int applylog;
    float inflation;
    double inf_ratio;
} orref_model;

static struct {
    int nj, ni, nmem_dynamic, nmem, stride;
    const float* T;             /* [nj][ni][nmem_dynamic][nmem] or NULL */
    const float* w;             /* [nj][ni][nmem] */
} orref_tf;

void* model_getvargrid(model* m, int vid)
{
    (void) vid;
    return ((orref_model*) m)->g;
}

int model_getvarislog(model* m, int vid)
{
    (void) vid;
    return ((orref_model*) m)->applylog;
}

void model_getvarinflation(model* m, int varid, float* inflation, double* inf_ratio)
{
    (void) varid;
    *inflation = ((orref_model*) m)->inflation;
    *inf_ratio = ((orref_model*) m)->inf_ratio;
}

static double orref_deflation = NAN, orref_sigma = NAN;

double model_getvardeflation(model* m, int varid)
{
    (void) m;
    (void) varid;
    return orref_deflation;
}

double model_getvarsigma(model* m, int varid)
{
    (void) m;
    (void) varid;
    return orref_sigma;
}

void model_getvargridsize(model* m, int vid, int* ni, int* nj, int* nk)
{
    orref_grid* g = ((orref_model*) m)->g;

    (void) vid;
    if (ni != NULL)
        *ni = g->mni;
    if (nj != NULL)
        *nj = g->mnj;
    if (nk != NULL)
        *nk = 1;
}

int model_getngrid(model* m)
{
    (void) m;
    return 1;
}

void* model_getgridbyid(model* m, int gridid)
{
    (void) gridid;
    return ((orref_model*) m)->g;
}

int grid_getid(grid* g)
{
    return ((orref_grid*) g)->id;
}

int grid_getstride(grid* g)
{
    return ((orref_grid*) g)->stride;
}

void* grid_getnumlevels(grid* g)
{
    return ((orref_grid*) g)->numlevels;
}

int grid_getsurflayerid(grid* g)
{
    return ((orref_grid*) g)->surfk;
}

int grid_isperiodic_i(grid* g)
{
    return ((orref_grid*) g)->periodic_i;
}

void grid_getsize(grid* g, int* ni, int* nj, int* nk)
{
    if (ni != NULL)
        *ni = ((orref_grid*) g)->mni;
    if (nj != NULL)
        *nj = ((orref_grid*) g)->mnj;
    if (nk != NULL)
        *nk = 1;
}

char* grid_getname(grid* g)
{
    (void) g;
    return "grid";
}

int grid_getaliasid(grid* g)
{
    (void) g;
    return -1;
}

void ncw_open(const char fname[], int mode, int* ncid)
{
    (void) fname;
    (void) mode;
    *ncid = 1;
}

void ncw_close(int ncid)
{
    (void) ncid;
}

void ncw_inq_varid(int ncid, const char varname[], int* varid)
{
    (void) ncid;
    if (strcmp(varname, "T") == 0 && orref_tf.T != NULL)
        *varid = 0;
    else if (strcmp(varname, "w") == 0)
        *varid = 1;
    else
        enkf_quit("ref_update: no variable \"%s\" in the in-memory transforms", varname);
}

void ncw_inq_vardims(int ncid, int varid, int maxndims, int* ndims, size_t dimlen[])
{
    int n = (varid == 0) ? 4 : 3;

    (void) ncid;
    if (ndims != NULL)
        *ndims = n;
    if (maxndims < n)
        enkf_quit("ref_update: maxndims = %d < %d", maxndims, n);
    dimlen[0] = orref_tf.nj;
    dimlen[1] = orref_tf.ni;
    if (varid == 0) {
        dimlen[2] = orref_tf.nmem_dynamic;
        dimlen[3] = orref_tf.nmem;
    } else
        dimlen[2] = orref_tf.nmem;
}

void ncw_get_att_int(int ncid, int varid, const char attname[], int v[])
{
    (void) ncid;
    (void) varid;
    if (strcmp(attname, "stride") != 0)
        enkf_quit("ref_update: no attribute \"%s\"", attname);
    v[0] = orref_tf.stride;
}

/* Reads whole rows j (start[0], count[0] = 1) with every other index at 0
 * and full extent, which is how update.c reads T and w. */
void ncw_get_vara_float(int ncid, int varid, const size_t start[], const size_t count[], float v[])
{
    size_t row = (size_t) orref_tf.ni * orref_tf.nmem * (varid == 0 ? orref_tf.nmem_dynamic : 1);
    const float* src = (varid == 0) ? orref_tf.T : orref_tf.w;

    (void) ncid;
    if (start[0] >= (size_t) orref_tf.nj || count[0] != 1 || start[1] != 0 || count[1] != (size_t) orref_tf.ni)
        enkf_quit("ref_update: unexpected hyperslab");
    memcpy(v, src + start[0] * row, row * sizeof(float));
}

/* ---- entry points ---- */

/* The grid and model for one field-layer; rows of numlevels as pointers. */
static int** orref_rows_int(int* a, int nj, int ni)
{
    int** r = malloc(nj * sizeof(int*));
    int j;

    for (j = 0; j < nj; ++j)
        r[j] = a + (size_t) j * ni;
    return r;
}

/* fieldbuffer layout of update.c: v[e][j][i] over [nmem][jsize][mni] */
static float*** orref_rows3(float* v, int nmem, int jsize, int mni)
{
    float*** r = malloc(nmem * sizeof(float**));
    int e, j;

    for (e = 0; e < nmem; ++e) {
        r[e] = malloc(jsize * sizeof(float*));
        for (j = 0; j < jsize; ++j)
            r[e][j] = v + ((size_t) e * jsize + j) * mni;
    }
    return r;
}

static void orref_free3(float*** r, int nmem)
{
    int e;

    for (e = 0; e < nmem; ++e)
        free(r[e]);
    free(r);
}

/*
 * das_updatefields (mode ENKF or HYBRID) or das_updatebg (mode ENOI) over
 * model rows j1..j2 of one field-layer.  mode: the reference's codes
 * (MODE_ENKF, MODE_ENOI, MODE_HYBRID of common/global.h).
 *   v        [nmem (+1 for ENOI: the background last)][j2-j1+1][mni], in place
 *   T, w     the transforms: T [nj][ni][nmem_dynamic][nmem] (NULL for ENOI),
 *            w [nj][ni][nmem], nj = (mnj-1)/stride+1, ni = (mni-1)/stride+1
 *   numlevels [mnj][mni]
 */
int ref_update_layer(int mode, int nmem, int nmem_dynamic, int stride, int periodic_i, int mni, int mnj,
                     int j1, int j2, int level, int surfk, int issurfacevar, float inflation, double inf_ratio,
                     int output_increment, int applylog, const float* T, const float* w, int* numlevels,
                     float* v)
{
    orref_grid g;
    orref_model mdl;
    dasystem das;
    field f;
    void* buf[1];
    int jsize = j2 - j1 + 1;
    int nrows = (mode == MODE_ENOI) ? nmem + 1 : nmem;
    float*** rows;

    memset(&g, 0, sizeof(g));
    g.id = 0;
    g.stride = stride;
    g.mni = mni;
    g.mnj = mnj;
    g.surfk = surfk;
    g.periodic_i = periodic_i;
    g.numlevels = orref_rows_int(numlevels, mnj, mni);
    mdl.g = &g;
    mdl.applylog = applylog;
    mdl.inflation = inflation;
    mdl.inf_ratio = inf_ratio;

    orref_tf.nj = (mnj - 1) / stride + 1;
    orref_tf.ni = (mni - 1) / stride + 1;
    orref_tf.nmem_dynamic = nmem_dynamic;
    orref_tf.nmem = nmem;
    orref_tf.stride = stride;
    orref_tf.T = (mode == MODE_ENOI) ? NULL : T;
    orref_tf.w = w;

    memset(&das, 0, sizeof(das));
    das.mode = mode;
    das.nmem = nmem;
    das.nmem_dynamic = (mode == MODE_ENOI) ? nmem : nmem_dynamic;
    das.nmem_static = nmem - das.nmem_dynamic;
    das.m = (model*) & mdl;
    das.updatespec = output_increment ? UPDATE_OUTPUTINC : 0;

    memset(&f, 0, sizeof(f));
    f.id = 0;
    f.varid = 0;
    f.issurfacevar = issurfacevar;
    f.level = level;
    f.isstructured = 1;
    f.j1 = j1;
    f.j2 = j2;

    rows = orref_rows3(v, nrows, jsize, mni);
    buf[0] = rows;
    if (mode == MODE_ENOI)
        das_updatebg(&das, 1, buf, &f);
    else
        das_updatefields(&das, 1, buf, &f);
    orref_free3(rows, nrows);
    free(g.numlevels);
    return 0;
}

/* DEFLATION and SIGMA of the variable of the next ref_update_layer (NaN
 * deflation: no RANDOMISE); the generator state of drand48, which
 * get_normalpair (common/utils.c:1477-1484) draws from; and one pair. */
void ref_set_noise(double deflation, double sigma)
{
    orref_deflation = deflation;
    orref_sigma = sigma;
}

void ref_srand48(long seed)
{
    srand48(seed);
}

void ref_normalpair(double* x)
{
    get_normalpair(x);
}

/* das_sethybridensemble on v [nmem + 2][nij] (rows nmem, nmem + 1 hold the
 * double mean, as the reference allocates them). */
int ref_sethybridensemble(int nmem, int nmem_dynamic, double gamma, int nij, float* v)
{
    dasystem das;
    float** rows = malloc((nmem + 2) * sizeof(float*));
    int e;

    memset(&das, 0, sizeof(das));
    das.mode = MODE_HYBRID;
    das.nmem = nmem;
    das.nmem_dynamic = nmem_dynamic;
    das.nmem_static = nmem - nmem_dynamic;
    das.gamma = gamma;
    for (e = 0; e < nmem + 2; ++e)
        rows[e] = v + (size_t) e * nij;
    das_sethybridensemble(&das, nij, rows);
    free(rows);
    return 0;
}
