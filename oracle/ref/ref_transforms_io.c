/*
 * ref_transforms_io.c -- link glue for oracle/_ref/libenkf_ref_transforms.so
 * (see ref_transforms.c).  TEST INFRASTRUCTURE ONLY.
 *
 * In-memory stand-ins for what das_calctransforms reads outside the
 * reference files compiled into the library: one model grid with one
 * variable (its size, stride, name, domain, coordinates of integer (i, j) =
 * (x[i], y[j]) as for a rectangular grid, the geographic flag), the
 * distribution of all iterations to this one process, and the NetCDF
 * wrappers of the transforms and diagnostics files, whose variable writes
 * are copied into the arrays ref_calctransforms was given; and
 * kd_printinfo, a print; and the point-log writer, whose transforms are
 * copied into the arrays ref_calcpointlogtransforms was given.  Everything else
 * the compiled files name (file input of observations and obstypes, point
 * logs) aborts if reached.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static struct {
    int mni, mnj, stride, geographic;
    const double* x;
    const double* y;
    int nj, ni, md, m, ntypes;
    float* T;
    float* w;
    int* nlobs;
    float* dfs;
    float* srf;
    int* pnlobs;
    float* pdfs;
    float* psrf;
} tio;

void orref_tio_set(int mni, int mnj, const double* x, const double* y, int stride, int geographic, int nj, int ni,
                   int md, int m, int ntypes, float* T, float* w, int* nlobs, float* dfs, float* srf, int* pnlobs,
                   float* pdfs, float* psrf)
{
    tio.mni = mni;
    tio.mnj = mnj;
    tio.x = x;
    tio.y = y;
    tio.stride = stride;
    tio.geographic = geographic;
    tio.nj = nj;
    tio.ni = ni;
    tio.md = md;
    tio.m = m;
    tio.ntypes = ntypes;
    tio.T = T;
    tio.w = w;
    tio.nlobs = nlobs;
    tio.dfs = dfs;
    tio.srf = srf;
    tio.pnlobs = pnlobs;
    tio.pdfs = pdfs;
    tio.psrf = psrf;
}

static void unreachable(const char* name)
{
    fprintf(stderr, "ref_transforms_io: %s is not available in this build\n", name);
    abort();
}

/* a diagnostic print of obs_createkdtrees (common/utils.c defines it only
 * for enkf_calc builds) */
void kd_printinfo(void* tree, char* offset)
{
    (void) tree;
    (void) offset;
}

/* ---- the model and its grid ---- */
static int orref_grid_handle;

int model_getngrid(void* m) { (void) m; return 1; }
void* model_getgridbyid(void* m, int id) { (void) m; (void) id; return &orref_grid_handle; }
int model_getnvar(void* m) { (void) m; return 1; }
int model_getvargridid(void* m, int vid) { (void) m; (void) vid; return 0; }
char* grid_getname(void* g) { (void) g; return "grid"; }
char* grid_getdomainname(void* g) { (void) g; return "grid"; }
int grid_getaliasid(void* g) { (void) g; return -1; }
int grid_getstride(void* g) { (void) g; return tio.stride; }
int grid_isgeographic(void* g) { (void) g; return tio.geographic; }

void grid_getsize(void* g, int* ni, int* nj, int* nk)
{
    (void) g;
    if (ni != NULL)
        *ni = tio.mni;
    if (nj != NULL)
        *nj = tio.mnj;
    if (nk != NULL)
        *nk = 1;
}

void grid_ij2xy(void* g, int* ij, double* x, double* y)
{
    (void) g;
    *x = tio.x[ij[0]];
    *y = tio.y[ij[1]];
}

/* ---- the distribution of iterations: all to this process ---- */
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

void das_getfname_transforms(void* das, int gridid, char fname[])
{
    (void) das;
    snprintf(fname, 64, "transforms-%d.nc", gridid);
}

/* ---- NetCDF: variable writes land in the caller's arrays ---- */
static const char* varnames[] = { "T", "w", "nlobs", "dfs", "srf", "pnlobs", "pdfs", "psrf" };
#define NVARS ((int) (sizeof(varnames) / sizeof(varnames[0])))

static int varid_of(const char* name)
{
    int i;

    for (i = 0; i < NVARS; ++i)
        if (strcmp(name, varnames[i]) == 0)
            return i;
    unreachable(name);
    return -1;
}

typedef void (*orref_quit_fn) (char* format, ...);
void ncw_set_quitfn(orref_quit_fn f) { (void) f; }
void ncu_set_quitfn(orref_quit_fn f) { (void) f; }
void ncw_create(const char fname[], int mode, int* ncid) { (void) fname; (void) mode; *ncid = 1; }
void ncw_open(const char fname[], int mode, int* ncid) { (void) fname; (void) mode; *ncid = 1; }
void ncw_close(int ncid) { (void) ncid; }
void ncw_enddef(int ncid) { (void) ncid; }
void ncw_def_deflate(int ncid, int shuffle, int deflate, int level) { (void) ncid; (void) shuffle; (void) deflate; (void) level; }
void ncw_def_dim(int ncid, const char name[], size_t len, int* dimid) { (void) ncid; (void) name; (void) len; *dimid = 0; }
void ncw_def_var(int ncid, const char name[], int type, int ndims, const int dimids[], int* varid)
{
    (void) ncid;
    (void) type;
    (void) ndims;
    (void) dimids;
    *varid = varid_of(name);
}
void ncw_inq_varid(int ncid, const char name[], int* varid) { (void) ncid; *varid = varid_of(name); }
void ncw_put_att_int(int ncid, int varid, const char name[], size_t len, const int v[]) { (void) ncid; (void) varid; (void) name; (void) len; (void) v; }
void ncw_put_att_text(int ncid, int varid, const char name[], const char v[]) { (void) ncid; (void) varid; (void) name; (void) v; }
int nc_def_var_chunking(int ncid, int varid, int storage, const size_t* chunks) { (void) ncid; (void) varid; (void) storage; (void) chunks; return 0; }

void ncw_put_vara_float(int ncid, int varid, const size_t start[], const size_t count[], const float v[])
{
    (void) ncid;
    if (varid == 0) {
        const size_t row = (size_t) tio.ni * tio.md * tio.m;

        memcpy(tio.T + start[0] * row, v, count[1] * count[2] * count[3] * sizeof(float));
    } else if (varid == 1) {
        const size_t row = (size_t) tio.ni * tio.m;

        memcpy(tio.w + start[0] * row, v, count[1] * count[2] * sizeof(float));
    } else
        unreachable("ncw_put_vara_float");
}

void ncw_put_var_int(int ncid, int varid, const int v[])
{
    const size_t n = (size_t) tio.nj * tio.ni;

    (void) ncid;
    if (varid == 2)
        memcpy(tio.nlobs, v, n * sizeof(int));
    else if (varid == 5)
        memcpy(tio.pnlobs, v, tio.ntypes * n * sizeof(int));
    else
        unreachable("ncw_put_var_int");
}

void ncw_put_var_float(int ncid, int varid, const float v[])
{
    const size_t n = (size_t) tio.nj * tio.ni;

    (void) ncid;
    if (varid == 3)
        memcpy(tio.dfs, v, n * sizeof(float));
    else if (varid == 4)
        memcpy(tio.srf, v, n * sizeof(float));
    else if (varid == 6)
        memcpy(tio.pdfs, v, tio.ntypes * n * sizeof(float));
    else if (varid == 7)
        memcpy(tio.psrf, v, tio.ntypes * n * sizeof(float));
    else
        unreachable("ncw_put_var_float");
}

/* ---- the point-log writer: the transforms land in the caller's arrays ---- */
static struct {
    int nmem;
    double* T;                  /* [nplog][nmem][nmem] or NULL */
    double* w;                  /* [nplog][nmem] */
} plo;

void orref_plog_set(int nmem, double* T, double* w)
{
    plo.nmem = nmem;
    plo.T = T;
    plo.w = w;
}

void das_createplog(void* das, int plogid, int ploc, int* lobs, double* lcoeffs)
{
    (void) das;
    (void) plogid;
    (void) ploc;
    (void) lobs;
    (void) lcoeffs;
}

void das_writeplogtransform(void* das, int plogid, int gid, int ploc, double* s, double* S, double* w, double* T)
{
    const size_t m = (size_t) plo.nmem;

    (void) das;
    (void) gid;
    (void) ploc;
    (void) s;
    (void) S;
    memcpy(plo.w + (size_t) plogid * m, w, m * sizeof(double));
    if (T != NULL && plo.T != NULL)
        memcpy(plo.T + (size_t) plogid * m * m, T, m * m * sizeof(double));
}

/* ---- not reached by das_calctransforms ---- */
#define UNREACHABLE(name) void name(void) { unreachable(#name); }

UNREACHABLE(ncw_att_exists)
UNREACHABLE(model_adddata)
UNREACHABLE(model_getdomainid)
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
UNREACHABLE(ncw_inq_varnatts)
UNREACHABLE(ncw_put_var_uchar)
UNREACHABLE(ncw_var_exists)
