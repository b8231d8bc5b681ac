/*
 * ref_transforms.c -- entry point into the reference's own calc/transforms.c
 * (das_calctransforms, compiled unmodified with calc/calcs.c,
 * common/observations.c, common/obstypes.c and common/kdtree.c) for
 * oracle/_ref/libenkf_ref_transforms.so.  TEST INFRASTRUCTURE ONLY: pins the
 * oracle's restatement of the transform stage -- the loop over the strided
 * grid, the search, the gather and taper, the solves, the relaxation, the
 * float cast and the diagnostics (calc/transforms.c:991-1637) -- against the
 * reference itself.
 *
 * What das_calctransforms reads outside those files is supplied in memory
 * (ref_transforms_io.c): one model grid (rectangular coordinates x[i],
 * y[j], a stride, the geographic flag) with one variable on it, the
 * distribution of all rows to this one process, and the transforms and
 * diagnostics files, whose writes land in the caller's arrays.  S and s come
 * in standardised: das_standardise, which das_calctransforms calls first,
 * is pinned on its own (ref_ensobs.c) and here only advances the state.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include "ncw.h"
#include "global.h"
#include "utils.h"
#include "observations.h"
#include "dasystem.h"
#include "pointlog.h"

observations* orref_obs_build(int nobs, const float* lon, const float* lat, const short* type, const short* status,
                              const float* value, const float* estd, int ntypes, int maxlocrad, const int* nlocrad,
                              const double* locrad, const double* locweight, const int* nlobsmax,
                              const int* visible, int geographic, const double* rfactor);
void orref_obs_free(observations* obs);
void orref_tio_set(int mni, int mnj, const double* x, const double* y, int stride, int geographic, int nj, int ni,
                   int md, int m, int ntypes, float* T, float* w, int* nlobs, float* dfs, float* srf, int* pnlobs,
                   float* pdfs, float* psrf);

void orref_plog_set(int nmem, double* T, double* w);

/* das_standardise (calc/ensobs.c:849-898) is pinned separately; the data
 * come in standardised */
void das_standardise(dasystem* das)
{
    if (das->s_mode == S_MODE_HA_f)
        das->s_mode = S_MODE_S_f;
    else if (das->s_mode == S_MODE_HA_a)
        das->s_mode = S_MODE_S_a;
}

/*
 * das_calctransforms on one mni x mnj rectangular grid (x[mni], y[mnj]) at
 * the given stride.  mode, scheme: the reference's codes (MODE_ENKF 1, ENOI
 * 2, HYBRID 3; SCHEME_DENKF 1, ETKF 2).  S [nmem][nobs] (float) and s
 * [nobs] standardised.  Outputs: T [nj][ni][nmem_dynamic][nmem] (ENKF and
 * HYBRID), w [nj][ni][nmem], nlobs, dfs, srf [nj][ni], pnlobs, pdfs, psrf
 * [ntypes][nj][ni], nj = (mnj - 1) / stride + 1, ni = (mni - 1) / stride + 1.
 */
int ref_calctransforms(int mode, int scheme, double alpha, int nmem, int nmem_dynamic, int nobs, const float* lon,
                       const float* lat, const short* type, const short* status, float* S, double* s, int ntypes,
                       int maxlocrad, const int* nlocrad, const double* locrad, const double* locweight,
                       const int* nlobsmax, const int* visible, int geographic, int mni, int mnj, const double* x,
                       const double* y, int stride, float* T, float* w, int* nlobs, float* dfs, float* srf,
                       int* pnlobs, float* pdfs, float* psrf)
{
    dasystem das;
    observations* obs = orref_obs_build(nobs, lon, lat, type, status, NULL, NULL, ntypes, maxlocrad, nlocrad, locrad,
                                        locweight, nlobsmax, visible, geographic, NULL);
    float** rows = malloc((nmem > 0 ? nmem : 1) * sizeof(float*));
    const int nj = (mnj - 1) / stride + 1, ni = (mni - 1) / stride + 1;
    int e;

    orref_tio_set(mni, mnj, x, y, stride, geographic, nj, ni, nmem_dynamic, nmem, ntypes, T, w, nlobs, dfs, srf,
                  pnlobs, pdfs, psrf);
    for (e = 0; e < nmem; ++e)
        rows[e] = S + (size_t) e * nobs;
    memset(&das, 0, sizeof(das));
    das.mode = mode;
    das.scheme = scheme;
    das.alpha = alpha;
    das.nmem = nmem;
    das.nmem_dynamic = nmem_dynamic;
    das.nmem_static = nmem - nmem_dynamic;
    das.obs = obs;
    das.S = rows;
    das.s_f = s;
    das.s_mode = S_MODE_HA_f;
    das.m = (model*) &das;      /* any non-NULL handle: the model stand-ins ignore it */
    enkf_verbose = 0;
    das_calctransforms(&das);
    free(rows);
    orref_obs_free(obs);
    return 0;
}

/*
 * das_calcpointlogtransforms (calc/transforms.c:1646-1773) at npl log points
 * (plon, plat) on the one model grid (geographic as given): the double T
 * [npl][nmem][nmem] (ENKF and HYBRID) and w [npl][nmem] it hands to the
 * point-log writer, after the relaxation and before any float cast.
 */
int ref_calcpointlogtransforms(int mode, int scheme, double alpha, int nmem, int nmem_dynamic, int nobs,
                               const float* lon, const float* lat, const short* type, const short* status, float* S,
                               double* s, int ntypes, int maxlocrad, const int* nlocrad, const double* locrad,
                               const double* locweight, const int* nlobsmax, int geographic, int npl,
                               const double* plon, const double* plat, double* T, double* w)
{
    dasystem das;
    observations* obs = orref_obs_build(nobs, lon, lat, type, status, NULL, NULL, ntypes, maxlocrad, nlocrad, locrad,
                                        locweight, nlobsmax, NULL, geographic, NULL);
    float** rows = malloc((nmem > 0 ? nmem : 1) * sizeof(float*));
    pointlog* plogs = calloc(npl > 0 ? npl : 1, sizeof(pointlog));
    static const double x0 = 0.0;
    int e, k;

    orref_tio_set(1, 1, &x0, &x0, 1, geographic, 1, 1, nmem_dynamic, nmem, ntypes, NULL, NULL, NULL, NULL, NULL,
                  NULL, NULL, NULL);
    orref_plog_set(nmem, T, w);
    for (k = 0; k < npl; ++k) {
        plogs[k].id = k;
        plogs[k].lon = plon[k];
        plogs[k].lat = plat[k];
        plogs[k].gridid = -1;
    }
    for (e = 0; e < nmem; ++e)
        rows[e] = S + (size_t) e * nobs;
    memset(&das, 0, sizeof(das));
    das.mode = mode;
    das.scheme = scheme;
    das.alpha = alpha;
    das.nmem = nmem;
    das.nmem_dynamic = nmem_dynamic;
    das.nmem_static = nmem - nmem_dynamic;
    das.obs = obs;
    das.S = rows;
    das.s_f = s;
    das.s_mode = S_MODE_S_f;
    das.m = (model*) &das;
    das.nplog = npl;
    das.plogs = plogs;
    enkf_verbose = 0;
    das_calcpointlogtransforms(&das);
    free(plogs);
    free(rows);
    orref_obs_free(obs);
    return 0;
}
