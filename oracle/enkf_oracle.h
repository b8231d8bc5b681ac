/*
 * enkf_oracle.h -- CPU oracle for the EnKF-C analysis hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the GPU library is compared
 * against, and the CPU baseline that is timed beside it.  Only the tests, the
 * smoke check and the CPU-baseline leg of the benchmark load it; the product
 * (libenkfg) never links, loads or calls anything from here.
 *
 * Every function restates, in plain C99, the reference routine cited in its
 * comment (paths are relative to the reference's enkf/ directory).  Floating
 * point semantics (which operations are float, which are double, the order of
 * accumulation) follow the reference line by line, and the file is compiled
 * with -ffp-contract=off so that neither x86 nor Arm fuses a multiply-add the
 * reference's -std=c99 -O2 build would not fuse.
 */
#ifndef ENKF_ORACLE_H
#define ENKF_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define OR_MAXLOCRAD 8
#define OR_MODE_ENKF 0
#define OR_MODE_ENOI 1
#define OR_MODE_HYBRID 2
#define OR_SCHEME_DENKF 0
#define OR_SCHEME_ETKF 1

typedef struct or_obsset or_obsset;

/* Observation set + per-type kd-trees (observations.c:1616-1733). lon/lat are
 * the float observation coordinates; locrad/locweight are [ntypes][OR_MAXLOCRAD].
 * nlobsmax[t] <= 0 means "no limit" (INT_MAX in the reference). */
or_obsset* or_obs_create(int nobs, const float* lon, const float* lat, const short* type, const short* status, int ntypes, const int* nlocrad, const double* locrad, const double* locweight, const int* nlobsmax, int geographic);
void or_obs_destroy(or_obsset* obs);

/* obs_findlocal (observations.c:1837-1927). Writes up to `cap` ids/coefficients
 * in the reference's order (type, then kd-tree depth-first order) and returns
 * the count; returns -(count) when cap is too small (nothing valid written). */
int or_findlocal(const or_obsset* obs, double x, double y, int* ids, double* lcoeffs, int cap);

/* Gaspari-Cohn taper (utils.c:1425-1443) and obstype_calclcoeff
 * (obstypes.c:800-809). */
double or_taper_gc(double x);
double or_calclcoeff(int nlocrad, const double* locrad, const double* locweight, double dist);

/* Per-point numerics (calcs.c).  S is Fortran p x m, i.e. row-major [m][p].
 * scheme/mode as above.  Outputs: w[m]; T row-major [m][m] with T[e1][e2]
 * (e1 < mout) as in the reference; G row-major [p][m] (Fortran m x p).
 * Returns 0, or the LAPACK info code on a factorisation failure. */
int or_calc_wT(int mode, int scheme, int m, int mout, int p, const double* s, double* S, double* w, double* T, double* G);

/* traceprod (calcs.c:41-97), compact storage only. */
double or_traceprod(int transposeA, int transposeB, int m, int n, const double* A, const double* B);

typedef struct {
    int mode, scheme;
    int nmem, nmem_dynamic;
    double alpha;
    int stride;
    int mni, mnj;
    const double* x;            /* rectangular grid: x[mni] */
    const double* y;            /* rectangular grid: y[mnj] */
    const double* x2d;          /* curvilinear: [mnj][mni] (or NULL) */
    const double* y2d;
    int ii0, ii1;               /* strided columns ii0 <= ii < ii1 (ii1 <= 0: all) */
} or_calcparams;

/* das_calctransforms inner loop (transforms.c:1150-1360) over strided rows
 * jj in [jj0, jj1) (and the strided columns p->ii0 .. p->ii1 - 1 of each).  All output arrays are full-size (indexed by the strided
 * row): T float [nj][ni][m_dyn][m] (NULL for EnOI), w float [nj][ni][m],
 * T64/w64 the same in double before the float cast (NULL to skip), nlobs/dfs/
 * srf [nj][ni], pnlobs/pdfs/psrf [ntypes][nj][ni] (NULL to skip).  S is
 * standardised float [nmem][nobs], s standardised innovations [nobs].
 * Returns 0 or the first LAPACK failure code. */
int or_calctransforms(const or_obsset* obs, const or_calcparams* p, const float* S, const double* s, const short* type, int jj0, int jj1, float* T, float* w, double* T64, double* w64, int* nlobs, float* dfs, float* srf, int* pnlobs, float* pdfs, float* psrf);

/* das_calcinnandspread (ensobs.c:541-690), S_MODE_HE_f branch: S holds HE
 * [nmem][nobs] on entry and HA on exit. */
void or_calcinnandspread(int nmem, int nobs, float* S, const float* value, const short* status, double* s_f, double* std_f);

/* das_standardise (ensobs.c:849-898). rfactor is per type. */
void or_standardise(int nmem, int nobs, float* S, double* s_f, const float* estd, const short* type, const double* rfactor);

/* ll2xyz (utils.c:1449-1458): lon/lat in degrees to xyz on the sphere of
 * radius 6371 km. */
void or_ll2xyz(const double in[2], double out[3]);

/* Forward operator on a structured grid, footprint 0.
 * or_interp2d: interpolate2d_structured (utils.c:1140-1210); v [nj][ni],
 * mask [nj][ni] (numlevels, nonzero = wet).
 * or_interp3d: interpolate3d_structured (utils.c:1252-1366); v [nk][nj][ni],
 * nlevels [nj][ni], ktop the surface layer (0 or nk - 1).
 * Both return NaN and set *badpos where the reference's index assert would
 * fail (the position is off the grid). */
float or_interp2d(double fi, double fj, int ni, int nj, const float* v, const int* mask, int periodic_i, int* badpos);
float or_interp3d(double fi, double fj, double fk, int ni, int nj, int nk, int ktop, const float* v, const int* nlevels, int periodic_i, int* badpos);

/* H_surf_standard / H_subsurf_standard (model2obs.c:127-181, 256-348) with
 * evaluate_2d_obs / interpolate_3d_obs (model2obs.c:37-124) for one member:
 * the observations ids[nids] (all of one type) are interpolated from field
 * (2-D: [nj][ni], the surface layer; 3-D: [nk][nj][ni]) minus the OFFSET data
 * (offset_kind 0 none, 1 [nk], 2 [nj][ni], 3 [nk][nj][ni]) into dst[id].
 * A value that is not finite or exceeds 999999 in magnitude becomes NaN when
 * skip_bad, else the call stops and returns 1 + the observation id (the
 * reference quits there).  Returns -(1 + id) for a position off the grid. */
int or_map_obs(int three_d, int ni, int nj, int nk, int ktop, int periodic_i, const int* numlevels, const float* offset, int offset_kind, const float* field, int nids, const int* ids, const double* fi, const double* fj, const float* fk, int skip_bad, float* dst);

/* End of das_getHE (ensobs.c:372-490) on HE [nmem][nobs] (and the EnOI
 * background row Hx [nobs]): with skip_bad, observations with a NaN forecast
 * get status 10 (STATUS_BADFC); then EnOI: S_e += Hx - mean (float); hybrid:
 * dynamic anomalies scaled by k_d and static ones by k_s about their own
 * means, both recentred on the dynamic mean.  Returns the number of
 * observations with status 10. */
int or_finish_HE(int mode, int nmem, int nmem_d, double gamma, int nobs, float* S, const float* Hx, int skip_bad, short* status);

typedef struct {
    int mode;                   /* OR_MODE_ENKF / OR_MODE_HYBRID (fields), OR_MODE_ENOI (bg) */
    int nmem, nmem_dynamic;
    int stride, periodic_i;
    int mni, mnj;               /* model grid */
    int ni, nj;                 /* strided transforms grid */
    int j1, j2;                 /* rows of this field tile, j1 % stride == 0 */
    int level, surfk, issurfacevar;
    float inflation0;
    double inf_ratio;           /* NaN: plain multiplicative inflation */
    int output_increment, applylog;
} or_updateparams;

/* das_updatefields (update.c:92-564) for one field (structured grid).
 * v is float [nmem][j2-j1+1][mni], updated in place; numlevels [mnj][mni];
 * infl (or NULL) receives [j2-j1+1][mni] inflation. */
int or_updatefields(const or_updateparams* p, const float* T, const float* w, const int* numlevels, float* v, float* infl);

/* das_updatebg (update.c:568-814): v is [nmem + 1][jsize][mni], slot nmem is
 * the background, updated in place. */
int or_updatebg(const or_updateparams* p, const float* w, const int* numlevels, float* v);

/* das_sethybridensemble (dasystem.c:775-819). v is [nmem][nij]; vmean
 * receives the double dynamic mean [nij]. */
void or_sethybridensemble(int nmem, int nmem_d, int nmem_s, double gamma, int nij, float* v, double* vmean);

/* addnoise (update.c:46-87) on one field of nmem members of ncell cells,
 * v [nmem][ncell] in place; random holds at least nmem standard normals
 * (copied: the member mean is removed from the copy). */
void or_addnoise(int nmem, long ncell, double deflation, double sigma, const double* random, float* v);

#ifdef __cplusplus
}
#endif
#endif
