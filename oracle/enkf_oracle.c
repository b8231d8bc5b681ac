/*
 * enkf_oracle.c -- CPU restatement of the EnKF-C analysis hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the CPU
 * baseline timed beside it.  Nothing in the product links or loads it.
 *
 * Each function cites the reference lines it restates (paths relative to the
 * reference's enkf/ directory).  Compile with -std=c99 -O2 -ffp-contract=off.
 */
#define _GNU_SOURCE
#include <assert.h>
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "enkf_oracle.h"
#include "or_blas.h"

#define OR_REARTH 6371.0                     /* common/global.h:121 */
#define OR_DEG2RAD (M_PI / 180.0)            /* common/global.h:122 */
#define OR_MAXOBSVAL 999999.0                /* common/global.h:119 */
#define OR_DFS_MIN 1.0e-6                    /* calc/transforms.c:32 */
#define OR_EPSF 1.0e-6f                      /* update/update.c:40 */
#define OR_NONE SIZE_MAX

/* ---------------------------------------------------------------------------
 * kd-tree: sequential insertion and depth-first range search with the same
 * split rule and pruning test as common/kdtree.c:194-215 (insert) and
 * 516-540 (search).  Storage is this file's own.
 * ------------------------------------------------------------------------- */
typedef struct {
    size_t left, right;
    int dir;
} or_kdnode;

typedef struct {
    int ndim;
    size_t n, cap;
    or_kdnode* nodes;
    double* coords;
} or_kdtree;

typedef struct {
    size_t id;
    double distsq;
} or_kdres;

static void kd_init(or_kdtree* t, int ndim, size_t cap)
{
    t->ndim = ndim;
    t->n = 0;
    t->cap = cap > 0 ? cap : 1;
    t->nodes = malloc(t->cap * sizeof(or_kdnode));
    t->coords = malloc(t->cap * ndim * sizeof(double));
}

static void kd_free(or_kdtree* t)
{
    free(t->nodes);
    free(t->coords);
}

/* kd_insertnode (kdtree.c:253-274) -> _kd_insertnode (194-215) */
static void kd_insert(or_kdtree* t, const double* c)
{
    int nd = t->ndim;
    size_t id, newid;
    int k;

    if (!isfinite(c[0]))
        return;
    assert(t->n < t->cap);
    newid = t->n;
    for (k = 0; k < nd; ++k)
        t->coords[newid * nd + k] = c[k];
    t->nodes[newid].left = OR_NONE;
    t->nodes[newid].right = OR_NONE;
    t->nodes[newid].dir = 0;
    if (newid > 0) {
        id = 0;
        for (;;) {
            or_kdnode* node = &t->nodes[id];
            size_t* next = (c[node->dir] < t->coords[id * nd + node->dir]) ? &node->left : &node->right;

            if (*next == OR_NONE) {
                *next = newid;
                t->nodes[newid].dir = (node->dir + 1) % nd;
                break;
            }
            id = *next;
        }
    }
    t->n++;
}

/* _kd_findnodeswithinrange (kdtree.c:516-540), depth-first pre-order with an
 * explicit stack (near subtree first, far subtree only if |dx| < range). */
static size_t kd_range(const or_kdtree* t, const double* q, double range, or_kdres** res, size_t* rescap, size_t** stack, size_t* stackcap)
{
    int nd = t->ndim;
    size_t nres = 0, top = 0;

    if (t->n == 0)
        return 0;
    if (*stackcap < 64) {
        *stackcap = 64;
        *stack = realloc(*stack, *stackcap * sizeof(size_t));
    }
    (*stack)[top++] = 0;
    while (top > 0) {
        size_t id = (*stack)[--top];
        const or_kdnode* node = &t->nodes[id];
        const double* nc = &t->coords[id * nd];
        double distsq = 0.0, dx;
        size_t near, far;
        int i;

        for (i = 0; i < nd; i++)
            distsq += (nc[i] - q[i]) * (nc[i] - q[i]);
        if (distsq <= range * range) {
            if (nres >= *rescap) {
                *rescap = *rescap * 2 + 1024;
                *res = realloc(*res, *rescap * sizeof(or_kdres));
            }
            (*res)[nres].id = id;
            (*res)[nres].distsq = distsq;
            nres++;
        }
        dx = q[node->dir] - nc[node->dir];
        near = dx <= 0.0 ? node->left : node->right;
        far = dx <= 0.0 ? node->right : node->left;
        if (top + 2 > *stackcap) {
            *stackcap *= 2;
            *stack = realloc(*stack, *stackcap * sizeof(size_t));
        }
        if (fabs(dx) < range && far != OR_NONE)
            (*stack)[top++] = far;
        if (near != OR_NONE)
            (*stack)[top++] = near;
    }
    return nres;
}

/* stable merge sort by distance; kdtree.c:569-570 sorts with qsort() when a
 * limit on the number of local obs is set */
static void sort_by_dist(or_kdres* a, size_t n)
{
    or_kdres* tmp;
    size_t width, i;

    if (n < 2)
        return;
    tmp = malloc(n * sizeof(or_kdres));
    for (width = 1; width < n; width *= 2) {
        for (i = 0; i < n; i += 2 * width) {
            size_t lo = i, mid = i + width < n ? i + width : n, hi = i + 2 * width < n ? i + 2 * width : n;
            size_t l = lo, r = mid, k = lo;

            while (l < mid && r < hi)
                tmp[k++] = (a[r].distsq < a[l].distsq) ? a[r++] : a[l++];
            while (l < mid)
                tmp[k++] = a[l++];
            while (r < hi)
                tmp[k++] = a[r++];
        }
        memcpy(a, tmp, n * sizeof(or_kdres));
    }
    free(tmp);
}

/* ---------------------------------------------------------------------------
 * observation set
 * ------------------------------------------------------------------------- */
struct or_obsset {
    int nobs, ntypes, geographic;
    int* nlocrad;
    double* locrad;             /* [ntypes][OR_MAXLOCRAD] */
    double* locweight;
    int* nlobsmax;
    short* status;
    or_kdtree* trees;           /* [ntypes] */
    int** obsids;               /* [ntypes][nobs_t]: obs index of kd data */
    int* nobs_t;
};

/* ll2xyz (utils.c:1449-1458) */
void or_ll2xyz(const double in[2], double out[3])
{
    double lon = in[0] * OR_DEG2RAD;
    double lat = in[1] * OR_DEG2RAD;
    double coslat = cos(lat);

    out[0] = OR_REARTH * cos(lon) * coslat;
    out[1] = OR_REARTH * sin(lon) * coslat;
    out[2] = OR_REARTH * sin(lat);
}

/* obstype_getmaxlocrad (obstypes.c:813-822) */
static double maxlocrad(const or_obsset* o, int t)
{
    double max = 0.0;
    int i;

    for (i = 0; i < o->nlocrad[t]; ++i)
        if (o->locrad[t * OR_MAXLOCRAD + i] > max)
            max = o->locrad[t * OR_MAXLOCRAD + i];
    return max;
}

/* obs_createkdtrees (observations.c:1616-1733) with obs_find_bytype
 * (observations.c:1543-1565): one tree per type, nodes inserted in obs order,
 * status != OK excluded, 3-D (x,y,z on the sphere) if geographic else 2-D. */
or_obsset* or_obs_create(int nobs, const float* lon, const float* lat, const short* type, const short* status, int ntypes, const int* nlocrad, const double* locrad, const double* locweight, const int* nlobsmax, int geographic)
{
    or_obsset* o = calloc(1, sizeof(or_obsset));
    int t, i;

    o->nobs = nobs;
    o->ntypes = ntypes;
    o->geographic = geographic;
    o->nlocrad = malloc(ntypes * sizeof(int));
    o->nlobsmax = malloc(ntypes * sizeof(int));
    o->locrad = malloc(ntypes * OR_MAXLOCRAD * sizeof(double));
    o->locweight = malloc(ntypes * OR_MAXLOCRAD * sizeof(double));
    memcpy(o->nlocrad, nlocrad, ntypes * sizeof(int));
    memcpy(o->locrad, locrad, ntypes * OR_MAXLOCRAD * sizeof(double));
    memcpy(o->locweight, locweight, ntypes * OR_MAXLOCRAD * sizeof(double));
    for (t = 0; t < ntypes; ++t)
        o->nlobsmax[t] = (nlobsmax == NULL || nlobsmax[t] <= 0) ? INT_MAX : nlobsmax[t];
    o->status = malloc((nobs > 0 ? nobs : 1) * sizeof(short));
    memcpy(o->status, status, nobs * sizeof(short));
    o->trees = calloc(ntypes, sizeof(or_kdtree));
    o->obsids = calloc(ntypes, sizeof(int*));
    o->nobs_t = calloc(ntypes, sizeof(int));

    for (t = 0; t < ntypes; ++t) {
        int n = 0;

        for (i = 0; i < nobs; ++i)
            if (type[i] == t && status[i] == 0)
                n++;
        o->nobs_t[t] = n;
        o->obsids[t] = malloc((n > 0 ? n : 1) * sizeof(int));
        kd_init(&o->trees[t], geographic ? 3 : 2, n);
        for (i = 0, n = 0; i < nobs; ++i)
            if (type[i] == t && status[i] == 0)
                o->obsids[t][n++] = i;
        for (i = 0; i < n; ++i) {
            int id = o->obsids[t][i];
            double ll[2] = { lon[id], lat[id] };

            if (geographic) {
                double xyz[3];

                or_ll2xyz(ll, xyz);
                kd_insert(&o->trees[t], xyz);
            } else
                kd_insert(&o->trees[t], ll);
        }
    }
    return o;
}

void or_obs_destroy(or_obsset* o)
{
    int t;

    if (o == NULL)
        return;
    for (t = 0; t < o->ntypes; ++t) {
        kd_free(&o->trees[t]);
        free(o->obsids[t]);
    }
    free(o->trees);
    free(o->obsids);
    free(o->nobs_t);
    free(o->nlocrad);
    free(o->nlobsmax);
    free(o->locrad);
    free(o->locweight);
    free(o->status);
    free(o);
}

/* taper_gc (utils.c:1425-1443): Gaspari-Cohn 5th-order piecewise rational
 * function with support at x = 1 (x is doubled internally). */
double or_taper_gc(double x)
{
    double x2, x3, f;

    if (x >= 1.0)
        return 0.0;
    x *= 2.0;
    x2 = x * x;
    x3 = x2 * x;
    if (x < 1.0)
        f = 1.0 + x2 * (-x3 / 4.0 + x2 / 2.0) + x3 * (5.0 / 8.0) - x2 * (5.0 / 3.0);
    else
        f = x2 * (x3 / 12.0 - x2 / 2.0) + x3 * (5.0 / 8.0) + x2 * (5.0 / 3.0) - x * 5.0 + 4.0 - (2.0 / 3.0) / x;
    return (f >= 0.0) ? f : 0.0;
}

/* obstype_calclcoeff (obstypes.c:800-809) */
double or_calclcoeff(int nlocrad, const double* locrad, const double* locweight, double dist)
{
    double sum = 0.0;
    int i;

    for (i = 0; i < nlocrad; ++i)
        if (dist <= locrad[i])
            sum += locweight[i] * or_taper_gc(dist / locrad[i]);
    return sum;
}

/* obs_findlocal (observations.c:1837-1927); domains are not modelled (every
 * type is visible from the single grid). */
int or_findlocal(const or_obsset* o, double lon, double lat, int* ids, double* lcoeffs, int cap)
{
    double q[3];
    or_kdres* res = NULL;
    size_t rescap = 0, stackcap = 0;
    size_t* stack = NULL;
    int t, n = 0, overflow = 0;

    if (isnan(lon + lat)) {
        /* obs_getglobal (observations.c:1773-1817): a point without
         * coordinates (grid type NONE) takes every observation with status
         * OK, type by type in id order, coefficient 1, no NLOBSMAX */
        for (t = 0; t < o->ntypes; ++t) {
            int i;

            for (i = 0; i < o->nobs_t[t]; ++i) {
                if (n < cap) {
                    ids[n] = o->obsids[t][i];
                    lcoeffs[n] = 1.0;
                } else
                    overflow = 1;
                n++;
            }
        }
        return overflow ? -n : n;
    }
    if (o->geographic) {
        double ll[2] = { lon, lat };

        or_ll2xyz(ll, q);
    } else {
        q[0] = lon;
        q[1] = lat;
        q[2] = NAN;
    }
    for (t = 0; t < o->ntypes; ++t) {
        size_t nloc, k;

        if (o->nobs_t[t] == 0)
            continue;
        nloc = kd_range(&o->trees[t], q, maxlocrad(o, t), &res, &rescap, &stack, &stackcap);
        if (o->nlobsmax[t] != INT_MAX) {
            sort_by_dist(res, nloc);
            if (nloc > (size_t) o->nlobsmax[t])
                nloc = o->nlobsmax[t];
        }
        for (k = 0; k < nloc; ++k) {
            int id = o->obsids[t][res[k].id];

            if (o->status[id] != 0)
                continue;
            if (n < cap) {
                ids[n] = id;
                lcoeffs[n] = or_calclcoeff(o->nlocrad[t], &o->locrad[t * OR_MAXLOCRAD], &o->locweight[t * OR_MAXLOCRAD], sqrt(res[k].distsq));
            } else
                overflow = 1;
            n++;
        }
    }
    free(res);
    free(stack);
    return overflow ? -n : n;
}

/* ---------------------------------------------------------------------------
 * per-point numerics (calc/calcs.c)
 * ------------------------------------------------------------------------- */

/* traceprod (calcs.c:41-97), compact-storage branch: A, B row-major blocks */
double or_traceprod(int transposeA, int transposeB, int m, int n, const double* A, const double* B)
{
    double trace = 0.0;
    int i, j;

    if (!transposeA && !transposeB) {
        for (i = 0; i < n; ++i)
            for (j = 0; j < m; ++j)
                trace += A[(size_t) j * n + i] * B[(size_t) i * m + j];
    } else if (transposeA && transposeB) {
        for (i = 0; i < n; ++i)
            for (j = 0; j < m; ++j)
                trace += B[(size_t) j * n + i] * A[(size_t) i * m + j];
    } else {
        for (i = 0; i < n * m; ++i)
            trace += A[i] * B[i];
    }
    return trace;
}

/* invm (calcs.c:103-132): Cholesky inverse, then mirror the upper triangle */
static int or_invm(int m, double* M)
{
    int info, i, j;

    if ((info = or_dpotrf('U', m, M, m)) != 0)
        return info;
    if ((info = or_dpotri('U', m, M, m)) != 0)
        return info;
    for (j = 1; j < m; ++j)
        for (i = 0; i < j; ++i)
            M[(size_t) i * m + j] = M[(size_t) j * m + i];
    return 0;
}

/* calc_G (calcs.c:189-221) with calc_Minv (141-178): G = inv(I + S'S) S' or
 * S' inv(I + SS'); M is workspace of n x n, n = min(m, p). */
static int or_calc_G(int m, int p, double* M, const double* S, double* G)
{
    int n = p < m ? p : m, i, info;

    if (p < m)
        or_dgemm('N', 'T', p, p, m, 1.0, S, p, S, p, 0.0, M, p);
    else
        or_dgemm('T', 'N', m, m, p, 1.0, S, p, S, p, 0.0, M, m);
    for (i = 0; i < n; ++i)
        M[(size_t) i * n + i] += 1.0;
    if ((info = or_invm(n, M)) != 0)
        return info;
    if (p < m)
        or_dgemm('T', 'N', m, p, p, 1.0, S, p, M, p, 0.0, G, m);
    else
        or_dgemm('N', 'T', m, p, m, 1.0, M, m, S, p, 0.0, G, m);
    return 0;
}

/* calc_wT_etkf (calcs.c:300-412): SVD of I + S'S (or I + SS'), T = I -
 * (M + M^1/2)^-1 S' S, G = M^-1 S', w = G s. */
static int or_calc_wT_etkf(int m, int mout, int p, const double* s, const double* S, double* w, double* T, double* G)
{
    int n = (p < m) ? p : m;
    double* M = malloc((size_t) (2 * n + 11) * n * sizeof(double));
    double* U = &M[(size_t) n * n];
    double* sig = &M[(size_t) 2 * n * n];
    double* work = &M[(size_t) (2 * n + 1) * n];
    int i, j, info;

    if (p < m)
        or_dgemm('N', 'T', p, p, m, 1.0, S, p, S, p, 0.0, M, p);
    else
        or_dgemm('T', 'N', m, m, p, 1.0, S, p, S, p, 0.0, M, m);
    for (i = 0; i < n; ++i)
        M[(size_t) i * n + i] += 1.0;
    info = or_dgesvd('A', 'N', n, n, M, n, sig, U, n, NULL, n, work, 10 * n);
    if (info != 0) {
        free(M);
        return info;
    }
    for (i = 0; i < n; ++i) {
        double sc = sqrt(sig[i] + sqrt(sig[i]));

        for (j = 0; j < n; ++j)
            U[(size_t) i * n + j] /= sc;
    }
    or_dgemm('N', 'T', n, n, n, 1.0, U, n, U, n, 0.0, M, n);
    if (p < m)
        or_dgemm('T', 'N', m, p, p, 1.0, S, p, M, p, 0.0, G, m);
    else
        or_dgemm('N', 'T', m, p, m, 1.0, M, m, S, p, 0.0, G, m);
    or_dgemm('N', 'N', m, mout, p, -1.0, G, m, S, p, 0.0, T, m);
    for (i = 0; i < mout; ++i)
        T[(size_t) i * m + i] += 1.0;
    for (i = 0; i < n; ++i) {
        double sc = sqrt(1.0 + 1.0 / sqrt(sig[i]));

        for (j = 0; j < n; ++j)
            U[(size_t) i * n + j] *= sc;
    }
    or_dgemm('N', 'T', n, n, n, 1.0, U, n, U, n, 0.0, M, n);
    if (p < m)
        or_dgemm('T', 'N', m, p, p, 1.0, S, p, M, p, 0.0, G, m);
    else
        or_dgemm('N', 'T', m, p, m, 1.0, M, m, S, p, 0.0, G, m);
    or_dgemv('N', m, p, 1.0, G, m, s, 0.0, w);
    free(M);
    return 0;
}

int or_calc_wT(int mode, int scheme, int m, int mout, int p, const double* s, double* S, double* w, double* T, double* G)
{
    int n = p < m ? p : m, info = 0, i;

    if (mode == OR_MODE_ENOI || scheme == OR_SCHEME_DENKF) {
        double* M = malloc((size_t) n * n * sizeof(double));

        /* calc_wT_denkf (calcs.c:279-284) / EnOI (transforms.c:1260-1262) */
        info = or_calc_G(m, p, M, S, G);
        free(M);
        if (info != 0)
            return info;
        if (mode != OR_MODE_ENOI) {
            /* calc_T_denkf (calcs.c:232-248) */
            or_dgemm('N', 'N', m, mout, p, -0.5, G, m, S, p, 0.0, T, m);
            for (i = 0; i < mout; ++i)
                T[(size_t) i * m + i] += 1.0;
        }
        /* calc_w (calcs.c:256-263) */
        or_dgemv('N', m, p, 1.0, G, m, s, 0.0, w);
        return 0;
    }
    return or_calc_wT_etkf(m, mout, p, s, S, w, T, G);
}

/* ---------------------------------------------------------------------------
 * das_calctransforms (calc/transforms.c:1150-1360)
 * ------------------------------------------------------------------------- */
int or_calctransforms(const or_obsset* obs, const or_calcparams* P, const float* S, const double* s, const short* type, int jj0, int jj1, float* T, float* w, double* T64, double* w64, int* nlobs, float* dfs, float* srf, int* pnlobs, float* pdfs, float* psrf)
{
    int m = P->nmem, md = P->nmem_dynamic, stride = P->stride;
    int nj = (P->mnj - 1) / stride + 1, ni = (P->mni - 1) / stride + 1;
    int nobs = obs->nobs, ntypes = obs->ntypes;
    int cap = nobs > 0 ? nobs : 1;
    int* lobs = malloc(cap * sizeof(int));
    double* lc = malloc(cap * sizeof(double));
    int* plobs = malloc(cap * sizeof(int));
    double* Tm = malloc((size_t) m * m * sizeof(double));
    double* wd = malloc(m * sizeof(double));
    int enkf = (P->mode == OR_MODE_ENKF || P->mode == OR_MODE_HYBRID);
    int jj, ii, e, o, ot, ret = 0;

    int iend = (P->ii1 > 0 && P->ii1 < ni) ? P->ii1 : ni;

    for (jj = jj0; jj < jj1 && jj < nj; ++jj) {
        int j = jj * stride;

        for (ii = P->ii0 > 0 ? P->ii0 : 0; ii < iend; ++ii) {
            int i = ii * stride;
            size_t cell = (size_t) jj * ni + ii;
            double lon, lat;
            int ploc;

            /* grid_ij2xy -> hgrid_ij2xy (hgrid.c:457-472) */
            if (P->x2d != NULL) {
                lon = P->x2d[(size_t) j * P->mni + i];
                lat = P->y2d[(size_t) j * P->mni + i];
            } else {
                lon = P->x[i];
                lat = P->y[j];
            }
            ploc = or_findlocal(obs, lon, lat, lobs, lc, cap);
            assert(ploc >= 0);

            if (ploc == 0) {
                /* transforms.c:1219-1236 */
                if (enkf && T != NULL) {
                    memset(&T[cell * md * m], 0, (size_t) md * m * sizeof(float));
                    for (e = 0; e < md; ++e)
                        T[cell * md * m + (size_t) e * m + e] = 1.0f;
                }
                if (enkf && T64 != NULL) {
                    memset(&T64[cell * md * m], 0, (size_t) md * m * sizeof(double));
                    for (e = 0; e < md; ++e)
                        T64[cell * md * m + (size_t) e * m + e] = 1.0;
                }
                memset(&w[cell * m], 0, m * sizeof(float));
                if (w64 != NULL)
                    memset(&w64[cell * m], 0, m * sizeof(double));
                if (nlobs != NULL) {
                    nlobs[cell] = 0;
                    dfs[cell] = 0.0f;
                    srf[cell] = 0.0f;
                }
                if (pnlobs != NULL)
                    for (ot = 0; ot < ntypes; ot++) {
                        pnlobs[(size_t) ot * nj * ni + cell] = 0;
                        pdfs[(size_t) ot * nj * ni + cell] = 0.0f;
                        psrf[(size_t) ot * nj * ni + cell] = 0.0f;
                    }
                continue;
            }
            {
                double* Sloc = malloc((size_t) m * ploc * sizeof(double));
                double* G = malloc((size_t) ploc * m * sizeof(double));
                double* sloc = malloc(ploc * sizeof(double));
                int info;

                /* transforms.c:1250-1258 */
                for (e = 0; e < m; ++e)
                    for (o = 0; o < ploc; ++o)
                        Sloc[(size_t) e * ploc + o] = (double) S[(size_t) e * nobs + lobs[o]] * lc[o];
                for (o = 0; o < ploc; ++o)
                    sloc[o] = s[lobs[o]] * lc[o];

                info = or_calc_wT(P->mode, P->scheme, m, md, ploc, sloc, Sloc, wd, Tm, G);
                if (info != 0 && ret == 0)
                    ret = info;

                if (enkf) {
                    int e1, e2;

                    /* relaxation to prior, transforms.c:1270-1286 */
                    for (e1 = 0; e1 < md; ++e1) {
                        double* Ti = &Tm[(size_t) e1 * m];

                        Ti[e1] -= 1.0;
                        for (e2 = 0; e2 < m; ++e2)
                            Ti[e2] *= P->alpha;
                        Ti[e1] += 1.0;
                    }
                    /* transforms.c:1288-1296 */
                    for (e1 = 0; e1 < md; ++e1)
                        for (e2 = 0; e2 < m; ++e2) {
                            if (T != NULL)
                                T[cell * md * m + (size_t) e1 * m + e2] = (float) Tm[(size_t) e1 * m + e2];
                            if (T64 != NULL)
                                T64[cell * md * m + (size_t) e1 * m + e2] = Tm[(size_t) e1 * m + e2];
                        }
                }
                for (e = 0; e < m; ++e) {
                    w[cell * m + e] = (float) wd[e];
                    if (w64 != NULL)
                        w64[cell * m + e] = wd[e];
                }

                /* diagnostics, transforms.c:1298-1345 */
                if (nlobs != NULL) {
                    nlobs[cell] = ploc;
                    dfs[cell] = (float) or_traceprod(0, 0, ploc, m, G, Sloc);
                    srf[cell] = (float) (sqrt(or_traceprod(0, 1, m, ploc, Sloc, Sloc) / dfs[cell]) - 1.0);
                }
                if (pnlobs != NULL) {
                    for (ot = 0; ot < ntypes; ++ot) {
                        size_t k = (size_t) ot * nj * ni + cell;
                        int pt = 0;

                        for (o = 0; o < ploc; ++o)
                            if (type[lobs[o]] == ot)
                                plobs[pt++] = o;
                        pnlobs[k] = pt;
                        if (pt == 0) {
                            pdfs[k] = 0.0f;
                            psrf[k] = 0.0f;
                        } else {
                            /* contiguous range starting at plobs[0], as the
                             * reference assumes (transforms.c:1313-1316) */
                            int o0 = plobs[0];
                            double tr = 0.0;

                            for (e = 0; e < m; ++e)
                                for (o = 0; o < pt; ++o)
                                    tr += G[(size_t) (o0 + o) * m + e] * Sloc[(size_t) e * ploc + o0 + o];
                            pdfs[k] = (float) tr;
                            if (pdfs[k] > OR_DFS_MIN) {
                                tr = 0.0;
                                for (e = 0; e < m; ++e)
                                    for (o = 0; o < pt; ++o)
                                        tr += Sloc[(size_t) e * ploc + o0 + o] * Sloc[(size_t) e * ploc + o0 + o];
                                psrf[k] = (float) (sqrt(tr / pdfs[k]) - 1.0);
                            } else
                                psrf[k] = 0.0f;
                        }
                    }
                }
                free(Sloc);
                free(G);
                free(sloc);
            }
        }
    }
    free(lobs);
    free(lc);
    free(plobs);
    free(Tm);
    free(wd);
    return ret;
}

/* ---------------------------------------------------------------------------
 * innovations and standardisation (calc/ensobs.c)
 * ------------------------------------------------------------------------- */

/* das_calcinnandspread (ensobs.c:541-690), S_MODE_HE_f branch */
void or_calcinnandspread(int nmem, int nobs, float* S, const float* value, const short* status, double* s_f, double* std_f)
{
    int e, o;

    memset(s_f, 0, nobs * sizeof(double));
    memset(std_f, 0, nobs * sizeof(double));
    for (e = 0; e < nmem; ++e)
        for (o = 0; o < nobs; ++o)
            s_f[o] += (double) S[(size_t) e * nobs + o];
    for (o = 0; o < nobs; ++o)
        s_f[o] /= (double) nmem;
    for (e = 0; e < nmem; ++e)
        for (o = 0; o < nobs; ++o)
            S[(size_t) e * nobs + o] -= (float) s_f[o];
    for (e = 0; e < nmem; ++e)
        for (o = 0; o < nobs; ++o) {
            float v = S[(size_t) e * nobs + o];

            std_f[o] += (double) (v * v);
        }
    for (o = 0; o < nobs; ++o) {
        if (status[o] != 0)
            continue;
        std_f[o] = sqrt(std_f[o] / (double) (nmem - 1));
        s_f[o] = value[o] - s_f[o];
    }
}

/* das_standardise (ensobs.c:849-898) */
void or_standardise(int nmem, int nobs, float* S, double* s_f, const float* estd, const short* type, const double* rfactor)
{
    double mult = sqrt((double) nmem - 1);
    int e, i;

    for (e = 0; e < nmem; ++e)
        for (i = 0; i < nobs; ++i)
            S[(size_t) e * nobs + i] /= estd[i] * sqrt(rfactor[type[i]]) * mult;
    if (s_f != NULL)
        for (i = 0; i < nobs; ++i)
            s_f[i] /= estd[i] * sqrt(rfactor[type[i]]) * mult;
}

/* ---------------------------------------------------------------------------
 * forward operator (calc/model2obs.c, common/utils.c) and the end of das_getHE
 * (calc/ensobs.c)
 * ------------------------------------------------------------------------- */

#define OR_EPS_EDGE 1.0e-7                   /* common/utils.c:51 (EPS_FLOAT) */
#define OR_STATUS_BADFC 10                   /* common/global.h:62 */

/* Horizontal corner indices and weights of a fractional position: lower and
 * upper index with weights (ceil - f) and (f - floor); a position on an integer
 * takes its one index with weight 1; the edge rules wrap (periodic in i) or
 * repeat the inner index (utils.c:1158-1184, 1270-1311).  Returns 0 where the
 * reference's index assert would fail. */
static int or_corners(double fi, double fj, int ni, int nj, int periodic_i, int i[2], int j[2], double wi[2], double wj[2])
{
    i[0] = (int) floor(fi);
    wi[0] = ceil(fi) - fi;
    i[1] = (int) ceil(fi);
    wi[1] = fi - floor(fi);
    j[0] = (int) floor(fj);
    wj[0] = ceil(fj) - fj;
    j[1] = (int) ceil(fj);
    wj[1] = fj - floor(fj);
    if (i[0] == i[1])
        wi[0] = 1.0;
    if (j[0] == j[1])
        wj[0] = 1.0;
    if (i[0] == -1)
        i[0] = periodic_i ? ni - 1 : i[1];
    if (i[1] == ni)
        i[1] = periodic_i ? 0 : i[0];
    if (j[0] == -1)
        j[0] = j[1];
    if (j[1] == nj)
        j[1] = j[0];
    return i[0] >= 0 && i[0] < ni && i[1] >= 0 && i[1] < ni && j[0] >= 0 && j[0] < nj && j[1] >= 0 && j[1] < nj;
}

/* interpolate2d_structured (common/utils.c:1140-1210): the four corners in
 * the order (j1,i1) (j1,i2) (j2,i1) (j2,i2), each kept where mask != 0, the
 * double sum renormalised by the kept weights and cast to float. */
float or_interp2d(double fi, double fj, int ni, int nj, const float* v, const int* mask, int periodic_i, int* badpos)
{
    int i[2], j[2], a, b;
    double wi[2], wj[2], sum = 0.0, w = 0.0;

    /* positions at or below -1 fail the reference's assert (or read outside
     * the row with weight 0); NaN fails here too */
    if (!(fi > -1.0 && fj > -1.0)) {
        *badpos = 1;
        return NAN;
    }
    if (fi >= (double) ni)
        fi = (double) ni - OR_EPS_EDGE;
    if (fj >= (double) nj)
        fj = (double) nj - OR_EPS_EDGE;
    if (!or_corners(fi, fj, ni, nj, periodic_i, i, j, wi, wj)) {
        *badpos = 1;
        return NAN;
    }
    for (b = 0; b < 2; ++b)
        for (a = 0; a < 2; ++a) {
            size_t c = (size_t) j[b] * ni + i[a];

            if (mask[c]) {
                double ww = wj[b] * wi[a];

                sum += v[c] * ww;
                w += ww;
            }
        }
    sum /= w;
    return (float) sum;
}

/* interpolate3d_structured (common/utils.c:1252-1366): fk clamped to
 * [0, nk-1]; layer k is wet at (j,i) when nlevels[j][i] > |ktop - k|; the
 * eight corners in the order k1 then k2, each (j1,i1) (j1,i2) (j2,i1) (j2,i2),
 * weight (wj wi) wk. */
float or_interp3d(double fi, double fj, double fk, int ni, int nj, int nk, int ktop, const float* v, const int* nlevels, int periodic_i, int* badpos)
{
    int i[2], j[2], k[2], ktp[2], a, b, c;
    double wi[2], wj[2], wk[2], sum = 0.0, w = 0.0;
    size_t nij = (size_t) ni * nj;

    if (!(fi > -1.0 && fj > -1.0) || isnan(fk)) {
        *badpos = 1;
        return NAN;
    }
    /* note the strict test on i (utils.c:1265) */
    if (fi > (double) ni)
        fi = (double) ni - OR_EPS_EDGE;
    if (fj >= (double) nj)
        fj = (double) nj - OR_EPS_EDGE;
    if (fk < 0.0)
        fk = 0.0;
    if (fk > (double) (nk - 1))
        fk = (double) (nk - 1);
    k[0] = (int) floor(fk);
    wk[0] = ceil(fk) - fk;
    k[1] = (int) ceil(fk);
    wk[1] = fk - floor(fk);
    if (wk[0] == 0.0 && wk[1] == 0.0)
        wk[0] = 1.0;
    if (k[0] == k[1])
        wk[0] = 1.0;
    ktp[0] = abs(ktop - k[0]);
    ktp[1] = abs(ktop - k[1]);
    if (!or_corners(fi, fj, ni, nj, periodic_i, i, j, wi, wj)) {
        *badpos = 1;
        return NAN;
    }
    for (c = 0; c < 2; ++c)
        for (b = 0; b < 2; ++b)
            for (a = 0; a < 2; ++a) {
                size_t q = (size_t) j[b] * ni + i[a];

                if (nlevels[q] > ktp[c]) {
                    double ww = wj[b] * wi[a] * wk[c];

                    sum += v[(size_t) k[c] * nij + q] * ww;
                    w += ww;
                }
            }
    sum = sum / w;
    return (float) sum;
}

/* H_surf_standard / H_subsurf_standard (calc/model2obs.c:127-181, 256-348):
 * the field minus its OFFSET data, then evaluate_2d_obs / interpolate_3d_obs
 * (calc/model2obs.c:37-124) with footprint 0, including the bad-forecast rule
 * (!finite or |v| > MAXOBSVAL: NaN with --skip-bad-forecast-obs, else quit). */
int or_map_obs(int three_d, int ni, int nj, int nk, int ktop, int periodic_i, const int* numlevels, const float* offset, int offset_kind, const float* field, int nids, const int* ids, const double* fi, const double* fj, const float* fk, int skip_bad, float* dst)
{
    size_t nij = (size_t) ni * nj, nv = three_d ? nij * (size_t) nk : nij, q;
    const float* src = field;
    float* tmp = NULL;
    int n, rc = 0;

    if (offset != NULL && offset_kind > 0) {
        tmp = malloc(nv * sizeof(float));
        for (q = 0; q < nv; ++q) {
            float off = offset_kind == 1 ? offset[q / nij] : offset_kind == 2 ? offset[q % nij] : offset[q];

            tmp[q] = field[q] - off;
        }
        src = tmp;
    }
    for (n = 0; n < nids; ++n) {
        int id = ids[n], bad = 0;
        float v = three_d ? or_interp3d(fi[id], fj[id], (double) fk[id], ni, nj, nk, ktop, src, numlevels, periodic_i, &bad)
            : or_interp2d(fi[id], fj[id], ni, nj, src, numlevels, periodic_i, &bad);

        if (bad) {
            rc = -(1 + id);
            break;
        }
        if (!isfinite(v) || fabs(v) > OR_MAXOBSVAL) {
            if (!skip_bad) {
                rc = 1 + id;
                break;
            }
            v = NAN;
        }
        dst[id] = v;
    }
    free(tmp);
    return rc;
}

/* das_getHE after the forward operators (calc/ensobs.c:372-490): the
 * bad-forecast status, then the EnOI recentring on the background (float
 * mean) or the hybrid rescaling (double means, k_d and k_s). */
int or_finish_HE(int mode, int nmem, int nmem_d, double gamma, int nobs, float* S, const float* Hx, int skip_bad, short* status)
{
    int e, i, nbad = 0;

    if (skip_bad) {
        for (e = 0; e < nmem; ++e)
            for (i = 0; i < nobs; ++i)
                if (isnan(S[(size_t) e * nobs + i]))
                    status[i] = OR_STATUS_BADFC;
        if (mode == OR_MODE_ENOI)
            for (i = 0; i < nobs; ++i)
                if (isnan(Hx[i]))
                    status[i] = OR_STATUS_BADFC;
    }
    for (i = 0; i < nobs; ++i)
        nbad += status[i] == OR_STATUS_BADFC;

    if (mode == OR_MODE_ENOI) {
        float* mean = calloc(nobs > 0 ? nobs : 1, sizeof(float));

        for (e = 0; e < nmem; ++e)
            for (i = 0; i < nobs; ++i)
                mean[i] += S[(size_t) e * nobs + i];
        for (i = 0; i < nobs; ++i)
            mean[i] /= (float) nmem;
        for (e = 0; e < nmem; ++e)
            for (i = 0; i < nobs; ++i)
                S[(size_t) e * nobs + i] += Hx[i] - mean[i];
        free(mean);
    } else if (mode == OR_MODE_HYBRID) {
        int nmem_s = nmem - nmem_d;
        double k_d = (nmem_d > 1) ? sqrt((double) (nmem - 1) / (double) (nmem_d - 1)) : 0.0;
        double k_s = sqrt(gamma * (double) (nmem - 1) / (double) (nmem_s - 1));
        double* md = calloc(nobs > 0 ? nobs : 1, sizeof(double));
        double* ms = calloc(nobs > 0 ? nobs : 1, sizeof(double));

        for (e = 0; e < nmem_d; ++e)
            for (i = 0; i < nobs; ++i)
                md[i] += S[(size_t) e * nobs + i];
        for (i = 0; i < nobs; ++i)
            md[i] /= (double) nmem_d;
        for (e = 0; e < nmem_d; ++e)
            for (i = 0; i < nobs; ++i) {
                float* p = &S[(size_t) e * nobs + i];

                *p = (*p - md[i]) * k_d + md[i];
            }
        for (e = nmem_d; e < nmem; ++e)
            for (i = 0; i < nobs; ++i)
                ms[i] += S[(size_t) e * nobs + i];
        for (i = 0; i < nobs; ++i)
            ms[i] /= (double) nmem_s;
        for (e = nmem_d; e < nmem; ++e)
            for (i = 0; i < nobs; ++i) {
                float* p = &S[(size_t) e * nobs + i];

                *p = (*p - ms[i]) * k_s + md[i];
            }
        free(md);
        free(ms);
    }
    return nbad;
}

/* ---------------------------------------------------------------------------
 * update (update/update.c, common/dasystem.c)
 * ------------------------------------------------------------------------- */

/* Stride interpolation of T and w for model row j (update.c:195-272).  The
 * state (Tjj, Tjj1, Tjj2, ...) is kept exactly as the reference keeps it. */
typedef struct {
    int nt;                     /* floats per T cell (0 for w only) */
    int m;
    int ni, nj, mni, stride, periodic_i;
    const float* T;
    const float* w;
    float *Tjj, *Tjj1, *Tjj2, *wjj, *wjj1, *wjj2;
    float *Tj, *wj;
} interp_state;

static void interp_init(interp_state* st, int nt, int m, const or_updateparams* P, const float* T, const float* w)
{
    memset(st, 0, sizeof(*st));
    st->nt = nt;
    st->m = m;
    st->ni = P->ni;
    st->nj = P->nj;
    st->mni = P->mni;
    st->stride = P->stride;
    st->periodic_i = P->periodic_i;
    st->T = T;
    st->w = w;
    st->Tj = malloc(((size_t) P->mni * nt + 1) * sizeof(float));
    st->wj = malloc((size_t) P->mni * m * sizeof(float));
    if (P->stride > 1) {
        size_t rowT = (size_t) P->ni * nt, roww = (size_t) P->ni * m;

        st->Tjj = malloc((rowT + 1) * sizeof(float));
        st->Tjj1 = malloc((rowT + 1) * sizeof(float));
        st->Tjj2 = malloc((rowT + 1) * sizeof(float));
        st->wjj = malloc(roww * sizeof(float));
        st->wjj1 = malloc(roww * sizeof(float));
        st->wjj2 = malloc(roww * sizeof(float));
        if (nt > 0)
            memcpy(st->Tjj2, &T[(size_t) (P->j1 / P->stride) * rowT], rowT * sizeof(float));
        memcpy(st->wjj2, &w[(size_t) (P->j1 / P->stride) * roww], roww * sizeof(float));
    }
}

static void interp_free(interp_state* st)
{
    free(st->Tj);
    free(st->wj);
    free(st->Tjj);
    free(st->Tjj1);
    free(st->Tjj2);
    free(st->wjj);
    free(st->wjj1);
    free(st->wjj2);
}

static void interp_row(interp_state* st, int jj, int stepj)
{
    int nt = st->nt, m = st->m, ni = st->ni, stride = st->stride, mni = st->mni;
    size_t rowT = (size_t) ni * nt, roww = (size_t) ni * m;
    int ii, i, stepi, e;

    if (stride == 1) {
        if (nt > 0)
            memcpy(st->Tj, &st->T[(size_t) jj * rowT], rowT * sizeof(float));
        memcpy(st->wj, &st->w[(size_t) jj * roww], roww * sizeof(float));
        return;
    }
    if (stepj == 0) {
        if (nt > 0) {
            memcpy(st->Tjj1, st->Tjj2, rowT * sizeof(float));
            memcpy(st->Tjj, st->Tjj2, rowT * sizeof(float));
        }
        memcpy(st->wjj, st->wjj2, roww * sizeof(float));
        memcpy(st->wjj1, st->wjj2, roww * sizeof(float));
        if (jj < st->nj - 1) {
            int jn = (jj + 1) % st->nj;

            if (nt > 0)
                memcpy(st->Tjj2, &st->T[(size_t) jn * rowT], rowT * sizeof(float));
            memcpy(st->wjj2, &st->w[(size_t) jn * roww], roww * sizeof(float));
        }
    } else {
        float weight2 = (float) stepj / (float) stride;
        float weight1 = 1.0f - weight2;

        for (e = 0; e < (int) rowT; ++e)
            st->Tjj[e] = st->Tjj1[e] * weight1 + st->Tjj2[e] * weight2;
        for (e = 0; e < (int) roww; ++e)
            st->wjj[e] = st->wjj1[e] * weight1 + st->wjj2[e] * weight2;
    }
    for (ii = 0, i = 0; ii < ni; ++ii) {
        for (stepi = 0; stepi < stride && i < mni; ++stepi, ++i) {
            if (stepi == 0) {
                if (nt > 0)
                    memcpy(&st->Tj[(size_t) i * nt], &st->Tjj[(size_t) ii * nt], nt * sizeof(float));
                memcpy(&st->wj[(size_t) i * m], &st->wjj[(size_t) ii * m], m * sizeof(float));
            } else {
                float weight2 = (float) stepi / (float) stride;
                float weight1 = 1.0f - weight2;
                int ii2 = (ii < ni - 1) ? ii + 1 : (st->periodic_i ? (ii + 1) % ni : ii);

                for (e = 0; e < nt; ++e)
                    st->Tj[(size_t) i * nt + e] = st->Tjj[(size_t) ii * nt + e] * weight1 + st->Tjj[(size_t) ii2 * nt + e] * weight2;
                for (e = 0; e < m; ++e)
                    st->wj[(size_t) i * m + e] = st->wjj[(size_t) ii * m + e] * weight1 + st->wjj[(size_t) ii2 * m + e] * weight2;
            }
        }
    }
}

/* das_updatefields (update.c:92-564), structured grid, one field */
int or_updatefields(const or_updateparams* P, const float* T, const float* w, const int* numlevels, float* v, float* infl)
{
    int m = P->nmem, md = P->nmem_dynamic, mni = P->mni, stride = P->stride;
    int jsize = P->j2 - P->j1 + 1;
    size_t plane = (size_t) jsize * mni;
    float* v_f = malloc(m * sizeof(float));
    float* v_a = malloc((md > 0 ? md : 1) * sizeof(float));
    interp_state st;
    int jj, j, stepj, i, e;

    interp_init(&st, md * m, m, P, T, w);
    for (jj = P->j1 / stride, j = 0; jj <= P->j2 / stride && jj < P->nj; ++jj) {
        for (stepj = 0; stepj < stride && j <= P->j2 - P->j1; ++stepj, ++j) {
            interp_row(&st, jj, stepj);
            for (i = 0; i < mni; ++i) {
                float inflation = P->inflation0;
                double v1_f, v1_a;
                size_t c = (size_t) j * mni + i;
                int nl = numlevels[(size_t) (P->j1 + j) * mni + i];
                const float* Tji = &st.Tj[(size_t) i * md * m];
                const float* wji = &st.wj[(size_t) i * m];

                /* the reference clears the row's inflation buffer first */
                if (infl != NULL)
                    infl[c] = 0.0f;
                if (P->surfk == 0) {
                    if (nl <= P->level) {
                        for (e = 0; e < m; ++e)
                            v[e * plane + c] = 0.0f;
                        continue;
                    }
                } else if (nl <= (P->issurfacevar ? 0 : P->surfk - P->level)) {
                    for (e = 0; e < m; ++e)
                        v[e * plane + c] = 0.0f;
                    continue;
                }
                for (e = 0; e < m; ++e)
                    if (!isfinite(v[e * plane + c]) || fabsf(v[e * plane + c]) > (float) OR_MAXOBSVAL)
                        break;
                if (e < md) {
                    for (e = 0; e < m; ++e)
                        v[e * plane + c] = 0.0f;
                    continue;
                } else if (e < m) {
                    for (e = md; e < m; ++e)
                        v[e * plane + c] = 0.0f;
                    if (md == 0)
                        continue;
                }
                for (e = 0; e < m; ++e)
                    v_f[e] = v[e * plane + c];

                for (e = 0, v1_f = 0.0; e < md; ++e)
                    v1_f += v_f[e];
                v1_f /= (double) md;
                for (e = 0; e < m; ++e)
                    v_f[e] -= v1_f;
                or_sgemv('T', m, md, 1.0f, Tji, m, v_f, 0.0f, v_a);
                for (e = 0, v1_a = 0.0; e < m; ++e)
                    v1_a += v_f[e] * wji[e];
                v1_a += v1_f;
                if (P->mode == OR_MODE_HYBRID) {
                    double k_d = (md > 1) ? sqrt((double) (m - 1) / (double) (md - 1)) : 1.0;

                    for (e = 0; e < md; ++e)
                        v_a[e] /= k_d;
                    for (e = 0; e < md; ++e)
                        v_f[e] /= k_d;
                }
                if (!isnan(P->inf_ratio)) {
                    double v2_f = 0.0, v2_a = 0.0;

                    for (e = 0; e < md; ++e) {
                        v2_f += v_f[e] * v_f[e];
                        v2_a += v_a[e] * v_a[e];
                    }
                    if (v2_a > 0.0) {
                        inflation = (float) (sqrt(v2_f / v2_a) * P->inf_ratio + 1.0 - P->inf_ratio);
                        if (inflation >= P->inflation0)
                            inflation = P->inflation0;
                    }
                }
                if (inflation - 1.0f > OR_EPSF)
                    for (e = 0; e < md; ++e)
                        v_a[e] = v_a[e] * inflation;
                else
                    inflation = 1.0f;
                for (e = 0; e < md; ++e)
                    v_a[e] += v1_a;
                for (e = 0; e < md; ++e)
                    v_f[e] += v1_f;
                if (!P->output_increment)
                    for (e = 0; e < md; ++e)
                        v[e * plane + c] = v_a[e];
                else if (!P->applylog)
                    for (e = 0; e < md; ++e)
                        v[e * plane + c] = v_a[e] - v_f[e];
                else
                    for (e = 0; e < md; ++e)
                        v[e * plane + c] = !isnormal(v_f[e]) ? 0.0f : (float) (exp10(v_a[e]) - exp10(v_f[e]));
                if (infl != NULL)
                    infl[c] = inflation;
            }
        }
    }
    interp_free(&st);
    free(v_f);
    free(v_a);
    return 0;
}

/* das_updatebg (update.c:568-814), structured grid, one field */
int or_updatebg(const or_updateparams* P, const float* w, const int* numlevels, float* v)
{
    int m = P->nmem, mni = P->mni, stride = P->stride;
    int jsize = P->j2 - P->j1 + 1;
    size_t plane = (size_t) jsize * mni;
    interp_state st;
    int jj, j, stepj, i, e;

    interp_init(&st, 0, m, P, NULL, w);
    for (jj = P->j1 / stride, j = 0; jj <= P->j2 / stride && jj < P->nj; ++jj) {
        for (stepj = 0; stepj < stride && j <= P->j2 - P->j1; ++stepj, ++j) {
            interp_row(&st, jj, stepj);
            for (i = 0; i < mni; ++i) {
                size_t c = (size_t) j * mni + i;
                int nl = numlevels[(size_t) (P->j1 + j) * mni + i];
                float* bg = &v[(size_t) m * plane + c];
                const float* wji = &st.wj[(size_t) i * m];
                float xmean = 0.0f;

                if (P->surfk == 0) {
                    if (nl <= P->level) {
                        *bg = 0.0f;
                        continue;
                    }
                } else if (nl <= (P->issurfacevar ? 1 : P->surfk - P->level)) {
                    *bg = 0.0f;
                    continue;
                }
                if (fabsf(*bg) > (float) OR_MAXOBSVAL) {
                    *bg = 0.0f;
                    continue;
                }
                for (e = 0; e < m; ++e)
                    if (fabsf(v[e * plane + c]) > (float) OR_MAXOBSVAL)
                        break;
                if (e < m) {
                    *bg = 0.0f;
                    continue;
                }
                for (e = 0; e < m; ++e)
                    xmean += v[e * plane + c];
                xmean /= (float) m;
                for (e = 0; e < m; ++e)
                    *bg += (v[e * plane + c] - xmean) * wji[e];
            }
        }
    }
    interp_free(&st);
    return 0;
}

/* addnoise (update.c:46-87): the member normals less their mean, then
 * v * (float) deflation + mult * r_e with mult a float; the float product
 * is widened to double for the sum, which is rounded back to float. */
void or_addnoise(int nmem, long ncell, double deflation, double sigma, const double* random, float* v)
{
    double* r = malloc(nmem * sizeof(double));
    double sum = 0.0;
    float mult;
    int e;
    long i;

    for (e = 0; e < nmem; ++e)
        sum += random[e];
    sum /= (double) nmem;
    for (e = 0; e < nmem; ++e)
        r[e] = random[e] - sum;
    mult = (float) (sqrt(1.0 - deflation * deflation) * sigma);
    for (e = 0; e < nmem; ++e) {
        float* vv = v + (size_t) e * ncell;

        for (i = 0; i < ncell; ++i)
            vv[i] = vv[i] * (float) deflation + mult * r[e];
    }
    free(r);
}

/* das_sethybridensemble (dasystem.c:775-819) */
void or_sethybridensemble(int nmem, int nmem_d, int nmem_s, double gamma, int nij, float* v, double* vmean)
{
    double k_d = (nmem_d > 1) ? sqrt((double) (nmem - 1) / (double) (nmem_d - 1)) : 0.0;
    double k_s = sqrt(gamma * (double) (nmem - 1) / (double) (nmem_s - 1));
    int i, e;

    memset(vmean, 0, nij * sizeof(double));
    for (e = 0; e < nmem_d; ++e)
        for (i = 0; i < nij; ++i)
            vmean[i] += (double) v[(size_t) e * nij + i];
    for (i = 0; i < nij; ++i)
        vmean[i] /= (double) nmem_d;
    for (e = 0; e < nmem_d; ++e)
        for (i = 0; i < nij; ++i) {
            float* ve = &v[(size_t) e * nij + i];

            *ve = (*ve - vmean[i]) * k_d + vmean[i];
        }
    for (e = nmem_d; e < nmem; ++e)
        for (i = 0; i < nij; ++i) {
            float* ve = &v[(size_t) e * nij + i];

            *ve = *ve * k_s + vmean[i];
        }
}
