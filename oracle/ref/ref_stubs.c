/*
 * ref_stubs.c -- glue for building the reference's calc/calcs.c and
 * common/kdtree.c (unmodified) into oracle/_ref/libenkf_ref.so.
 * TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement against the
 * reference's own numerics and kd-tree in the container that holds the
 * reference sources.
 *
 * Provides the few utilities those two files link against (enkf_quit,
 * alloc2d, cast2d, seed_rand48: reference common/utils.c) written here from
 * their documented behaviour, and flat entry points convenient for ctypes
 * (the LAPACK wrappers named by shim.h are in ref_blas.c).
 */
#define _GNU_SOURCE
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include "../or_blas.h"

long int seed_rand48 = 0;

void enkf_quit(char* format, ...)
{
    va_list args;

    va_start(args, format);
    vfprintf(stderr, format, args);
    va_end(args);
    fprintf(stderr, "\n");
    abort();
}

/* a contiguous nj x ni block behind an array of row pointers */
void* alloc2d(size_t nj, size_t ni, size_t unitsize)
{
    size_t i;
    char* p;
    void** pp = malloc(nj * sizeof(void*) + nj * ni * unitsize);

    p = (char*) &pp[nj];
    for (i = 0; i < nj; ++i)
        pp[i] = p + i * ni * unitsize;
    return pp;
}

void* cast2d(void* p, size_t nj, size_t ni, size_t unitsize)
{
    size_t i;
    void** pp = malloc(nj * sizeof(void*));

    for (i = 0; i < nj; ++i)
        pp[i] = (char*) p + i * ni * unitsize;
    return pp;
}


/* --- the reference API (calc/calcs.h, common/kdtree.h) ------------------- */
void calc_G(int m, int p, double** Min, double** S, double** G);
void calc_w(int m, int p, double** G, double* s, double* w);
void calc_wT_denkf(int m, int mout, int p, double* s, double** S, double** Sa, double** M, double** G, double* w, double** T);
void calc_wT_etkf(int m, int mout, int p, double* s, double** S, double** Sa, double** M, double** G, double* w, double** T);

typedef struct kdtree kdtree;
typedef struct {
    size_t id;
    double distsq;
} kdresult;
kdtree* kd_create(char* name, size_t ndim);
void kd_destroy(kdtree* tree);
void kd_insertnode(kdtree* tree, const double* coords, size_t data);
void kd_setstorage(kdtree* tree, size_t n, void* storage, int ismaster);
void kd_findnodeswithinrange(kdtree* tree, const double* coords, double range, int ordered, size_t* n, kdresult** results);
size_t kd_getnodedata(const kdtree* tree, size_t id);

/* Flat wrapper over calc_wT_etkf / calc_wT_denkf / calc_G + calc_w, the way
 * das_calctransforms calls them (transforms.c:1260-1268). S is [m][p]. */
int ref_calc_wT(int mode, int scheme, int m, int mout, int p, double* s, double* S, double* w, double* T, double* G)
{
    double** Sr = cast2d(S, m, p, sizeof(double));
    double** Gr = cast2d(G, p, m, sizeof(double));
    double** Tr = cast2d(T, m, m, sizeof(double));

    if (mode == 1) {
        calc_G(m, p, NULL, Sr, Gr);
        calc_w(m, p, Gr, s, w);
    } else if (scheme == 0)
        calc_wT_denkf(m, mout, p, s, Sr, Sr, NULL, Gr, w, Tr);
    else
        calc_wT_etkf(m, mout, p, s, Sr, Sr, NULL, Gr, w, Tr);
    free(Sr);
    free(Gr);
    free(Tr);
    return 0;
}

/* One kd-tree of n nodes (ndim 2 or 3) built the way obs_createkdtrees does
 * (observations.c:1660-1718 without SHMEM): kd_setstorage(NULL), then one
 * kd_insertnode per obs with data = insertion index. */
void* ref_kd_build(int ndim, int n, const double* coords)
{
    kdtree* t = kd_create("ref", ndim);
    int i;

    if (n > 0)
        kd_setstorage(t, n, NULL, -1);
    for (i = 0; i < n; ++i)
        kd_insertnode(t, &coords[(size_t) i * ndim], i);
    return t;
}

void ref_kd_free(void* t)
{
    kd_destroy((kdtree*) t);
}

/* kd_findnodeswithinrange; writes node data (insertion index) and distsq in
 * the tree's result order.  Returns the count, or -count if cap is short. */
int ref_kd_range(void* t, const double* q, double range, int ordered, int* data, double* distsq, int cap)
{
    size_t n, i;
    kdresult* res;

    kd_findnodeswithinrange((kdtree*) t, q, range, ordered, &n, &res);
    if ((int) n > cap)
        return -(int) n;
    for (i = 0; i < n; ++i) {
        data[i] = (int) kd_getnodedata((kdtree*) t, res[i].id);
        distsq[i] = res[i].distsq;
    }
    return (int) n;
}
