/*
 * or_blas.c -- run-time binding of BLAS/LAPACK for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY (see or_blas.h).
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
#include "or_blas.h"

typedef int32_t i32;
typedef int64_t i64;

/* LP64 prototypes */
typedef void (*dgemm32_t)(const char*, const char*, const i32*, const i32*, const i32*, const double*, const double*, const i32*, const double*, const i32*, const double*, double*, const i32*);
typedef void (*dgemv32_t)(const char*, const i32*, const i32*, const double*, const double*, const i32*, const double*, const i32*, const double*, double*, const i32*);
typedef void (*sgemv32_t)(const char*, const i32*, const i32*, const float*, const float*, const i32*, const float*, const i32*, const float*, float*, const i32*);
typedef void (*dpotrf32_t)(const char*, const i32*, double*, const i32*, i32*);
typedef void (*dgesvd32_t)(const char*, const char*, const i32*, const i32*, double*, const i32*, double*, double*, const i32*, double*, const i32*, double*, const i32*, i32*);
/* ILP64 prototypes */
typedef void (*dgemm64_t)(const char*, const char*, const i64*, const i64*, const i64*, const double*, const double*, const i64*, const double*, const i64*, const double*, double*, const i64*);
typedef void (*dgemv64_t)(const char*, const i64*, const i64*, const double*, const double*, const i64*, const double*, const i64*, const double*, double*, const i64*);
typedef void (*sgemv64_t)(const char*, const i64*, const i64*, const float*, const float*, const i64*, const float*, const i64*, const float*, float*, const i64*);
typedef void (*dpotrf64_t)(const char*, const i64*, double*, const i64*, i64*);
typedef void (*dgesvd64_t)(const char*, const char*, const i64*, const i64*, double*, const i64*, double*, double*, const i64*, double*, const i64*, double*, const i64*, i64*);

static int g_ilp64 = -1;        /* -1: not loaded */
static void* g_fn[6];           /* dgemm dgemv sgemv dpotrf dpotri dgesvd */

static void* find(void* h, const char* base, int ilp64)
{
    char name[128];
    void* f;

    if (!ilp64) {
        snprintf(name, sizeof(name), "scipy_%s_", base);
        if ((f = dlsym(h, name)) != NULL)
            return f;
        snprintf(name, sizeof(name), "%s_", base);
        return dlsym(h, name);
    }
    snprintf(name, sizeof(name), "scipy_%s_64_", base);
    if ((f = dlsym(h, name)) != NULL)
        return f;
    snprintf(name, sizeof(name), "%s_64_", base);
    return dlsym(h, name);
}

int or_blas_load(const char* path)
{
    static const char* names[6] = { "dgemm", "dgemv", "sgemv", "dpotrf", "dpotri", "dgesvd" };
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    int ilp64, i;

    if (h == NULL)
        return -100;
    for (ilp64 = 0; ilp64 < 2; ++ilp64) {
        for (i = 0; i < 6; ++i)
            if ((g_fn[i] = find(h, names[i], ilp64)) == NULL)
                break;
        if (i == 6)
            break;
    }
    if (ilp64 == 2)
        return -(i + 1);
    g_ilp64 = ilp64;
    {
        /* one BLAS thread per caller: the oracle parallelises over rows */
        typedef void (*setn_t)(int);
        const char* tn[4] = { "scipy_openblas_set_num_threads", "openblas_set_num_threads", "scipy_openblas_set_num_threads64_", "openblas_set_num_threads64_" };
        for (i = 0; i < 4; ++i) {
            setn_t f = (setn_t) dlsym(h, tn[i]);
            if (f != NULL) {
                f(1);
                break;
            }
        }
    }
    return 0;
}

int or_blas_loaded(void)
{
    return g_ilp64 >= 0;
}

void or_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc)
{
    if (!g_ilp64) {
        i32 M = m, N = n, K = k, la = lda, lb = ldb, lc = ldc;
        ((dgemm32_t) g_fn[0]) (&ta, &tb, &M, &N, &K, &alpha, A, &la, B, &lb, &beta, C, &lc);
    } else {
        i64 M = m, N = n, K = k, la = lda, lb = ldb, lc = ldc;
        ((dgemm64_t) g_fn[0]) (&ta, &tb, &M, &N, &K, &alpha, A, &la, B, &lb, &beta, C, &lc);
    }
}

void or_dgemv(char t, int m, int n, double alpha, const double* A, int lda, const double* x, double beta, double* y)
{
    if (!g_ilp64) {
        i32 M = m, N = n, la = lda, one = 1;
        ((dgemv32_t) g_fn[1]) (&t, &M, &N, &alpha, A, &la, x, &one, &beta, y, &one);
    } else {
        i64 M = m, N = n, la = lda, one = 1;
        ((dgemv64_t) g_fn[1]) (&t, &M, &N, &alpha, A, &la, x, &one, &beta, y, &one);
    }
}

void or_sgemv(char t, int m, int n, float alpha, const float* A, int lda, const float* x, float beta, float* y)
{
    if (!g_ilp64) {
        i32 M = m, N = n, la = lda, one = 1;
        ((sgemv32_t) g_fn[2]) (&t, &M, &N, &alpha, A, &la, x, &one, &beta, y, &one);
    } else {
        i64 M = m, N = n, la = lda, one = 1;
        ((sgemv64_t) g_fn[2]) (&t, &M, &N, &alpha, A, &la, x, &one, &beta, y, &one);
    }
}

static int potrx(int which, char uplo, int n, double* A, int lda)
{
    if (!g_ilp64) {
        i32 N = n, la = lda, info = 0;
        ((dpotrf32_t) g_fn[which]) (&uplo, &N, A, &la, &info);
        return (int) info;
    } else {
        i64 N = n, la = lda, info = 0;
        ((dpotrf64_t) g_fn[which]) (&uplo, &N, A, &la, &info);
        return (int) info;
    }
}

int or_dpotrf(char uplo, int n, double* A, int lda)
{
    return potrx(3, uplo, n, A, lda);
}

int or_dpotri(char uplo, int n, double* A, int lda)
{
    return potrx(4, uplo, n, A, lda);
}

int or_dgesvd(char jobu, char jobvt, int m, int n, double* A, int lda, double* S, double* U, int ldu, double* VT, int ldvt, double* work, int lwork)
{
    if (!g_ilp64) {
        i32 M = m, N = n, la = lda, lu = ldu, lv = ldvt, lw = lwork, info = 0;
        ((dgesvd32_t) g_fn[5]) (&jobu, &jobvt, &M, &N, A, &la, S, U, &lu, VT, &lv, work, &lw, &info);
        return (int) info;
    } else {
        i64 M = m, N = n, la = lda, lu = ldu, lv = ldvt, lw = lwork, info = 0;
        ((dgesvd64_t) g_fn[5]) (&jobu, &jobvt, &M, &N, A, &la, S, U, &lu, VT, &lv, work, &lw, &info);
        return (int) info;
    }
}
