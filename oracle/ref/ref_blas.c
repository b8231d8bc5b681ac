/*
 * ref_blas.c -- the LAPACK/BLAS names shim.h routes the reference's Fortran
 * calls to (common/lapack.h), forwarded to the OpenBLAS bound at run time by
 * ../or_blas.c.  TEST INFRASTRUCTURE ONLY (oracle/_ref libraries).
 */
#include "../or_blas.h"

int orref_dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* a, double* A, int* lda, double* B, int* ldb, double* b, double* C, int* ldc)
{
    or_dgemm(*ta, *tb, *m, *n, *k, *a, A, *lda, B, *ldb, *b, C, *ldc);
    return 0;
}

int orref_dgemv_(char* t, int* m, int* n, double* a, double* A, int* lda, double* x, int* incx, double* b, double* y, int* incy)
{
    (void) incx;
    (void) incy;
    or_dgemv(*t, *m, *n, *a, A, *lda, x, *b, y);
    return 0;
}

int orref_sgemv_(char* t, int* m, int* n, float* a, float* A, int* lda, float* x, int* incx, float* b, float* y, int* incy)
{
    (void) incx;
    (void) incy;
    or_sgemv(*t, *m, *n, *a, A, *lda, x, *b, y);
    return 0;
}

int orref_dpotrf_(char* uplo, int* n, double* A, int* lda, int* info)
{
    *info = or_dpotrf(*uplo, *n, A, *lda);
    return 0;
}

int orref_dpotri_(char* uplo, int* n, double* A, int* lda, int* info)
{
    *info = or_dpotri(*uplo, *n, A, *lda);
    return 0;
}

int orref_dgesvd_(char* ju, char* jv, int* m, int* n, double* A, int* lda, double* S, double* U, int* ldu, double* VT, int* ldvt, double* work, int* lwork, int* info)
{
    *info = or_dgesvd(*ju, *jv, *m, *n, A, *lda, S, U, *ldu, VT, *ldvt, work, *lwork);
    return 0;
}
