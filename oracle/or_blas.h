/*
 * or_blas.h -- BLAS/LAPACK entry points for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the GPU library;
 * it is never linked into, loaded by, or called from the product path.
 *
 * EnKF-C calls LAPACK/BLAS through the Fortran ABI (reference
 * enkf/common/lapack.h:17-28: dgemm_, dgemv_, sgemv_, dpotrf_, dpotri_,
 * dgesvd_).  Neither MKL nor a system LAPACK is present on the machines this
 * project runs on, so the oracle binds those six routines at run time from the
 * OpenBLAS that ships inside the scipy wheel (LP64 "scipy_" prefixed symbols,
 * or the ILP64 "scipy_..._64_" build as a fallback).  This is the one recorded
 * deviation of the oracle from the reference build (MKL).
 */
#ifndef OR_BLAS_H
#define OR_BLAS_H

#ifdef __cplusplus
extern "C" {
#endif

/* Load the library at `path` and resolve the routines.  Returns 0 on success,
 * a negative number naming the first routine that could not be resolved
 * otherwise.  Also pins the library to one thread per caller. */
int or_blas_load(const char* path);
int or_blas_loaded(void);

/* Fortran-ABI style wrappers (LP64 ints), same argument meaning as LAPACK. */
void or_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb, double beta, double* C, int ldc);
void or_dgemv(char t, int m, int n, double alpha, const double* A, int lda, const double* x, double beta, double* y);
void or_sgemv(char t, int m, int n, float alpha, const float* A, int lda, const float* x, float beta, float* y);
int or_dpotrf(char uplo, int n, double* A, int lda);
int or_dpotri(char uplo, int n, double* A, int lda);
int or_dgesvd(char jobu, char jobvt, int m, int n, double* A, int lda, double* S, double* U, int ldu, double* VT, int ldvt, double* work, int lwork);

#ifdef __cplusplus
}
#endif
#endif
