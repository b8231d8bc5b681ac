/*
 * shim.h -- force-included when compiling the reference's own calc/calcs.c
 * and common/kdtree.c (unmodified) into oracle/_ref.  TEST INFRASTRUCTURE.
 *
 * The reference calls LAPACK/BLAS by their Fortran names (common/lapack.h);
 * these names are routed to wrappers in ref_stubs.c, which call the OpenBLAS
 * bound at run time by ../or_blas.c.
 */
#define dgemm_ orref_dgemm_
#define dgemv_ orref_dgemv_
#define sgemv_ orref_sgemv_
#define dpotrf_ orref_dpotrf_
#define dpotri_ orref_dpotri_
#define dgesvd_ orref_dgesvd_
