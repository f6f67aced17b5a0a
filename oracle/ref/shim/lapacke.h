/* Prototype-only LAPACKE header for building the reference CPU path as a test oracle.
 * Declarations follow the public LAPACKE interface; symbols resolve to the
 * scipy-bundled OpenBLAS (LP64), whose exported names carry a "scipy_" prefix. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
double     scipy_LAPACKE_dlange(int layout, char norm, lapack_int m, lapack_int n, const double* a, lapack_int lda);
lapack_int scipy_LAPACKE_dsptrf(int layout, char uplo, lapack_int n, double* ap, lapack_int* ipiv);
lapack_int scipy_LAPACKE_dsptrs(int layout, char uplo, lapack_int n, lapack_int nrhs, const double* ap,
                                const lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int scipy_LAPACKE_dsptri(int layout, char uplo, lapack_int n, double* ap, const lapack_int* ipiv);
lapack_int scipy_LAPACKE_dpptrf(int layout, char uplo, lapack_int n, double* ap);
lapack_int scipy_LAPACKE_dpptri(int layout, char uplo, lapack_int n, double* ap);
lapack_int scipy_LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv);
lapack_int scipy_LAPACKE_dgetri(int layout, lapack_int n, double* a, lapack_int lda, const lapack_int* ipiv);
lapack_int scipy_LAPACKE_dgesdd(int layout, char jobz, lapack_int m, lapack_int n, double* a, lapack_int lda, double* s,
                                double* u, lapack_int ldu, double* vt, lapack_int ldvt);
lapack_int scipy_LAPACKE_dspevd(int layout, char jobz, char uplo, lapack_int n, double* ap, double* w, double* z,
                                lapack_int ldz);
lapack_int scipy_LAPACKE_dtptri(int layout, char uplo, char diag, lapack_int n, double* ap);
#ifdef __cplusplus
}
#endif
#define LAPACKE_dlange scipy_LAPACKE_dlange
#define LAPACKE_dsptrf scipy_LAPACKE_dsptrf
#define LAPACKE_dsptrs scipy_LAPACKE_dsptrs
#define LAPACKE_dsptri scipy_LAPACKE_dsptri
#define LAPACKE_dpptrf scipy_LAPACKE_dpptrf
#define LAPACKE_dpptri scipy_LAPACKE_dpptri
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_dgetri scipy_LAPACKE_dgetri
#define LAPACKE_dgesdd scipy_LAPACKE_dgesdd
#define LAPACKE_dspevd scipy_LAPACKE_dspevd
#define LAPACKE_dtptri scipy_LAPACKE_dtptri
