/* Prototype-only CBLAS header for building the reference CPU path as a test oracle.
 * Declarations follow the public CBLAS interface; symbols resolve to the
 * scipy-bundled OpenBLAS (LP64), whose exported names carry a "scipy_" prefix. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER     { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO      { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG      { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE      { CblasLeft = 141, CblasRight = 142 };
typedef enum CBLAS_ORDER CBLAS_LAYOUT;

void   scipy_cblas_daxpy(int n, double a, const double* x, int incx, double* y, int incy);
void   scipy_cblas_dcopy(int n, const double* x, int incx, double* y, int incy);
double scipy_cblas_ddot(int n, const double* x, int incx, const double* y, int incy);
double scipy_cblas_dnrm2(int n, const double* x, int incx);
void   scipy_cblas_dscal(int n, double a, double* x, int incx);
void   scipy_cblas_dgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n, int k,
                         double alpha, const double* a, int lda, const double* b, int ldb, double beta, double* c, int ldc);
void   scipy_cblas_dgemv(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE t, int m, int n, double alpha, const double* a, int lda,
                         const double* x, int incx, double beta, double* y, int incy);
void   scipy_cblas_dger(enum CBLAS_ORDER o, int m, int n, double alpha, const double* x, int incx, const double* y, int incy,
                        double* a, int lda);
void   scipy_cblas_dspmv(enum CBLAS_ORDER o, enum CBLAS_UPLO u, int n, double alpha, const double* ap, const double* x, int incx,
                         double beta, double* y, int incy);
void   scipy_cblas_dsymm(enum CBLAS_ORDER o, enum CBLAS_SIDE s, enum CBLAS_UPLO u, int m, int n, double alpha, const double* a,
                         int lda, const double* b, int ldb, double beta, double* c, int ldc);
void   scipy_cblas_dtpmv(enum CBLAS_ORDER o, enum CBLAS_UPLO u, enum CBLAS_TRANSPOSE t, enum CBLAS_DIAG d, int n,
                         const double* ap, double* x, int incx);
void   scipy_cblas_dtrmm(enum CBLAS_ORDER o, enum CBLAS_SIDE s, enum CBLAS_UPLO u, enum CBLAS_TRANSPOSE t, enum CBLAS_DIAG d,
                         int m, int n, double alpha, const double* a, int lda, double* b, int ldb);
#ifdef __cplusplus
}
#endif
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_dcopy scipy_cblas_dcopy
#define cblas_ddot  scipy_cblas_ddot
#define cblas_dnrm2 scipy_cblas_dnrm2
#define cblas_dscal scipy_cblas_dscal
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_dger  scipy_cblas_dger
#define cblas_dspmv scipy_cblas_dspmv
#define cblas_dsymm scipy_cblas_dsymm
#define cblas_dtpmv scipy_cblas_dtpmv
#define cblas_dtrmm scipy_cblas_dtrmm
