/* Stand-in for macOS <Accelerate/Accelerate.h>, used only to compile the
 * reference's own sources (src/phipade.cpp includes it via include/phipade.h)
 * into oracle/_ref on Linux.  Declares the six BLAS/LAPACK routines the
 * reference calls and routes them to the OpenBLAS that ships with scipy
 * (LP64 symbols prefixed scipy_). */
#ifndef TSR_REF_ACCELERATE_SHIM_H
#define TSR_REF_ACCELERATE_SHIM_H
#include <stddef.h>
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
extern "C" {
void scipy_cblas_dcopy(int n, const double* x, int incx, double* y, int incy);
void scipy_cblas_dscal(int n, double a, double* x, int incx);
void scipy_cblas_daxpy(int n, double a, const double* x, int incx, double* y, int incy);
void scipy_cblas_dgemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m,
                       int n, int k, double alpha, const double* A, int lda, const double* B,
                       int ldb, double beta, double* C, int ldc);
double scipy_dlange_(const char* norm, const int* m, const int* n, const double* a, const int* lda,
                     double* work, size_t norm_len);
void scipy_dgesv_(const int* n, const int* nrhs, double* a, const int* lda, int* ipiv, double* b,
                  const int* ldb, int* info);
}
#define cblas_dcopy scipy_cblas_dcopy
#define cblas_dscal scipy_cblas_dscal
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_dgemm scipy_cblas_dgemm
static inline double dlange_(char* norm, int* m, int* n, double* a, int* lda, double* work)
{
    return scipy_dlange_(norm, m, n, a, lda, work, 1);
}
static inline void dgesv_(int* n, int* nrhs, double* a, int* lda, int* ipiv, double* b, int* ldb,
                          int* info)
{
    scipy_dgesv_(n, nrhs, a, lda, ipiv, b, ldb, info);
}
#endif
