/*
 * Oracle build support (test infrastructure only): the CBLAS prototypes the
 * reference CPU backend calls (vlm_backend_cpu_blas.cpp), bound to the
 * prefixed exports of scipy's bundled OpenBLAS (32-bit integers).
 */
#ifndef ORACLE_REF_CBLAS_H
#define ORACLE_REF_CBLAS_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_ORDER;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef CBLAS_ORDER CBLAS_LAYOUT;

void scipy_cblas_sgemv(CBLAS_ORDER o, CBLAS_TRANSPOSE t, int m, int n, float alpha, const float* a, int lda,
                       const float* x, int incx, float beta, float* y, int incy);
void scipy_cblas_dgemv(CBLAS_ORDER o, CBLAS_TRANSPOSE t, int m, int n, double alpha, const double* a, int lda,
                       const double* x, int incx, double beta, double* y, int incy);
void scipy_cblas_sgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k, float alpha,
                       const float* a, int lda, const float* b, int ldb, float beta, float* c, int ldc);
void scipy_cblas_dgemm(CBLAS_ORDER o, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, int m, int n, int k, double alpha,
                       const double* a, int lda, const double* b, int ldb, double beta, double* c, int ldc);
void scipy_cblas_saxpy(int n, float alpha, const float* x, int incx, float* y, int incy);
void scipy_cblas_daxpy(int n, double alpha, const double* x, int incx, double* y, int incy);
void scipy_cblas_sscal(int n, float alpha, float* x, int incx);
void scipy_cblas_dscal(int n, double alpha, double* x, int incx);
float scipy_cblas_snrm2(int n, const float* x, int incx);
double scipy_cblas_dnrm2(int n, const double* x, int incx);

#define cblas_sgemv scipy_cblas_sgemv
#define cblas_dgemv scipy_cblas_dgemv
#define cblas_sgemm scipy_cblas_sgemm
#define cblas_dgemm scipy_cblas_dgemm
#define cblas_saxpy scipy_cblas_saxpy
#define cblas_daxpy scipy_cblas_daxpy
#define cblas_sscal scipy_cblas_sscal
#define cblas_dscal scipy_cblas_dscal
#define cblas_snrm2 scipy_cblas_snrm2
#define cblas_dnrm2 scipy_cblas_dnrm2

#ifdef __cplusplus
}
#endif
#endif
