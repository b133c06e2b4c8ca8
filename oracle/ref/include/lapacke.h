/*
 * Oracle build support (test infrastructure only): the LAPACKE prototypes the
 * reference CPU backend calls (vlm_backend_cpu_lapack.cpp), bound to the
 * prefixed exports of scipy's bundled OpenBLAS (32-bit integers), which is
 * the library this build links.  The reference pins OpenBLAS 0.3.26/0.3.29
 * (packages/openblas.lua); scipy bundles 0.3.31.
 */
#ifndef ORACLE_REF_LAPACKE_H
#define ORACLE_REF_LAPACKE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

lapack_int scipy_LAPACKE_sgetrf(int layout, lapack_int m, lapack_int n, float* a, lapack_int lda, lapack_int* ipiv);
lapack_int scipy_LAPACKE_dgetrf(int layout, lapack_int m, lapack_int n, double* a, lapack_int lda, lapack_int* ipiv);
lapack_int scipy_LAPACKE_sgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const float* a, lapack_int lda,
                                const lapack_int* ipiv, float* b, lapack_int ldb);
lapack_int scipy_LAPACKE_dgetrs(int layout, char trans, lapack_int n, lapack_int nrhs, const double* a,
                                lapack_int lda, const lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int scipy_LAPACKE_sgels_work(int layout, char trans, lapack_int m, lapack_int n, lapack_int nrhs, float* a,
                                    lapack_int lda, float* b, lapack_int ldb, float* work, lapack_int lwork);
lapack_int scipy_LAPACKE_dgels_work(int layout, char trans, lapack_int m, lapack_int n, lapack_int nrhs, double* a,
                                    lapack_int lda, double* b, lapack_int ldb, double* work, lapack_int lwork);

#define LAPACKE_sgetrf scipy_LAPACKE_sgetrf
#define LAPACKE_dgetrf scipy_LAPACKE_dgetrf
#define LAPACKE_sgetrs scipy_LAPACKE_sgetrs
#define LAPACKE_dgetrs scipy_LAPACKE_dgetrs
#define LAPACKE_sgels_work scipy_LAPACKE_sgels_work
#define LAPACKE_dgels_work scipy_LAPACKE_dgels_work

#ifdef __cplusplus
}
#endif
#endif
