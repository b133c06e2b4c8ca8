/*
 * Oracle build support (test infrastructure only): the four ISPC kernels the
 * reference CPU backend calls, as thin forwards to the oracle's plain-C
 * restatement (oracle/vlm_oracle_impl.h, compiled into the same binary from
 * oracle/vlm_oracle.c).  The argument lists are the ISPC exports'
 * (vlm_backend_cpu_kernels.ispc:106, :150, :419, :463).
 */
#include <stdint.h>

#include "vlm_backend_cpu_kernels_ispc.h"

void orc_influence_f(int64_t m, float* lhs, const float* collocs, int64_t collocs_ld, const float* v, int64_t v_ld,
                     int64_t v_rld, const float* normals, int64_t normals_ld, float sigma);
void orc_influence_d(int64_t m, double* lhs, const double* collocs, int64_t collocs_ld, const double* v,
                     int64_t v_ld, int64_t v_rld, const double* normals, int64_t normals_ld, double sigma);
void orc_wake_influence_f(const float* colloc, int64_t colloc_ld, const float* normals, int64_t normals_ld,
                          const float* v, int64_t v_ld, int64_t v_m, int64_t v_n, const float* gamma, float* rhs,
                          float sigma, int32_t iteration);
void orc_wake_influence_d(const double* colloc, int64_t colloc_ld, const double* normals, int64_t normals_ld,
                          const double* v, int64_t v_ld, int64_t v_m, int64_t v_n, const double* gamma, double* rhs,
                          double sigma, int32_t iteration);

void kernel_influence(int64_t m, float* lhs, float* collocs, int64_t collocs_ld, float* v, int64_t v_ld,
                      int64_t v_rld, float* normals, int64_t normals_ld, float sigma) {
    orc_influence_f(m, lhs, collocs, collocs_ld, v, v_ld, v_rld, normals, normals_ld, sigma);
}

void kernel_wake_influence(float* colloc, int64_t colloc_ld, float* normals, int64_t normals_ld, float* v,
                           int64_t v_ld, int64_t v_m, int64_t v_n, float* gamma, float* rhs, float sigma,
                           int32_t iteration) {
    orc_wake_influence_f(colloc, colloc_ld, normals, normals_ld, v, v_ld, v_m, v_n, gamma, rhs, sigma, iteration);
}

void dkernel_influence(int64_t m, double* lhs, double* collocs, int64_t collocs_ld, double* v, int64_t v_ld,
                       int64_t v_rld, double* normals, int64_t normals_ld, double sigma) {
    orc_influence_d(m, lhs, collocs, collocs_ld, v, v_ld, v_rld, normals, normals_ld, sigma);
}

void dkernel_wake_influence(double* colloc, int64_t colloc_ld, double* normals, int64_t normals_ld, double* v,
                            int64_t v_ld, int64_t v_m, int64_t v_n, double* gamma, double* rhs, double sigma,
                            int32_t iteration) {
    orc_wake_influence_d(colloc, colloc_ld, normals, normals_ld, v, v_ld, v_m, v_n, gamma, rhs, sigma, iteration);
}
