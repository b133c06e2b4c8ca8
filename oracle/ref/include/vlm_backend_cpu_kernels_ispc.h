// Oracle build support (test infrastructure only): the header the ISPC
// compiler would generate for vlm/backends/cpu/src/vlm_backend_cpu_kernels.ispc
// (there is no ispc compiler here).  The exported kernels keep their names
// and argument lists (ispc :106, :150, :419, :463) and are defined in
// oracle/ref/ispc_kernels.c on top of the oracle's plain-C restatement of the
// same kernels (oracle/vlm_oracle_impl.h).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
namespace ispc {
extern "C" {
#endif

void kernel_influence(int64_t m, float* lhs, float* collocs, int64_t collocs_ld, float* v, int64_t v_ld,
                      int64_t v_rld, float* normals, int64_t normals_ld, float sigma);
void kernel_wake_influence(float* colloc, int64_t colloc_ld, float* normals, int64_t normals_ld, float* v,
                           int64_t v_ld, int64_t v_m, int64_t v_n, float* gamma, float* rhs, float sigma,
                           int32_t iteration);
void dkernel_influence(int64_t m, double* lhs, double* collocs, int64_t collocs_ld, double* v, int64_t v_ld,
                       int64_t v_rld, double* normals, int64_t normals_ld, double sigma);
void dkernel_wake_influence(double* colloc, int64_t colloc_ld, double* normals, int64_t normals_ld, double* v,
                            int64_t v_ld, int64_t v_m, int64_t v_n, double* gamma, double* rhs, double sigma,
                            int32_t iteration);

#ifdef __cplusplus
}  // extern "C"
}  // namespace ispc
#endif
