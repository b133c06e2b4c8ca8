// Host-side helpers shared by the gbvlm translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/gbvlm.h"

namespace gbvlm {

void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define GB_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) return ::gbvlm::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

#define GB_LAUNCH_CHECK() GB_CUDA(cudaGetLastError())

#define GB_REQUIRE(cond, ...)                  \
    do {                                       \
        if (!(cond)) {                         \
            ::gbvlm::set_error(__VA_ARGS__);   \
            return GBVLM_ERR_ARG;              \
        }                                      \
    } while (0)

inline cudaStream_t to_cuda(gbvlm_stream s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Launch-shape parameters (gbvlm_tune_set); defaults are the hand-measured
// shapes, the autotuner's table overrides them per workload shape.
struct TuneParams {
    int64_t wake_waves = 4;            // split-K slices of the wake sums: about waves x SMs CTAs
    int64_t hbvlm_waves = 4;           // slices of the HBVLM wake operator, likewise
    int64_t hbvlm_min_rows = 32;       // wake rows per operator slice at least
    int64_t batch_group_hi = 1024;     // batch LU size groups: n > hi, lo < n <= hi, n <= lo
    int64_t batch_group_lo = 384;
    int64_t batch_group_mid = 0;       // 0, or a fourth group: hi > mid > lo splits lo < n <= hi at mid
    int64_t batch_loads_threads = 0;   // loads block: 0 = 64 up to 4096 unknowns, 256 beyond
    int64_t batch_assembly_span = 128; // rings per span chunk of a batch assembly tile
    int64_t batch_assembly_rows = 4;   // chordwise ring rows per float assembly tile (1-4; at most 2 with span 256)
};
TuneParams tune();
// SM count of the current device (cached per device)
int sm_count();

// Device memory for plans created and destroyed while other streams run (a
// served batch): mem == nullptr takes cudaMalloc / cudaFree; otherwise the
// memory comes stream-ordered from the device's default pool on stream
// `mem` (its release threshold raised once per device, so freed blocks stay
// in the pool), and neither allocation nor release synchronises the device
// as cudaMalloc / cudaFree do.  dev_alloc returns memory usable on any
// stream; dev_free is ordered after what `mem` waits on.
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t mem);
void dev_free(void* p, cudaStream_t mem);
// Small pinned host blocks kept for reuse (cudaFreeHost would synchronise).
void* pinned_take(size_t bytes);
void pinned_give(void* p, size_t bytes);

// Per-thread pinned staging buffer for synchronous scalar read-backs.
void* host_scratch(size_t bytes);
// Per-device small device buffer for reductions (grown on demand).
int device_scratch(size_t bytes, void** out, cudaStream_t s);

// ---------------------------------------------------------------------------
// Launch-only forms of a few operators for code captured into a CUDA graph
// and replayed at every time step: the step-dependent argument (wake rows,
// wake column, state index) is read from device memory, and nothing is
// allocated or copied from the host.
// ---------------------------------------------------------------------------
// float single-system LU solve of one right-hand side: the device tables are
// staged once by lu_solve_prepare_f32 (after the factorisation of A)
int lu_solve_prepare_f32(gbvlm_lu h, const float* A, int64_t n, float* X, void** tables, cudaStream_t st);
int lu_solve_prepared_f32(gbvlm_lu h, void* tables, int64_t n, cudaStream_t st);
void lu_solve_tables_free(void* tables);
// GBVLM_OK, or an error if a bounded wait of a float solve since the last
// factorisation ran out (synchronises st)
int lu_solve_check(gbvlm_lu h, cudaStream_t st);
// rhs -= wake influence with *it_dev active ring rows per lifting wake
// (it_dev <= it_max); scratch of WAKE_DEV_MAX_SLICES x (total panels) floats
constexpr int64_t WAKE_DEV_MAX_SLICES = 608;
int wake_influence_dev_f32(float* rhs, int32_t nsurf, const gbvlm_dims* dims, const float* const* gamma_wake,
                           const float* const* colloc, const float* const* normals, const float* const* verts_wake,
                           const int32_t* lifting, const int64_t* it_dev, int32_t it_max, float* scratch,
                           cudaStream_t st);
// wake row nwv - 1 - *it_dev <- the wing's trailing-edge row
int wake_shed_dev_f32(int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_wing, float* const* verts_wake,
                      const int64_t* it_dev, cudaStream_t st);
// gbvlm_gamma_update_f32 with the wake column col_base - *it_dev
int gamma_update_dev_f32(int64_t ns, int64_t nc, const float* x, float* gamma, float* gamma_delta, float* gamma_wake,
                         int64_t col_base, const int64_t* it_dev, const float* gamma_prev, float* dgamma_dt, float dt,
                         cudaStream_t st);
// gbvlm_newmark_step with v_i = v + ndof * (*i_dev), a_i = a + ndof * (*i_dev)
int newmark_step_dev(gbvlm_newmark h, const double* M, const double* C, const double* v, const double* a,
                     const int64_t* i_dev, double* du, double* dv, double* da, const double* delta_F, double dt,
                     cudaStream_t st);

}  // namespace gbvlm
