/*
 * gbvlm -- GB300-native vortex-lattice hot path, C ABI.
 *
 * One entry point per operator of the tinyvlm plugin API (class vlm::Backend
 * and its BLAS/LU helpers, vlm/include/vlm_backend.hpp:13-136) in both of the
 * reference's precisions, plus the simulation drivers (vlm/include/vlm.hpp)
 * and the batched steady solver.  Each declaration cites the reference
 * interface it replaces.
 *
 * Conventions (identical to the reference's tensors, vlm/include/vlm_memory.hpp):
 *  - every array is column-major (first index fastest) and contiguous;
 *  - per surface m (a half wing mirrored in y = 0):
 *      wing vertices  (ns+1, nc+1, 4)   x, y, z, w planes
 *      panel vectors  (ns, nc, 3)       colloc, normals, velocities, forces
 *      panel scalars  (ns, nc)          areas, gamma, gamma_delta, dgamma_dt
 *      wake vertices  (ns+1, nwv, 4)    newest row at index nwv-1-iteration
 *      wake gamma     (ns, nwv-1)
 *  - the LHS is (n, n) with leading dimension ld: row = collocation point,
 *    column = influencing ring; surface blocks are contiguous;
 *  - multi-surface arguments are HOST arrays holding one DEVICE pointer per
 *    surface (the reference's MultiTensorView);
 *  - scalars returned through a host pointer are read back synchronously,
 *    like the reference's scalar-returning backend calls; every other call
 *    is asynchronous on `stream` (0 = legacy default stream);
 *  - every function returns GBVLM_OK or an error code; gbvlm_last_error()
 *    gives the message.  The reference prints and exits instead
 *    (vlm_backend_cuda.cu:21-29); callers that want that behaviour test the
 *    return code.
 */
#ifndef GBVLM_H
#define GBVLM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gbvlm_stream; /* same handle as cudaStream_t */

enum {
    GBVLM_OK = 0,
    GBVLM_ERR_ARG = 1,      /* invalid argument (sizes, null pointers, too many surfaces) */
    GBVLM_ERR_CUDA = 2,     /* a CUDA runtime call failed */
    GBVLM_ERR_SINGULAR = 3, /* exact zero pivot met in an LU factorisation */
    GBVLM_ERR_NOMEM = 4,    /* device allocation failed */
    GBVLM_ERR_IO = 5,       /* mesh file could not be read */
    GBVLM_ERR_STATE = 6     /* handle used out of order */
};

#define GBVLM_MAX_SURFACES 16

/* Sizes of one surface: ns spanwise panels, nc chordwise panels, nwv wake
 * vertex rows (0 when the call does not touch the wake). */
typedef struct {
    int64_t ns, nc, nwv;
} gbvlm_dims;

const char* gbvlm_last_error(void);
int gbvlm_version(void);

/* ---------------------------------------------------------------------------
 * Memory: replaces vlm::Memory (vlm/include/vlm_memory.hpp:22-37), the
 * manager Backend::create_memory_manager returns (vlm_backend.hpp:72).
 * Locations follow vlm::Location: Device memory is cudaMalloc'd, Host memory
 * is pinned (cudaMallocHost), as the reference's CUDA backend allocates it
 * (vlm_backend_cuda.cu:90-107).
 * ------------------------------------------------------------------------- */
enum { GBVLM_LOC_DEVICE = 0, GBVLM_LOC_HOST = 1 };
/* Memory::alloc / Memory::free.  GBVLM_ERR_NOMEM when the allocation fails. */
int gbvlm_mem_alloc(int32_t location, int64_t bytes, void** out);
int gbvlm_mem_free(int32_t location, void* ptr);
/* Memory::copy: `size` elements of `elem_size` bytes, element strides
 * dst_stride and src_stride (>= 1).  Stream-ordered between device buffers;
 * synchronous when either side is host memory (the reference's copy returns
 * with the data in place, vlm_backend_cuda.cu:109-126). */
int gbvlm_mem_copy(int32_t dst_loc, void* dst, int64_t dst_stride, int32_t src_loc, const void* src,
                   int64_t src_stride, int64_t elem_size, int64_t size, gbvlm_stream stream);
/* Memory::fill (float and double overloads). */
int gbvlm_mem_fill_f32(int32_t location, float* ptr, int64_t stride, float value, int64_t size, gbvlm_stream stream);
int gbvlm_mem_fill_f64(int32_t location, double* ptr, int64_t stride, double value, int64_t size,
                       gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * BLAS: replaces vlm::BLAS (vlm_backend.hpp:78-97) with the argument meaning
 * of the reference's CBLAS/cuBLAS calls (vlm_backend_cpu_blas.cpp,
 * vlm_backend_cuda_blas.cu): column-major, trans = 0 (Trans::No) or 1
 * (Trans::Yes), element strides inc >= 1.  Stream-ordered except nrm2,
 * which returns its scalar synchronously like BLAS::norm.
 * ------------------------------------------------------------------------- */
/* BLAS::gemv: y = alpha op(A) x + beta y, A m x n (beta = 0: y is not read). */
int gbvlm_blas_gemv_f32(int32_t trans, int64_t m, int64_t n, float alpha, const float* A, int64_t lda,
                        const float* x, int64_t incx, float beta, float* y, int64_t incy, gbvlm_stream stream);
int gbvlm_blas_gemv_f64(int32_t trans, int64_t m, int64_t n, double alpha, const double* A, int64_t lda,
                        const double* x, int64_t incx, double beta, double* y, int64_t incy, gbvlm_stream stream);
/* BLAS::gemm: C = alpha op(A) op(B) + beta C, C m x n, inner size k. */
int gbvlm_blas_gemm_f32(int32_t trans_a, int32_t trans_b, int64_t m, int64_t n, int64_t k, float alpha,
                        const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                        gbvlm_stream stream);
int gbvlm_blas_gemm_f64(int32_t trans_a, int32_t trans_b, int64_t m, int64_t n, int64_t k, double alpha,
                        const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
                        int64_t ldc, gbvlm_stream stream);
/* BLAS::axpy, 1-D: y += alpha x. */
int gbvlm_blas_axpy_f32(int64_t n, float alpha, const float* x, int64_t incx, float* y, int64_t incy,
                        gbvlm_stream stream);
int gbvlm_blas_axpy_f64(int64_t n, double alpha, const double* x, int64_t incx, double* y, int64_t incy,
                        gbvlm_stream stream);
/* BLAS::axpy, 2-D (vlm_backend_cpu_blas.cpp:101-106): y(i, j) += alpha x(i, j)
 * over an m x n view, element strides (s0, s1) for each operand. */
int gbvlm_blas_axpy2d_f32(int64_t m, int64_t n, float alpha, const float* x, int64_t x_s0, int64_t x_s1, float* y,
                          int64_t y_s0, int64_t y_s1, gbvlm_stream stream);
int gbvlm_blas_axpy2d_f64(int64_t m, int64_t n, double alpha, const double* x, int64_t x_s0, int64_t x_s1, double* y,
                          int64_t y_s0, int64_t y_s1, gbvlm_stream stream);
/* BLAS::scal: x *= alpha. */
int gbvlm_blas_scal_f32(int64_t n, float alpha, float* x, int64_t incx, gbvlm_stream stream);
int gbvlm_blas_scal_f64(int64_t n, double alpha, double* x, int64_t incx, gbvlm_stream stream);
/* BLAS::norm: Euclidean norm into *out (host), scaled so no finite input
 * overflows. */
int gbvlm_blas_nrm2_f32(int64_t n, const float* x, int64_t incx, float* out, gbvlm_stream stream);
int gbvlm_blas_nrm2_f64(int64_t n, const double* x, int64_t incx, double* out, gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * LSQ: replaces vlm::LSQ::solve (vlm_backend.hpp:121-133;
 * vlm_backend_cpu_lapack.cpp:123-205, LAPACK ?gels with trans = 'N'):
 * min ||A x - B|| for A m x n (m >= n, full column rank) by Householder QR.
 * The first n rows of B receive x, rows n..m-1 the residual components; A is
 * overwritten (R in its upper triangle).  Synchronous; GBVLM_ERR_SINGULAR if
 * R has an exactly zero diagonal.  LSQ::init has nothing to size: the
 * solver keeps no workspace.
 * ------------------------------------------------------------------------- */
int gbvlm_lsq_solve_f32(int64_t m, int64_t n, float* A, int64_t lda, float* B, int64_t nrhs, int64_t ldb,
                        gbvlm_stream stream);
int gbvlm_lsq_solve_f64(int64_t m, int64_t n, double* A, int64_t lda, double* B, int64_t nrhs, int64_t ldb,
                        gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Streams, events and device queries: no reference counterpart (the
 * reference's CUDA backend runs on the legacy default stream).  They let a
 * host without another CUDA binding order, time and size its work.
 * ------------------------------------------------------------------------- */
typedef struct CUevent_st* gbvlm_event; /* same handle as cudaEvent_t */
int gbvlm_stream_create(gbvlm_stream* out); /* non-blocking stream */
int gbvlm_stream_destroy(gbvlm_stream s);
int gbvlm_stream_synchronize(gbvlm_stream s);
int gbvlm_device_synchronize(void);
int gbvlm_event_create(gbvlm_event* out);
int gbvlm_event_destroy(gbvlm_event e);
int gbvlm_event_record(gbvlm_event e, gbvlm_stream s);
int gbvlm_event_synchronize(gbvlm_event e);
int gbvlm_event_elapsed_ms(gbvlm_event start, gbvlm_event end, float* ms);
/* Current device: SM count and free / total device memory in bytes (NULL
 * pointers are skipped). */
int gbvlm_device_info(int32_t* sm_count, int64_t* free_bytes, int64_t* total_bytes);

/* ---------------------------------------------------------------------------
 * Launch-shape tuning: no reference counterpart (the reference fixes its
 * launch shapes, e.g. kernel_influence's (32, 16) blocks,
 * vlm_backend_cuda.cu:171).  A process-wide table of named integer
 * parameters; tinyvlm_gb300/autotune.py searches them per workload shape and
 * keeps the choices in a committed table.  Defaults are the hand-measured
 * shapes.  A batch plan copies the values when it is created; the other
 * calls read them at each launch.
 *   wake.waves           1..16   split-K slices of the wake sums: about
 *                                waves x SMs CTAs (default 4)
 *   hbvlm.waves          1..16   slices of the HBVLM wake operator (4)
 *   hbvlm.min_rows       8..512  wake rows per operator slice at least (32)
 *   batch.group_hi/lo            batch LU size groups: n > hi, lo < n <= hi,
 *                                n <= lo (1024, 384); hi > lo
 *   batch.group_mid      0 or hi > mid > lo: a fourth group, lo < n <= hi split at
 *                        mid (0)
 *   batch.loads_threads  0, 32, 64, 128, 256: the loads block (0: by size)
 *   batch.assembly_span  64, 128, 256: rings per assembly span chunk (128)
 *   batch.assembly_rows  1-4: chordwise ring rows per float assembly tile (4; at most 2 with
 *                        span 256)
 * ------------------------------------------------------------------------- */
int gbvlm_tune_set(const char* name, int64_t value);
int gbvlm_tune_get(const char* name, int64_t* value);
int gbvlm_tune_reset(void);
/* The parameters: their number, and name and range by index. */
int gbvlm_tune_count(int32_t* n);
int gbvlm_tune_name(int32_t i, const char** name, int64_t* lo, int64_t* hi);

/* ---------------------------------------------------------------------------
 * Backend operators.  Replaces the pure virtuals of vlm::Backend
 * (vlm/include/vlm_backend.hpp:31-55); semantics follow the CPU backend
 * vlm/backends/cpu/src/vlm_backend_cpu.cpp (f32) and vlm_backend_cpud.cpp (f64).
 * ------------------------------------------------------------------------- */

/* Backend::lhs_assemble (vlm_backend.hpp:31/45; vlm_backend_cpu.cpp:84-148).
 * lhs += AIC; the trailing-edge columns also get the wake ring rows
 * nwv-2-c, c < iteration (Kutta condition).  Zero lhs first. */
int gbvlm_lhs_assemble_f32(float* lhs, int64_t ld, int32_t nsurf, const gbvlm_dims* dims,
                           const float* const* colloc, const float* const* normals,
                           const float* const* verts_wing, const float* const* verts_wake,
                           int32_t iteration, float sigma, gbvlm_stream stream);
int gbvlm_lhs_assemble_f64(double* lhs, int64_t ld, int32_t nsurf, const gbvlm_dims* dims,
                           const double* const* colloc, const double* const* normals,
                           const double* const* verts_wing, const double* const* verts_wake,
                           int32_t iteration, double sigma, gbvlm_stream stream);

/* Backend::rhs_assemble_velocities (vlm_backend.hpp:32/46; vlm_backend_cpu.cpp:156-179).
 * rhs[p] += -(V_p . n_p), surfaces packed in order. */
int gbvlm_rhs_assemble_velocities_f32(float* rhs, int32_t nsurf, const gbvlm_dims* dims,
                                      const float* const* normals, const float* const* velocities,
                                      gbvlm_stream stream);
int gbvlm_rhs_assemble_velocities_f64(double* rhs, int32_t nsurf, const gbvlm_dims* dims,
                                      const double* const* normals, const double* const* velocities,
                                      gbvlm_stream stream);

/* Backend::rhs_assemble_wake_influence (vlm_backend.hpp:33/47; vlm_backend_cpu.cpp:181-224).
 * rhs[p] -= (sum over the last `iteration` wake ring rows of every lifting
 * surface of gamma_r v_r(colloc_p)) . n_p.  The f32 variant keeps the
 * reference's 5000-row window.  lifting is a host array of nsurf flags. */
int gbvlm_rhs_assemble_wake_influence_f32(float* rhs, int32_t nsurf, const gbvlm_dims* dims,
                                          const float* const* gamma_wake, const float* const* colloc,
                                          const float* const* normals, const float* const* verts_wake,
                                          const int32_t* lifting, int32_t iteration, float sigma,
                                          gbvlm_stream stream);
int gbvlm_rhs_assemble_wake_influence_f64(double* rhs, int32_t nsurf, const gbvlm_dims* dims,
                                          const double* const* gamma_wake, const double* const* colloc,
                                          const double* const* normals, const double* const* verts_wake,
                                          const int32_t* lifting, int32_t iteration, double sigma,
                                          gbvlm_stream stream);

/* No counterpart in the reference.  Same as
 * gbvlm_rhs_assemble_wake_influence_f32, for callers that cannot allocate
 * device memory: a host application whose device memory is owned by its own
 * allocator, a serving loop held to a fixed device-memory budget, or a
 * latency path that must not take cudaMalloc's device-wide synchronisation.
 * The split-K partial sums go to a fixed 4 MiB array in this library's
 * device image instead of scratch grown with cudaMalloc.  At most 1,048,576
 * collocation points (all surfaces); larger problems are rejected with
 * GBVLM_ERR_ARG.  The first call on a device looks the array up with
 * cudaGetSymbolAddress.  Calls share the array, so calls whose kernels
 * overlap on the GPU race. */
int gbvlm_rhs_assemble_wake_influence_f32_noalloc(float* rhs, int32_t nsurf, const gbvlm_dims* dims,
                                                  const float* const* gamma_wake, const float* const* colloc,
                                                  const float* const* normals, const float* const* verts_wake,
                                                  const int32_t* lifting, int32_t iteration, float sigma,
                                                  gbvlm_stream stream);

/* Backend::forces_steady (vlm_backend.hpp:34/48; vlm_backend_cpu.cpp:276-297), rho = 1. */
int gbvlm_forces_steady_f32(int64_t ns, int64_t nc, const float* verts_wing, const float* gamma_delta,
                            const float* velocities, float* forces, gbvlm_stream stream);
int gbvlm_forces_steady_f64(int64_t ns, int64_t nc, const double* verts_wing, const double* gamma_delta,
                            const double* velocities, double* forces, gbvlm_stream stream);

/* Backend::forces_unsteady (vlm_backend.hpp:35/49; vlm_backend_cpu.cpp:299-321), rho = 1. */
int gbvlm_forces_unsteady_f32(int64_t ns, int64_t nc, const float* verts_wing, const float* gamma_delta,
                              const float* dgamma_dt, const float* velocities, const float* areas,
                              const float* normals, float* forces, gbvlm_stream stream);
int gbvlm_forces_unsteady_f64(int64_t ns, int64_t nc, const double* verts_wing, const double* gamma_delta,
                              const double* dgamma_dt, const double* velocities, const double* areas,
                              const double* normals, double* forces, gbvlm_stream stream);

/* Backend::coeff_cl (vlm_backend.hpp:36/50; vlm_backend_cpu.cpp:323-338).
 * lift_axis, freestream: host float[3]/double[3].  Sums in double with
 * compensation.  *out is written synchronously. */
int gbvlm_coeff_cl_f32(int64_t ns, int64_t nc, const float* forces, const float* lift_axis,
                       const float* freestream, float rho, float area, float* out, gbvlm_stream stream);
int gbvlm_coeff_cl_f64(int64_t ns, int64_t nc, const double* forces, const double* lift_axis,
                       const double* freestream, double rho, double area, double* out, gbvlm_stream stream);

/* Backend::coeff_cm (vlm_backend.hpp:37/51; vlm_backend_cpu.cpp:340-362).  out: host [3]. */
int gbvlm_coeff_cm_f32(int64_t ns, int64_t nc, const float* forces, const float* verts_wing,
                       const float* ref_pt, const float* freestream, float rho, float area, float mac,
                       float* out, gbvlm_stream stream);
int gbvlm_coeff_cm_f64(int64_t ns, int64_t nc, const double* forces, const double* verts_wing,
                       const double* ref_pt, const double* freestream, double rho, double area, double mac,
                       double* out, gbvlm_stream stream);

/* Backend::mesh_metrics (vlm_backend.hpp:38/52; vlm_backend_cpu.cpp:391-433):
 * normals, areas and collocation points with the high-AoA factor. */
int gbvlm_mesh_metrics_f32(float alpha_rad, int32_t nsurf, const gbvlm_dims* dims,
                           const float* const* verts_wing, float* const* colloc, float* const* normals,
                           float* const* areas, gbvlm_stream stream);
int gbvlm_mesh_metrics_f64(double alpha_rad, int32_t nsurf, const gbvlm_dims* dims,
                           const double* const* verts_wing, double* const* colloc, double* const* normals,
                           double* const* areas, gbvlm_stream stream);

/* Backend::mesh_mac (vlm_backend.hpp:39/53; vlm_backend_cpu.cpp:443-468). *out synchronous. */
int gbvlm_mesh_mac_f32(int64_t ns, int64_t nc, const float* verts_wing, const float* areas, float* out,
                       gbvlm_stream stream);
int gbvlm_mesh_mac_f64(int64_t ns, int64_t nc, const double* verts_wing, const double* areas, double* out,
                       gbvlm_stream stream);

/* Backend::gamma_wake_from_coeffs (vlm_backend.hpp:40/54; vlm_backend_cpu.cpp:470-503).
 * gamma_wake (ns, ncols), coeffs (ns, 2*harmonics+1); fills the last
 * `iteration` columns. */
int gbvlm_gamma_wake_from_coeffs_f32(float* gamma_wake, int64_t ns, int64_t ncols, const float* coeffs,
                                     int32_t harmonics, float tn, float omega, float dt, int64_t iteration,
                                     gbvlm_stream stream);
int gbvlm_gamma_wake_from_coeffs_f64(double* gamma_wake, int64_t ns, int64_t ncols, const double* coeffs,
                                     int32_t harmonics, double tn, double omega, double dt, int64_t iteration,
                                     gbvlm_stream stream);

/* Backend::sum (vlm_backend.hpp:41-42/55-56; vlm_backend_cpu.cpp:506-523). *out synchronous. */
int gbvlm_sum_f32(const float* x, int64_t n, float* out, gbvlm_stream stream);
int gbvlm_sum_f64(const double* x, int64_t n, double* out, gbvlm_stream stream);
/* Backend::sum(TV2f&) (vlm_backend.hpp:43/54; vlm_backend_cpu.cpp:515-523):
 * the sum of an m x n view with element strides (stride0, stride1),
 * compensated in double, returned synchronously. */
int gbvlm_sum2d_f32(const float* x, int64_t m, int64_t n, int64_t stride0, int64_t stride1, float* out,
                    gbvlm_stream stream);
int gbvlm_sum2d_f64(const double* x, int64_t m, int64_t n, int64_t stride0, int64_t stride1, double* out,
                    gbvlm_stream stream);

/* Backend::displace_wing (vlm_backend.hpp:59/66; vlm_backend.cpp:50-69):
 * verts = verts_init . T^T per surface; transforms: device 4x4 column-major. */
int gbvlm_displace_wing_f32(int32_t nsurf, const gbvlm_dims* dims, const float* const* transforms,
                            float* const* verts_wing, const float* const* verts_wing_init, gbvlm_stream stream);
int gbvlm_displace_wing_f64(int32_t nsurf, const gbvlm_dims* dims, const double* const* transforms,
                            double* const* verts_wing, const double* const* verts_wing_init, gbvlm_stream stream);

/* Backend::wake_shed (vlm_backend.hpp:60/67; vlm_backend.cpp:43-47):
 * wing trailing-edge vertex row -> wake row nwv-1-iteration. */
int gbvlm_wake_shed_f32(int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_wing,
                        float* const* verts_wake, int32_t iteration, gbvlm_stream stream);
int gbvlm_wake_shed_f64(int32_t nsurf, const gbvlm_dims* dims, const double* const* verts_wing,
                        double* const* verts_wake, int32_t iteration, gbvlm_stream stream);

/* Free-wake roll-up: ispc::kernel_rollup (vlm_backend_cpu_kernels.ispc:215-271),
 * whose caller the reference comments out (vlm_backend_cpu.cpp:226-274).
 * Moves wake vertex rows [nwv-iteration, nwv) of every surface by dt times
 * the velocity of all wing rings (gamma_wing (ns,nc)) and of the last
 * `iteration` ring rows of every lifting wake.  Positions are read before
 * any is written. */
int gbvlm_wake_rollup_f32(int32_t nsurf, const gbvlm_dims* dims, float* const* verts_wake,
                          const float* const* verts_wing, const float* const* gamma_wing,
                          const float* const* gamma_wake, const int32_t* lifting, float sigma, float dt,
                          int32_t iteration, gbvlm_stream stream);
int gbvlm_wake_rollup_f64(int32_t nsurf, const gbvlm_dims* dims, double* const* verts_wake,
                          const double* const* verts_wing, const double* const* gamma_wing,
                          const double* const* gamma_wake, const int32_t* lifting, double sigma, double dt,
                          int32_t iteration, gbvlm_stream stream);

/* Trefftz-plane induced drag: ispc::kernel_trefftz_cd
 * (vlm_backend_cpu_kernels.ispc:273-323) divided by |V|^2 * area as its
 * commented caller does (vlm_backend_cpu.cpp:364-369).  *out synchronous. */
int gbvlm_trefftz_cd_f32(int64_t ns, int64_t nwv, const float* verts_wake, const float* gamma_wake,
                         const float* freestream, float area, float sigma, float* out, gbvlm_stream stream);
int gbvlm_trefftz_cd_f64(int64_t ns, int64_t nwv, const double* verts_wake, const double* gamma_wake,
                         const double* freestream, double area, double sigma, double* out, gbvlm_stream stream);

/* Circulation post-processing of one surface after a solve, fused
 * (vlm/src/vlm.cpp:442-458): gamma = x[0:ns*nc]; gamma_delta = gamma with
 * the previous chordwise row subtracted; if gamma_wake is not null, the
 * trailing-edge row goes to wake column `wake_col`; if dgamma_dt is not null,
 * dgamma_dt = (gamma - gamma_prev) / dt.  gamma_prev is then left untouched. */
int gbvlm_gamma_update_f32(int64_t ns, int64_t nc, const float* x, float* gamma, float* gamma_delta,
                           float* gamma_wake, int64_t wake_col, const float* gamma_prev, float* dgamma_dt,
                           float dt, gbvlm_stream stream);
int gbvlm_gamma_update_f64(int64_t ns, int64_t nc, const double* x, double* gamma, double* gamma_delta,
                           double* gamma_wake, int64_t wake_col, const double* gamma_prev, double* dgamma_dt,
                           double dt, gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Dense LU.  Replaces vlm::LU (vlm_backend.hpp:99-119): CPU LAPACKE
 * ?getrf/?getrs (vlm_backend_cpu_lapack.cpp:17-94), CUDA cuSOLVER
 * (vlm_backend_cuda_solvers.cu:39-102).  Partial pivoting (LAPACK pivot
 * order: largest |a|, first index on ties); ipiv is 0-based on device.
 * ------------------------------------------------------------------------- */
typedef struct gbvlm_lu_s* gbvlm_lu;
int gbvlm_lu_create(gbvlm_lu* out);
int gbvlm_lu_destroy(gbvlm_lu h);
/* LU::init: reserve workspace for an n x n matrix */
int gbvlm_lu_init(gbvlm_lu h, int64_t n);
/* LU::factorize: A (n x n, leading dimension ld) overwritten by L\U */
int gbvlm_lu_factor_f32(gbvlm_lu h, float* A, int64_t n, int64_t ld, gbvlm_stream stream);
int gbvlm_lu_factor_f64(gbvlm_lu h, double* A, int64_t n, int64_t ld, gbvlm_stream stream);
/* LU::solve: X (n x nrhs, leading dimension ldx) overwritten by A^-1 X */
int gbvlm_lu_solve_f32(gbvlm_lu h, const float* A, int64_t n, int64_t ld, float* X, int64_t ldx,
                       int64_t nrhs, gbvlm_stream stream);
int gbvlm_lu_solve_f64(gbvlm_lu h, const double* A, int64_t n, int64_t ld, double* X, int64_t ldx,
                       int64_t nrhs, gbvlm_stream stream);
/* Mixed precision: solve A x = b with the float LU of A (from
 * gbvlm_lu_factor_f32 of a copy) and `iters` steps of iterative refinement
 * whose residual b - A x is formed in double from the unfactored float A.
 * b, x: double (n x nrhs).  Returns the final max-norm relative residual
 * correction in *last_update when not null (synchronous only then). */
int gbvlm_lu_solve_refined(gbvlm_lu h, const float* LU, const float* A, int64_t n, int64_t ld,
                           const double* B, double* X, int64_t nrhs, int32_t iters, double* last_update,
                           gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Simulation drivers (vlm/include/vlm.hpp), device-resident.
 * ------------------------------------------------------------------------- */
typedef struct gbvlm_vlm_s* gbvlm_vlm;

/* Results of one steady solve.  cl follows VLM::run (vlm/src/vlm.cpp:97-151);
 * cdi is the Trefftz drag (area-weighted like CL) and cm the
 * coeff_cm_multibody moment about ref_pt, which VLM::run leaves at zero. */
typedef struct {
    double cl, cdi, cm[3];
} gbvlm_coeffs;

/* VLM(backend, meshes) (vlm/src/vlm.cpp:17-58).  verts_init: HOST arrays,
 * one (ns+1, nc+1, 4) float array per surface, already quarter-chord
 * shifted (the plot3d reader does it, gbvlm_read_plot3d).  precision: 32
 * runs the reference's float semantics; 64 the plain per-solve double
 * path. */
int gbvlm_vlm_create(gbvlm_vlm* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                     int32_t precision);
int gbvlm_vlm_destroy(gbvlm_vlm h);
/* VLM::run(FlowData) (vlm/src/vlm.cpp:97-151) plus CDi and CM.
 * gamma_out: optional HOST double array of n entries (surfaces packed). */
int gbvlm_vlm_run(gbvlm_vlm h, double alpha, double beta, double u_inf, double rho, const double* ref_pt,
                  gbvlm_coeffs* out, double* gamma_out, gbvlm_stream stream);
/* The shared-AIC sweep on the plain per-solve path, no single reference
 * counterpart: the AIC of VLM::run at alpha = 0 (wake row along +x,
 * vlm.cpp:104-126) assembled and factored once in the handle's precision,
 * then for each of the nalpha angles the operator sequence of
 * vlm.cpp:115-151 with the free stream V(alpha) as the right-hand side.
 * out[k] and gamma_out + k*n (optional, HOST) per angle. */
int gbvlm_vlm_run_shared(gbvlm_vlm h, int32_t nalpha, const double* alphas, double u_inf, double rho,
                         const double* ref_pt, gbvlm_coeffs* out, double* gamma_out, gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Batched steady solves: many single-surface cases of uneven size, each with
 * several angles of attack, in one CUDA graph.  No reference counterpart as
 * one call: it runs, per case and angle, the operator sequence of
 * VLM::run (vlm/src/vlm.cpp:97-151) -- geometry, lhs_assemble,
 * rhs_assemble_velocities, LU factorize/solve, forces_steady, coeff_cl,
 * coeff_cm -- plus the Trefftz CDi.  Geometry is formed in double, the AIC in
 * float from double-float relative vectors, the LU in float, and
 * `refine_iters` steps of refinement with a double residual recover double
 * accuracy of the stored system; loads are summed in double.
 *   GBVLM_BATCH_EXACT : one AIC per (case, alpha) with the reference's
 *                       alpha-dependent collocation points and wake;
 *   GBVLM_BATCH_SHARED: one AIC per case built at alpha = 0, each alpha a
 *                       right-hand side V_inf(alpha) (the classical linear
 *                       VLM; fewer factorizations).
 * ------------------------------------------------------------------------- */
enum { GBVLM_BATCH_EXACT = 0, GBVLM_BATCH_SHARED = 1 };
/* Plan flags of gbvlm_batch_create_ex.
 *   GBVLM_BATCH_FP64_RESIDUAL: the refinement residual b - A x measures the
 *     FP64 system, not its float-rounded copy.  The plan also evaluates the
 *     AIC in float-pair arithmetic (about 44 bits, fp32 pipes) and keeps the
 *     difference from the stored float AIC (one more n x n float per
 *     system), so the refined circulations converge to the FP64 system's
 *     solution: gamma, not only CL/CM, within 1e-5 of the FP64 LU solve of a
 *     system whose condition number is near 1e4 (the reference's elliptic
 *     128 x 128 wing).  Needs refine_iters >= 1. */
enum { GBVLM_BATCH_FP64_RESIDUAL = 1 };
typedef struct gbvlm_batch_s* gbvlm_batch;

/* dims[c].ns/.nc: panels of case c; nalpha[c] in [1, 64] angles. */
int gbvlm_batch_create(gbvlm_batch* out, int32_t ncases, const gbvlm_dims* dims, const int32_t* nalpha,
                       int32_t mode, int32_t refine_iters);
/* gbvlm_batch_create with plan flags (GBVLM_BATCH_FP64_RESIDUAL). */
int gbvlm_batch_create_ex(gbvlm_batch* out, int32_t ncases, const gbvlm_dims* dims, const int32_t* nalpha,
                          int32_t mode, int32_t refine_iters, int32_t flags);
int gbvlm_batch_destroy(gbvlm_batch h);
/* Sizes of the plan: solves (= sum nalpha), systems, gamma floats, Biot-Savart
 * ring-point interactions and LU flops per run, device bytes held. */
int gbvlm_batch_info(gbvlm_batch h, int64_t* nsolve, int64_t* nsys, int64_t* gamma_floats, double* interactions,
                     double* lu_flops, int64_t* arena_bytes);
/* Kernel launches one gbvlm_batch_run makes (after the first run). */
int gbvlm_batch_launches(gbvlm_batch h, int64_t* out);
/* verts: every case's (ns+1, nc+1, 4) float vertices (quarter-chord shifted)
 * packed in case order, host (pageable or pinned) or device memory;
 * alphas: host, sum(nalpha) radians in case order; ref_pt: host [3] moment
 * reference in the wing frame (may be NULL = origin). */
int gbvlm_batch_set_inputs(gbvlm_batch h, const float* verts, const double* alphas, double u_inf, double rho,
                           const double* ref_pt, gbvlm_stream stream);
/* Enqueue the whole solve (a CUDA graph captured on first use) on stream. */
int gbvlm_batch_run(gbvlm_batch h, int32_t want_gamma, gbvlm_stream stream);
/* The same solve launched kernel by kernel, without capturing a graph: for a
 * batch solved once (a served request), where capture and instantiation would
 * cost more than the launches they save. */
int gbvlm_batch_run_eager(gbvlm_batch h, int32_t want_gamma, gbvlm_stream stream);
/* Run the stages once without the graph, each bracketed by CUDA events on
 * `stream`; stage_ms[6] = geometry, assembly, rhs, LU factor, solve +
 * refinement, loads (milliseconds).  Synchronous. */
int gbvlm_batch_profile(gbvlm_batch h, float* stage_ms, gbvlm_stream stream);
/* Measurement hook, no reference counterpart: run the solve once without the
 * graph (the LU's size groups one after another) with CUDA events around
 * every tensor-core trailing-update launch of the LU; out[4] = total milliseconds of those launches, their number, and
 * their algorithmic flops (2 m^2 W) and bytes (8 m^2 + 8 m W) per solve of
 * the batch (m = trailing size, W = outer block width).  Synchronous. */
int gbvlm_batch_update_profile(gbvlm_batch h, double* out, gbvlm_stream stream);
/* Synchronous read-back in case/alpha order: coeffs[5*k..] = cl, cdi, cm_x,
 * cm_y, cm_z; gamma (optional, needs want_gamma) = each solve's n floats. */
int gbvlm_batch_results(gbvlm_batch h, double* coeffs, float* gamma, gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Unsteady VLM, UVLM::run (vlm/src/vlm.cpp:358-509), with the time loop on
 * the device.  The caller evaluates each surface's kinematic transform and
 * its time derivative at t_i = i*dt, i in [0, t_steps] (the reference does
 * this with dual numbers, vlm/include/vlm_kinematics.hpp:215-239):
 *   transforms[(i*nsurf + m)*16 ..]  4x4 column-major T_m(t_i)
 *   dtransforms[...]                  dT_m/dt (t_i)
 *   freestream[i*3 ..]                -V_body(t_i) (vlm.cpp:414)
 *   ref_pt[i*3 ..]                    moment reference at t_i (may be NULL)
 * Results per step i (i >= 1, as the reference skips i = 0): CL(t_i) and
 * CM(t_i) (coeff_cl_multibody / coeff_cm_multibody, vlm.cpp:461-475).
 * rollup != 0 adds the free-wake roll-up of kernel_rollup
 * (vlm_backend_cpu_kernels.ispc:215-271) after each solve; the reference's
 * wake is purely kinematic. */
typedef struct gbvlm_uvlm_s* gbvlm_uvlm;
int gbvlm_uvlm_create(gbvlm_uvlm* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                      const int32_t* lifting, int64_t t_steps, int32_t precision);
int gbvlm_uvlm_destroy(gbvlm_uvlm h);
int gbvlm_uvlm_set_kinematics(gbvlm_uvlm h, const double* transforms, const double* dtransforms,
                              const double* freestream, const double* ref_pt);
int gbvlm_uvlm_run(gbvlm_uvlm h, double dt, int32_t rollup, double sigma, gbvlm_stream stream);
/* Step-wise use (a resident case advanced one step per call): begin places
 * the wing, assembles and factors the AIC; each step advances one time
 * step and, if cl/cm are not NULL, reads that step's coefficients back
 * (synchronous then).  At most t_steps-1 steps. */
int gbvlm_uvlm_begin(gbvlm_uvlm h, double dt, int32_t rollup, double sigma, gbvlm_stream stream);
int gbvlm_uvlm_step(gbvlm_uvlm h, int64_t* step_index, double* cl, double* cm, gbvlm_stream stream);
/* The same step (vlm.cpp:410-508) as one CUDA-graph launch: every
 * step-dependent argument (wake rows, wake column, pose at t_{i+1}) is read
 * from a device counter, so the graph captured on the first call replays for
 * every later step.  Float runs without roll-up, from the second step on
 * (take the first with gbvlm_uvlm_step); the two may be mixed.  Results equal
 * gbvlm_uvlm_step's within float rounding (the wake sums are sliced for the
 * run's last row count). */
int gbvlm_uvlm_step_graph(gbvlm_uvlm h, int64_t* step_index, double* cl, double* cm, gbvlm_stream stream);

/* Device-resident request loop over a resident case (serving; no reference
 * counterpart: it advances the case as gbvlm_uvlm_step_graph does, one step
 * per request).  One CUDA graph whose while node takes a step, writes that
 * step's coefficients into mapped host memory and waits on the GPU, for at
 * most poll_s (0 < poll_s <= 1), for the next request; without one it ends,
 * and the next submit launches it again.  submit raises a counter in mapped
 * host memory (a graph launch only when the loop had ended) and returns a
 * ticket; wait polls that ticket's completion for at most timeout_s.  Steps
 * run in ticket order.  While a loop exists the case takes no other step or
 * begin and cannot be destroyed; after gbvlm_uvlm_loop_destroy it continues
 * from the loop's last step.  Needs a float case without roll-up, its first
 * step taken, and native atomics on host memory (GB300 with Grace). */
typedef struct gbvlm_uvlm_loop_s* gbvlm_uvlm_loop;
int gbvlm_uvlm_loop_create(gbvlm_uvlm_loop* out, gbvlm_uvlm h, double poll_s);
int gbvlm_uvlm_loop_submit(gbvlm_uvlm_loop l, int64_t* ticket);
int gbvlm_uvlm_loop_wait(gbvlm_uvlm_loop l, int64_t ticket, double timeout_s, int64_t* step_index, double* cl,
                         double* cm);
/* requests submitted and completed so far, and graph launches they took */
int gbvlm_uvlm_loop_stats(gbvlm_uvlm_loop l, int64_t* submitted, int64_t* completed, int64_t* launches);
int gbvlm_uvlm_loop_destroy(gbvlm_uvlm_loop l);
/* cl: t_steps doubles, cm: 3*t_steps, gamma_last: n doubles of the last step (each may be NULL). Synchronous. */
int gbvlm_uvlm_results(gbvlm_uvlm h, double* cl, double* cm, double* gamma_last, gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Structural integrator: Newmark-beta in incremental form (class NewmarkBeta,
 * vlm/include/vlm_integrator.hpp:7-41, vlm/src/vlm_integrator.cpp:5-68), in
 * double on the device (the reference's is float).  Matrices are (ndof, ndof)
 * column-major, vectors ndof long, all DEVICE double; ndof <= 16.
 * ------------------------------------------------------------------------- */
typedef struct gbvlm_newmark_s* gbvlm_newmark;
/* NewmarkBeta(backend, beta = 0.25, gamma = 0.5) (vlm_integrator.hpp:9-15). */
int gbvlm_newmark_create(gbvlm_newmark* out, double beta, double gamma);
int gbvlm_newmark_destroy(gbvlm_newmark h);
/* NewmarkBeta::init (vlm_integrator.cpp:5-26): K_eff = K + M/(beta dt^2) +
 * gamma C/(beta dt), LU-factored on the device.  Synchronous (returns
 * GBVLM_ERR_SINGULAR for a singular K_eff). */
int gbvlm_newmark_init(gbvlm_newmark h, int32_t ndof, const double* M, const double* C, const double* K, double dt,
                       gbvlm_stream stream);
/* NewmarkBeta::step (vlm_integrator.cpp:28-68): du, dv, da of one step from
 * v_i, a_i and the load increment delta_F; coefficients from this dt, K_eff
 * from init.  Asynchronous; outputs must not alias inputs. */
int gbvlm_newmark_step(gbvlm_newmark h, const double* M, const double* C, const double* v_i, const double* a_i,
                       double* du, double* dv, double* da, const double* delta_F, double dt, gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Coupled aeroelastic 2-DOF (pitch-plunge) UVLM: class UVLM_2DOF of the
 * reference's tests/uvlm_2dof.cpp:52-808 (COUPLED branch).  Aerodynamics in
 * float as the reference; the structure (Newmark-beta, Newton loop on the load
 * increment per time step) in double on the device.  The moving surfaces
 * follow freestream(-t) . heave(-h) . pitch(alpha about x = 1 + a_h); the
 * time step is the chord of the last surface's last chordwise panel
 * (nondimensional), t_steps = t_final / dt.
 * ------------------------------------------------------------------------- */
typedef struct {
    double b, k_a, rho, a_h, omega, zeta_a, zeta_h, x_a, mu, r_a, U_a; /* UVLM_2DOF_Vars, uvlm_2dof.cpp:23-39 */
} gbvlm_2dof_vars;
typedef struct gbvlm_aero2dof_s* gbvlm_aero2dof;
/* Set-up of UVLM_2DOF::run (uvlm_2dof.cpp:437-515): verts_init HOST float
 * (ns+1, nc+1, 4) per surface in dimensional units; returns t_steps and dt.
 * Synchronous. */
int gbvlm_aero2dof_create(gbvlm_aero2dof* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                          const int32_t* lifting, const gbvlm_2dof_vars* vars, double t_final, int64_t* t_steps,
                          double* dt, gbvlm_stream stream);
int gbvlm_aero2dof_destroy(gbvlm_aero2dof h);
/* Advance `steps` time steps (uvlm_2dof.cpp:588-808), at most t_steps-2 in
 * all; each Newton loop stops when |du_prev - du| <= FLT_EPSILON or after
 * max_iter + 1 iterations (the reference uses 50).  Synchronous. */
int gbvlm_aero2dof_run(gbvlm_aero2dof h, int64_t steps, int32_t max_iter, gbvlm_stream stream);
/* HOST outputs for steps 0..steps_done: u, v, a, F ((steps_done+1) x 2 each,
 * row-major: h, alpha), iters (steps_done Newton counts); each may be NULL. */
int gbvlm_aero2dof_results(gbvlm_aero2dof h, int64_t* steps_done, double* u, double* v, double* a, double* F,
                           int32_t* iters, gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Harmonic-balance VLM (lib/libhbvlm3.cpp:262-552; 2-DOF lib/libhbvlm.cpp:230-468),
 * double.  Exactly one surface is lifting; its wake carries the
 * trailing-edge gamma rebuilt from Fourier coefficients.  The host supplies
 * the kinematics (per-step wake transforms and per-instance transforms and
 * rates, N = 2*harmonics + 1 instances) and the DFT matrix.
 * ------------------------------------------------------------------------- */
typedef struct gbvlm_hbvlm_s* gbvlm_hbvlm;
/* HBVLM(backend, meshes): verts_init HOST double (ns+1, nc+1, 4) per surface, already scaled. */
int gbvlm_hbvlm_create(gbvlm_hbvlm* out, int32_t nsurf, const gbvlm_dims* dims, const double* const* verts_init,
                       const int32_t* lifting);
int gbvlm_hbvlm_destroy(gbvlm_hbvlm h);
/* libhbvlm3.cpp:266-347: metrics at the undisplaced pose, AIC (no wake) and
 * its factors, wake pre-generation over max_t_steps steps
 * (wake_transforms[(i*nsurf+m)*16]), then per instance q (t_steps[q],
 * times[q], transforms/dtransforms[(q*nsurf+m)*16]) the geometry and -V.n
 * right-hand side; dft is the (N x N) column-major DFT matrix. */
int gbvlm_hbvlm_prepare(gbvlm_hbvlm h, int32_t harmonics, int64_t max_t_steps, const double* wake_transforms,
                        const int64_t* t_steps, const double* times, const double* transforms,
                        const double* dtransforms, const double* dft, gbvlm_stream stream);
/* One fixed-point map x_in -> x_out (HOST, n x N column-major) (libhbvlm3.cpp:349-410). */
int gbvlm_hbvlm_map(gbvlm_hbvlm h, const double* x_in, double* x_out, double omega, double dt, gbvlm_stream stream);
/* anderson_acceleration (vlm/src/vlm_solvers.cpp:6-115) of the map from x (HOST, updated in place). */
int gbvlm_hbvlm_solve(gbvlm_hbvlm h, double* x, double omega, double dt, int32_t max_iter, double tol, int32_t m,
                      int32_t* iters, gbvlm_stream stream);
/* K independent parameter sets on the same meshes (for instance the
 * columns of a finite-difference Jacobian, scripts/continuation.py:192-195
 * through scripts/finite_diff.py:26-48), solved together: the AIC factors
 * are shared, every map of every set runs in the same launches and one
 * solve, and each set runs its own Anderson iteration (stopping on its own
 * test).  Per set c: max_t_steps[c] and wake_transforms[c] (max_t_steps[c]
 * x nsurf x 16); t_steps, times, transforms, dtransforms and dft are the
 * single-set arrays concatenated over the K sets.  The single-set calls
 * above are these with K = 1. */
int gbvlm_hbvlm_prepare_batch(gbvlm_hbvlm h, int32_t K, int32_t harmonics, const int64_t* max_t_steps,
                              const double* const* wake_transforms, const int64_t* t_steps, const double* times,
                              const double* transforms, const double* dtransforms, const double* dft,
                              gbvlm_stream stream);
/* gbvlm_hbvlm_prepare_batch with the wake transforms evaluated on the device
 * from the libhbvlm kinematic chain (libhbvlm3.cpp:559-641, libhbvlm.cpp:
 * 470-515) instead of uploaded: per set, chain holds 6 + 3 (2H+1) doubles:
 * sigma (free-stream speed), omega, dt, px (pitch axis x), qx (control
 * axis x), flap (1 when the lifting surface follows the control rotation),
 * then the heave, pitch and control Fourier rows.  Not in the reference:
 * there the host evaluates every step's transform. */
int gbvlm_hbvlm_prepare_batch_chain(gbvlm_hbvlm h, int32_t K, int32_t harmonics, const int64_t* max_t_steps,
                                    const double* chain, const int64_t* t_steps, const double* times,
                                    const double* transforms, const double* dtransforms, const double* dft,
                                    gbvlm_stream stream);
/* x: HOST K x (n x N) column-major iterates, updated in place; omega, dt,
 * iters: K each. */
int gbvlm_hbvlm_solve_batch(gbvlm_hbvlm h, int32_t K, double* x, const double* omega, const double* dt,
                            int32_t max_iter, double tol, int32_t m, int32_t* iters, gbvlm_stream stream);
/* gbvlm_hbvlm_loads for K sets: every array the single-set arrays
 * concatenated over the sets (ref_b may be NULL); out: K x 3 x N. */
int gbvlm_hbvlm_loads_batch(gbvlm_hbvlm h, int32_t K, const double* coeffs, const double* dft, const double* ddft,
                            const double* transforms, const double* dtransforms, const double* freestream,
                            const double* ref_a, const double* ref_b, int32_t coupled_te, double* out,
                            gbvlm_stream stream);
/* Loads at N force instances (libhbvlm3.cpp:428-550): out (3 x N, row-major)
 * = CL, CM_y about ref_a (multibody), CM_y of surface 1 about ref_b (if
 * ref_b != NULL, else 0).  coupled_te: surface m's first chordwise gamma delta also
 * subtracts surface m-1's trailing-edge gamma (wing + flap). */
int gbvlm_hbvlm_loads(gbvlm_hbvlm h, const double* coeffs, const double* dft, const double* ddft,
                      const double* transforms, const double* dtransforms, const double* freestream,
                      const double* ref_a, const double* ref_b, int32_t coupled_te, double* out, gbvlm_stream stream);

/* plot3d reader (vlm/src/vlm_mesh.cpp:34-123): dims first (verts == NULL),
 * then the vertices into a HOST float (ns+1, nc+1, 4) array. */
int gbvlm_read_plot3d(const char* path, int32_t quarter_chord, gbvlm_dims* dims, float* verts);

/* Test hook with no counterpart in the reference: runs the batched
 * dataflow triangular solve on an identity system of n unknowns (two to four
 * 128-row blocks) with the first block withheld, so the second block's wait
 * for it must run out (after 2 s).  Returns GBVLM_ERR_CUDA with the solve's
 * timeout message when the bounded wait works; the CUDA context stays
 * usable. */
int gbvlm_test_flow_wait_timeout(int32_t n, gbvlm_stream stream);
/* Test hook with no counterpart in the reference: one tensor-core update tile
 * (128 x 128, K = 32) whose MMA-issuing thread issues and commits nothing, so
 * the tile's bounded mbarrier wait must run out (after 2 s).  No MMA is in
 * flight; the tile frees its tensor memory and sets its error word.  Returns
 * GBVLM_ERR_CUDA with the timeout message when the bounded wait works; the
 * CUDA context stays usable. */
int gbvlm_test_tc_wait_timeout(gbvlm_stream stream);

/* ---------------------------------------------------------------------------
 * Nonlinear VLM: NLVLM::run (vlm/include/vlm.hpp:87-115, vlm/src/vlm.cpp:
 * 153-295), the strip-wise correction of the angle of attack toward a 2D
 * lift polar.  The polar is (db_alpha[i], db_cl[i]), n_db >= 4 points with
 * increasing angles, interpolated as tiny::AkimaInterpolator does
 * (Database2D::interpolate_CL, vlm_data.hpp:85-90: one profile).  The
 * reference's defaults are tol = 1e-5 and max_iter = 100 (vlm.hpp:90-91).
 * Returns the final CL (strips reset to alpha, as the reference does), the
 * iterations run, the last L1 correction per panel, and optionally the strip
 * angles before the reset (sum of ns floats over the surfaces, host memory).
 * Synchronous.
 * ------------------------------------------------------------------------- */
typedef struct gbvlm_nlvlm_s* gbvlm_nlvlm;
int gbvlm_nlvlm_create(gbvlm_nlvlm* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                       int32_t precision);
int gbvlm_nlvlm_destroy(gbvlm_nlvlm h);
int gbvlm_nlvlm_run(gbvlm_nlvlm h, double alpha, double beta, double u_inf, double rho, const float* db_alpha,
                    const float* db_cl, int32_t n_db, double tol, int32_t max_iter, double* cl, int32_t* iters,
                    double* err, float* strip_alpha, gbvlm_stream stream);

#ifdef __cplusplus
}
#endif
#endif /* GBVLM_H */
