/*
 * Oracle (test infrastructure only, never linked by the product): CPU
 * restatement of the tinyvlm vortex-lattice hot path, built as
 * oracle/_build/libvlm_oracle.so by oracle/build.py and loaded through
 * oracle/oracle.py by the tests, the smoke check and the CPU-baseline leg of
 * bench.py.
 *
 * Precision variants mirror the reference's two backends:
 *   *_f : vlm/backends/cpu/src/vlm_backend_cpu.cpp + ispc float kernels
 *   *_d : vlm/backends/cpu/src/vlm_backend_cpud.cpp + ispc double kernels
 * OpenMP stands in for the reference's Taskflow parallel-for loops
 * (vlm/include/vlm_executor.hpp); it changes no per-element arithmetic.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define ORC_PI_F 3.141593f           /* vlm_backend_cpu_kernels.ispc:12 */
#define ORC_EPS_F 1.19209e-07f       /* vlm/include/vlm_types.hpp:24 */

/* ---- float ---- */
#define T float
#define SFX f
#define SQRT sqrtf
#define SIN sinf
#define COS cosf
#define ORC_RCUT 1e-10f              /* ispc:9 */
#define ORC_RCUT_NORM 1e-5f          /* ispc:10, float kernel cuts |r1|,|r2| at RCUT2 */
#define ORC_FOURPI (4.0f * ORC_PI_F)
#define ORC_WAKE_WINDOW 5000         /* ispc:158-162 */
#include "vlm_oracle_impl.h"
#undef T
#undef SFX
#undef SQRT
#undef SIN
#undef COS
#undef ORC_RCUT
#undef ORC_RCUT_NORM
#undef ORC_FOURPI
#undef ORC_WAKE_WINDOW
#undef V3

/* ---- double ---- */
static const float orc_fourpi_float = 4.0f * ORC_PI_F; /* ispc:400 keeps the float product */
#define T double
#define SFX d
#define SQRT sqrt
#define SIN sin
#define COS cos
#define ORC_RCUT 1e-10               /* ispc:393 */
#define ORC_RCUT_NORM 1e-10
#define ORC_FOURPI ((double)orc_fourpi_float)
#define ORC_WAKE_WINDOW 0            /* ispc:471: no window in double */
#include "vlm_oracle_impl.h"

/* Number of OpenMP threads the oracle uses (for reporting). */
int orc_num_threads(void) {
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
