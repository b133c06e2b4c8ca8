// Structural integrator: Newmark-beta in incremental form, double precision
// on the device (vlm/include/vlm_integrator.hpp:7-41,
// vlm/src/vlm_integrator.cpp:5-68; the reference keeps it in float).
//
// init:  K_eff = K + M / (beta dt^2) + gamma C / (beta dt), LU-factored with
//        partial pivoting once (vlm_integrator.cpp:5-26)
// step:  F_eff = dF + M (v/(beta dt) + a/(2 beta))
//                   + C (gamma/beta v - dt (1 - gamma/(2 beta)) a)
//        du = K_eff^-1 F_eff
//        dv = gamma/(beta dt) du - gamma/beta v + dt (1 - gamma/(2 beta)) a
//        da = du/(beta dt^2) - v/(beta dt) - a/(2 beta)          (:28-68)
// The coefficients of a step use the step's dt and K_eff the factorisation
// made at init, as in the reference.  Systems are small (the aeroelastic
// drivers have 2 or 3 degrees of freedom): one thread does a step, so a step
// is one launch that reads its inputs and writes its outputs on the device.
#include <cuda_runtime.h>
#include <math.h>

#include "gbvlm_internal.h"

namespace gbvlm {

constexpr int NM_MAX_DOF = 16;

struct NewmarkDev {
    double lu[NM_MAX_DOF * NM_MAX_DOF];  // factored K_eff, column-major
    int piv[NM_MAX_DOF];
    int info;  // 0, or the first column with an exactly zero pivot (1-based)
};

// K_eff = K + x0 M + x1 C, then LU with partial pivoting (one thread)
__global__ void k_newmark_init(int nd, const double* M, const double* C, const double* K, double x0, double x1,
                               NewmarkDev* dev) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double* a = dev->lu;
    for (int c = 0; c < nd; c++)
        for (int r = 0; r < nd; r++) a[r + c * nd] = K[r + c * nd] + x0 * M[r + c * nd] + x1 * C[r + c * nd];
    dev->info = 0;
    for (int k = 0; k < nd; k++) {
        int p = k;
        double best = fabs(a[k + k * nd]);
        for (int r = k + 1; r < nd; r++)
            if (fabs(a[r + k * nd]) > best) {
                best = fabs(a[r + k * nd]);
                p = r;
            }
        dev->piv[k] = p;
        if (p != k)
            for (int c = 0; c < nd; c++) {
                const double t = a[k + c * nd];
                a[k + c * nd] = a[p + c * nd];
                a[p + c * nd] = t;
            }
        const double d = a[k + k * nd];
        if (d == 0.0) {
            if (dev->info == 0) dev->info = k + 1;
            continue;
        }
        for (int r = k + 1; r < nd; r++) a[r + k * nd] /= d;
        for (int c = k + 1; c < nd; c++)
            for (int r = k + 1; r < nd; r++) a[r + c * nd] -= a[r + k * nd] * a[k + c * nd];
    }
}

struct NewmarkCoef {
    double x0, x1, xd0, xd1, xdd0, xdd1;
};

__host__ __device__ inline NewmarkCoef newmark_coef(double beta, double gamma, double dt) {
    NewmarkCoef c;
    c.x1 = gamma / (beta * dt);
    c.x0 = 1.0 / (beta * dt * dt);
    c.xd0 = 1.0 / (beta * dt);
    c.xd1 = gamma / beta;
    c.xdd0 = 1.0 / (2.0 * beta);
    c.xdd1 = -dt * (1.0 - gamma / (2.0 * beta));
    return c;
}

// one incremental step (one thread); outputs may not alias the inputs
__device__ inline void newmark_step_dev(int nd, const NewmarkDev* dev, NewmarkCoef k, const double* M, const double* C,
                                        const double* v, const double* a, const double* dF, double* du, double* dv,
                                        double* da) {
    double f[NM_MAX_DOF], fm[NM_MAX_DOF], fc[NM_MAX_DOF];
    for (int r = 0; r < nd; r++) {
        fm[r] = k.xd0 * v[r] + k.xdd0 * a[r];
        fc[r] = k.xd1 * v[r] + k.xdd1 * a[r];
    }
    for (int r = 0; r < nd; r++) {
        double s = dF[r];
        for (int c = 0; c < nd; c++) s += M[r + c * nd] * fm[c];
        for (int c = 0; c < nd; c++) s += C[r + c * nd] * fc[c];
        f[r] = s;
    }
    const double* lu = dev->lu;
    for (int r = 0; r < nd; r++) {  // row interchanges, then L (unit) and U
        const int p = dev->piv[r];
        const double t = f[r];
        f[r] = f[p];
        f[p] = t;
    }
    for (int r = 0; r < nd; r++)
        for (int c = 0; c < r; c++) f[r] -= lu[r + c * nd] * f[c];
    for (int r = nd - 1; r >= 0; r--) {
        for (int c = r + 1; c < nd; c++) f[r] -= lu[r + c * nd] * f[c];
        f[r] /= lu[r + r * nd];
    }
    for (int r = 0; r < nd; r++) {
        du[r] = f[r];
        dv[r] = k.x1 * f[r] - k.xd1 * v[r] - k.xdd1 * a[r];
        da[r] = k.x0 * f[r] - k.xd0 * v[r] - k.xdd0 * a[r];
    }
}

__global__ void k_newmark_step(int nd, const NewmarkDev* dev, NewmarkCoef k, const double* M, const double* C,
                               const double* v, const double* a, const double* dF, double* du, double* dv, double* da) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    newmark_step_dev(nd, dev, k, M, C, v, a, dF, du, dv, da);
}

// the step with the state of step *i_dev (graph replay)
__global__ void k_newmark_step_dev(int nd, const NewmarkDev* dev, NewmarkCoef k, const double* M, const double* C,
                                   const double* v, const double* a, const int64_t* i_dev, const double* dF,
                                   double* du, double* dv, double* da) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int64_t i = *i_dev;
    newmark_step_dev(nd, dev, k, M, C, v + nd * i, a + nd * i, dF, du, dv, da);
}

}  // namespace gbvlm

using namespace gbvlm;

struct gbvlm_newmark_s {
    double beta = 0.25, gamma = 0.5;
    int32_t nd = 0;
    NewmarkDev* dev = nullptr;
    ~gbvlm_newmark_s() {
        if (dev) cudaFree(dev);
    }
};

extern "C" {

int gbvlm_newmark_create(gbvlm_newmark* out, double beta, double gamma) {
    GB_REQUIRE(out, "null argument");
    GB_REQUIRE(beta > 0 && gamma > 0, "Newmark: beta and gamma must be positive");
    auto* h = new gbvlm_newmark_s();
    h->beta = beta;
    h->gamma = gamma;
    cudaError_t e = cudaMalloc(&h->dev, sizeof(NewmarkDev));
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    }
    *out = h;
    return GBVLM_OK;
}

int gbvlm_newmark_destroy(gbvlm_newmark h) {
    delete h;
    return GBVLM_OK;
}

int gbvlm_newmark_init(gbvlm_newmark h, int32_t ndof, const double* M, const double* C, const double* K, double dt,
                       gbvlm_stream stream) {
    GB_REQUIRE(h && M && C && K, "null argument");
    GB_REQUIRE(ndof >= 1 && ndof <= NM_MAX_DOF, "Newmark: %d degrees of freedom outside [1, %d]", ndof, NM_MAX_DOF);
    GB_REQUIRE(dt > 0, "Newmark: dt must be positive");
    cudaStream_t st = to_cuda(stream);
    const NewmarkCoef k = newmark_coef(h->beta, h->gamma, dt);
    h->nd = ndof;
    k_newmark_init<<<1, 32, 0, st>>>(ndof, M, C, K, k.x0, k.x1, h->dev);
    GB_LAUNCH_CHECK();
    int info = 0;
    GB_CUDA(cudaMemcpyAsync(&info, &h->dev->info, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (info) {
        set_error("Newmark: effective stiffness singular at column %d", info);
        return GBVLM_ERR_SINGULAR;
    }
    return GBVLM_OK;
}

int gbvlm_newmark_step(gbvlm_newmark h, const double* M, const double* C, const double* v_i, const double* a_i,
                       double* du, double* dv, double* da, const double* delta_F, double dt, gbvlm_stream stream) {
    GB_REQUIRE(h && M && C && v_i && a_i && du && dv && da && delta_F, "null argument");
    GB_REQUIRE(h->nd > 0, "Newmark: step before init");
    GB_REQUIRE(dt > 0, "Newmark: dt must be positive");
    const NewmarkCoef k = newmark_coef(h->beta, h->gamma, dt);
    k_newmark_step<<<1, 32, 0, to_cuda(stream)>>>(h->nd, h->dev, k, M, C, v_i, a_i, delta_F, du, dv, da);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

}  // extern "C"

namespace gbvlm {

int newmark_step_dev(gbvlm_newmark h, const double* M, const double* C, const double* v, const double* a,
                     const int64_t* i_dev, double* du, double* dv, double* da, const double* delta_F, double dt,
                     cudaStream_t st) {
    GB_REQUIRE(h && M && C && v && a && i_dev && du && dv && da && delta_F, "null argument");
    GB_REQUIRE(h->nd > 0, "Newmark: step before init");
    GB_REQUIRE(dt > 0, "Newmark: dt must be positive");
    const NewmarkCoef k = newmark_coef(h->beta, h->gamma, dt);
    k_newmark_step_dev<<<1, 32, 0, st>>>(h->nd, h->dev, k, M, C, v, a, i_dev, delta_F, du, dv, da);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

}  // namespace gbvlm
