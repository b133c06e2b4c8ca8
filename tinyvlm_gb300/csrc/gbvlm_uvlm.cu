// Unsteady VLM driver (vlm/src/vlm.cpp:297-509) with the whole time loop on
// the device.  The caller evaluates each surface's kinematic transform and
// its time derivative at t_i = i dt (the reference does this on the host
// with forward-mode dual numbers, vlm/include/vlm_kinematics.hpp:215-239)
// and uploads all steps at once; the loop then runs without host
// round-trips: CL(t) and CM(t) land in device arrays read at the end.
//
// Per step i (t = i dt), as UVLM::run:
//   wake_shed(i); V_p = -dT(t)/dt [c0_p, 1] at the t = 0 collocation points;
//   rhs = -V.n - wake influence (i rows); LU solve (AIC factored once at
//   t = 0 without wake); gamma, gamma_delta, dgamma/dt, TE gamma shed to the
//   wake; for i > 0 unsteady forces, CL and CM about ref(t); optional free-
//   wake roll-up (the reference's kernel_rollup, whose caller it disables);
//   move to t + dt and recompute the panel metrics.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "gbvlm_internal.h"
#include "gbvlm_math.cuh"

namespace gbvlm {

template <class T>
__global__ void k_dual_velocity(const T* Td, const T* c0, T* vel, int64_t np) {
    const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const T x = c0[p], y = c0[np + p], z = c0[2 * np + p];
    // -(dT/dt) [x y z 1], column-major 4x4
    for (int r = 0; r < 3; r++) vel[r * np + p] = -(Td[r] * x + Td[r + 4] * y + Td[r + 8] * z + Td[r + 12]);
}

// Multibody CL and CM of one step (vlm/src/vlm_backend.cpp:72-139) in
// double, written to out[0] (cl) and out[1..3] (cm).  One block.
template <class T>
struct CoefArgs {
    int32_t n;
    int64_t ns[GBVLM_MAX_SURFACES], nc[GBVLM_MAX_SURFACES];
    const T* forces[GBVLM_MAX_SURFACES];
    const T* verts[GBVLM_MAX_SURFACES];
    const T* areas[GBVLM_MAX_SURFACES];
};

__device__ double blk_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];
    return r;
}

template <class T>
__global__ void __launch_bounds__(512) k_step_coeffs(CoefArgs<T> a, const T* fs_all, const T* ref_all, int64_t step,
                                                    double rho, double* out) {
    __shared__ double sh[32];
    const T* fsp = fs_all + 3 * step;
    const T* rp = ref_all + 3 * step;
    const double fx = fsp[0], fy = fsp[1], fz = fsp[2];
    double lx = -fz, lz = fx;
    const double ll = sqrt(lx * lx + lz * lz);
    lx /= ll;
    lz /= ll;
    const double v2 = fx * fx + fy * fy + fz * fz;
    double cl = 0, ta = 0, tm = 0, cm[3] = {0, 0, 0};
    for (int m = 0; m < a.n; m++) {
        const int64_t ns = a.ns[m], nc = a.nc[m], np = ns * nc, vld = (ns + 1) * (nc + 1);
        const T* F = a.forces[m];
        const T* v = a.verts[m];
        CSum sl, sa, sx, sy, sz, smac;
        for (int64_t p = threadIdx.x; p < np; p += blockDim.x) {
            const int64_t i = p % ns, j = p / ns, ia = i + j * (ns + 1), ib = ia + 1;
            const double Fx = F[p], Fy = F[np + p], Fz = F[2 * np + p];
            sl.add(Fx * lx + Fz * lz);
            sa.add((double)a.areas[m][p]);
            const double ex = 0.5 * ((double)v[ia] + v[ib]) - rp[0];
            const double ey = 0.5 * ((double)v[vld + ia] + v[vld + ib]) - rp[1];
            const double ez = 0.5 * ((double)v[2 * vld + ia] + v[2 * vld + ib]) - rp[2];
            sx.add(ey * Fz - ez * Fy);
            sy.add(ez * Fx - ex * Fz);
            sz.add(ex * Fy - ey * Fx);
        }
        const int64_t last = nc * (ns + 1);
        for (int64_t i = threadIdx.x; i < ns; i += blockDim.x) {
            auto chord = [&](int64_t q) {
                const double dx = (double)v[q] - v[last + q], dy = (double)v[vld + q] - v[vld + last + q];
                const double dz = (double)v[2 * vld + q] - v[2 * vld + last + q];
                return sqrt(dx * dx + dy * dy + dz * dz);
            };
            const double c0 = chord(i), c1 = chord(i + 1);
            const double dx = (double)v[i + 1] - v[i], dy = (double)v[vld + i + 1] - v[vld + i];
            const double dz = (double)v[2 * vld + i + 1] - v[2 * vld + i];
            smac.add(0.5 * (c0 * c0 + c1 * c1) * sqrt(dx * dx + dy * dy + dz * dz));
        }
        const double L = blk_sum(sl.value(), sh), S = blk_sum(sa.value(), sh);
        const double Mx = blk_sum(sx.value(), sh), My = blk_sum(sy.value(), sh), Mz = blk_sum(sz.value(), sh);
        const double mac = blk_sum(smac.value(), sh) / S;
        const double q = 0.5 * rho * v2;
        cl += L / (q * S) * S;
        cm[0] += Mx / (q * S * mac) * S * mac;
        cm[1] += My / (q * S * mac) * S * mac;
        cm[2] += Mz / (q * S * mac) * S * mac;
        ta += S;
        tm += mac;
    }
    if (threadIdx.x == 0) {
        out[0] = cl / ta;
        for (int k = 0; k < 3; k++) out[1 + k] = cm[k] / (ta * tm);
    }
}

template <class T>
struct Ops2;
#define OPS2(T, sfx)                                                                                                \
    template <>                                                                                                     \
    struct Ops2<T> {                                                                                                \
        static int metrics(int32_t ns, const gbvlm_dims* d, const T* const* v, T* const* c, T* const* n,            \
                           T* const* ar, gbvlm_stream s) {                                                          \
            return gbvlm_mesh_metrics_##sfx((T)0, ns, d, v, c, n, ar, s);                                          \
        }                                                                                                           \
        static int lhs(T* a, int64_t ld, int32_t ns, const gbvlm_dims* d, const T* const* c, const T* const* n,     \
                       const T* const* vw, T sg, gbvlm_stream s) {                                                   \
            return gbvlm_lhs_assemble_##sfx(a, ld, ns, d, c, n, vw, nullptr, 0, sg, s);                             \
        }                                                                                                           \
        static int displace(int32_t ns, const gbvlm_dims* d, const T* const* t, T* const* v, const T* const* vi,    \
                            gbvlm_stream s) {                                                                       \
            return gbvlm_displace_wing_##sfx(ns, d, t, v, vi, s);                                                  \
        }                                                                                                           \
        static int shed(int32_t ns, const gbvlm_dims* d, const T* const* v, T* const* k, int32_t it,                \
                        gbvlm_stream s) {                                                                           \
            return gbvlm_wake_shed_##sfx(ns, d, v, k, it, s);                                                      \
        }                                                                                                           \
        static int rhsv(T* r, int32_t ns, const gbvlm_dims* d, const T* const* n, const T* const* v,                \
                        gbvlm_stream s) {                                                                           \
            return gbvlm_rhs_assemble_velocities_##sfx(r, ns, d, n, v, s);                                         \
        }                                                                                                           \
        static int wake(T* r, int32_t ns, const gbvlm_dims* d, const T* const* g, const T* const* c,                \
                        const T* const* n, const T* const* k, const int32_t* lf, int32_t it, T sg, gbvlm_stream s) { \
            return gbvlm_rhs_assemble_wake_influence_##sfx(r, ns, d, g, c, n, k, lf, it, sg, s);                   \
        }                                                                                                           \
        static int rollup(int32_t ns, const gbvlm_dims* d, T* const* k, const T* const* v, const T* const* g,       \
                          const T* const* gw, const int32_t* lf, T sg, T dt, int32_t it, gbvlm_stream s) {           \
            return gbvlm_wake_rollup_##sfx(ns, d, k, v, g, gw, lf, sg, dt, it, s);                                 \
        }                                                                                                           \
        static int factor(gbvlm_lu h, T* a, int64_t n, gbvlm_stream s) { return gbvlm_lu_factor_##sfx(h, a, n, n, s); } \
        static int solve(gbvlm_lu h, const T* a, int64_t n, T* x, gbvlm_stream s) {                                 \
            return gbvlm_lu_solve_##sfx(h, a, n, n, x, n, 1, s);                                                    \
        }                                                                                                           \
        static int gupd(int64_t ns, int64_t nc, const T* x, T* g, T* gd, T* gw, int64_t col, const T* gp, T* dg,    \
                        T dt, gbvlm_stream s) {                                                                     \
            return gbvlm_gamma_update_##sfx(ns, nc, x, g, gd, gw, col, gp, dg, dt, s);                              \
        }                                                                                                           \
        static int forces(int64_t ns, int64_t nc, const T* v, const T* gd, const T* dg, const T* vel, const T* ar,  \
                          const T* nr, T* f, gbvlm_stream s) {                                                      \
            return gbvlm_forces_unsteady_##sfx(ns, nc, v, gd, dg, vel, ar, nr, f, s);                              \
        }                                                                                                           \
    };
OPS2(float, f32)
OPS2(double, f64)

// Device-indexed UVLM step (float, no roll-up): the step index i lives in
// idx[0] on the device.  The pose kernel stages T(i+1) and Td(i) of every
// surface and the step's free stream and moment point into fixed buffers,
// so one captured graph advances the case any number of times.
template <class T>
__global__ void k_uvlm_dev_pose(const int64_t* idx, const T* Tm, const T* Tdm, const T* fs, const T* ref, int nsurf,
                                T* pose) {
    const int64_t i = idx[0];
    for (int q = threadIdx.x; q < 16 * nsurf; q += blockDim.x) {
        pose[q] = Tm[16 * (i + 1) * nsurf + q];
        pose[16 * nsurf + q] = Tdm[16 * i * nsurf + q];
    }
    if (threadIdx.x < 3) {
        pose[32 * nsurf + threadIdx.x] = fs[3 * i + threadIdx.x];
        pose[32 * nsurf + 3 + threadIdx.x] = ref[3 * i + threadIdx.x];
    }
}

// the step's coefficients into the run's record, then i -> i + 1
__global__ void k_uvlm_dev_end(int64_t* idx, const double* coef, double* res) {
    const int64_t i = idx[0];
    if (threadIdx.x < 4) res[4 * i + threadIdx.x] = coef[threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) idx[0] = i + 1;
}

struct UvlmBase {
    virtual ~UvlmBase() = default;
    virtual int set_kinematics(const double* T, const double* Td, const double* fs, const double* ref) = 0;
    virtual int run(double dt, int32_t rollup, double sigma, cudaStream_t st) = 0;
    virtual int begin(double dt, int32_t rollup, double sigma, cudaStream_t st) = 0;
    virtual int step(cudaStream_t st) = 0;
    virtual int step_graph(cudaStream_t st) = 0;
    virtual int step_result(int64_t i, double* cl, double* cm, cudaStream_t st) = 0;
    virtual int64_t last_step() const = 0;
    virtual int results(double* cl, double* cm, double* gamma_last, cudaStream_t st) = 0;
    int64_t t_steps = 0, n = 0;
    bool looping = false;  // a request loop (gbvlm_uvlm_loop_*) owns the steps
};

template <class T>
struct UvlmState : UvlmBase {
    int32_t nsurf = 0;
    std::vector<gbvlm_dims> dims;
    std::vector<int32_t> lifting;
    void* mem = nullptr;
    std::vector<T*> vinit, vpos, verts, wake, colloc, colloc0, normals, areas, gamma, gprev, gdelta, gdt, gwake, vel,
        forces;
    T *lhs = nullptr, *rhs = nullptr, *Tm = nullptr, *Tdm = nullptr, *fs = nullptr, *ref = nullptr;
    double* res = nullptr;  // [t_steps][4]
    gbvlm_lu lu = nullptr;

    // device-indexed step (step_graph): counter, staged pose, wake scratch,
    // coefficients, the staged LU solve and the captured graph
    int64_t* d_idx = nullptr;
    T* d_pose = nullptr;
    float* wsc = nullptr;
    double* d_coef = nullptr;
    void* dmem = nullptr;
    void* lut = nullptr;
    int64_t dev_idx = -1;  // the value idx[0] holds on the device (-1: unknown)
    cudaStream_t scap = nullptr;
    cudaGraph_t sgraph = nullptr;
    cudaGraphExec_t sexec = nullptr;

    ~UvlmState() override {
        if (sexec) cudaGraphExecDestroy(sexec);
        if (sgraph) cudaGraphDestroy(sgraph);
        if (scap) cudaStreamDestroy(scap);
        if (lut) lu_solve_tables_free(lut);
        if (dmem) cudaFree(dmem);
        if (lu) gbvlm_lu_destroy(lu);
        if (mem) cudaFree(mem);
    }

    int init(int32_t ns_, const gbvlm_dims* d, const float* const* vh, const int32_t* lift, int64_t steps) {
        nsurf = ns_;
        t_steps = steps;
        dims.assign(d, d + ns_);
        lifting.assign(lift, lift + ns_);
        size_t bytes = 0;
        n = 0;
        auto al = [](size_t b) { return (b + 255) / 256 * 256; };
        for (auto& x : dims) {
            x.nwv = t_steps;  // wake (ns+1, t_steps, 4) (vlm.cpp:388-399)
            const int64_t np = x.ns * x.nc, nv = (x.ns + 1) * (x.nc + 1);
            n += np;
            bytes += al(sizeof(T) * 4 * nv) * 3 + al(sizeof(T) * 4 * (x.ns + 1) * t_steps) + al(sizeof(T) * 3 * np) * 5 +
                     al(sizeof(T) * np) * 5 + al(sizeof(T) * x.ns * (t_steps - 1));
        }
        bytes += al(sizeof(T) * n * n) + al(sizeof(T) * n) + 2 * al(sizeof(T) * 16 * nsurf * (t_steps + 1)) +
                 2 * al(sizeof(T) * 3 * (t_steps + 1)) + al(sizeof(double) * 4 * t_steps);
        GB_CUDA(cudaMalloc(&mem, bytes));
        GB_CUDA(cudaMemset(mem, 0, bytes));
        char* p = (char*)mem;
        auto take = [&](size_t cnt) {
            T* r = (T*)p;
            p += al(sizeof(T) * cnt);
            return r;
        };
        lhs = take(n * n);
        rhs = take(n);
        Tm = take(16 * nsurf * (t_steps + 1));
        Tdm = take(16 * nsurf * (t_steps + 1));
        fs = take(3 * (t_steps + 1));
        ref = take(3 * (t_steps + 1));
        res = (double*)p;
        p += al(sizeof(double) * 4 * t_steps);
        for (auto& x : dims) {
            const int64_t np = x.ns * x.nc, nv = (x.ns + 1) * (x.nc + 1);
            vinit.push_back(take(4 * nv));
            vpos.push_back(take(4 * nv));
            verts.push_back(take(4 * nv));
            wake.push_back(take(4 * (x.ns + 1) * t_steps));
            colloc.push_back(take(3 * np));
            colloc0.push_back(take(3 * np));
            normals.push_back(take(3 * np));
            vel.push_back(take(3 * np));
            forces.push_back(take(3 * np));
            areas.push_back(take(np));
            gamma.push_back(take(np));
            gprev.push_back(take(np));
            gdelta.push_back(take(np));
            gdt.push_back(take(np));
            gwake.push_back(take(x.ns * (t_steps - 1)));
        }
        for (int m = 0; m < nsurf; m++) {
            const int64_t nv = (dims[m].ns + 1) * (dims[m].nc + 1);
            std::vector<T> h(4 * nv);
            for (int64_t q = 0; q < 4 * nv; q++) h[q] = (T)vh[m][q];
            GB_CUDA(cudaMemcpy(vinit[m], h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
            std::vector<T> ones((dims[m].ns + 1) * t_steps, (T)1);  // wake w plane
            GB_CUDA(cudaMemcpy(wake[m] + 3 * (dims[m].ns + 1) * t_steps, ones.data(), sizeof(T) * ones.size(),
                               cudaMemcpyHostToDevice));
        }
        int rc = gbvlm_lu_create(&lu);
        if (rc) return rc;
        return gbvlm_lu_init(lu, n);
    }

    int set_kinematics(const double* Th, const double* Tdh, const double* fsh, const double* refh) override {
        const size_t nt = (size_t)16 * nsurf * (t_steps + 1);
        std::vector<T> a(nt), b(nt), c(3 * (t_steps + 1)), d(3 * (t_steps + 1));
        for (size_t i = 0; i < nt; i++) {
            a[i] = (T)Th[i];
            b[i] = (T)Tdh[i];
        }
        for (size_t i = 0; i < c.size(); i++) {
            c[i] = (T)fsh[i];
            d[i] = refh ? (T)refh[i] : (T)0;
        }
        GB_CUDA(cudaMemcpy(Tm, a.data(), sizeof(T) * nt, cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(Tdm, b.data(), sizeof(T) * nt, cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(fs, c.data(), sizeof(T) * c.size(), cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(ref, d.data(), sizeof(T) * d.size(), cudaMemcpyHostToDevice));
        return GBVLM_OK;
    }

    std::vector<const T*> tr_at(const T* base, int64_t i) {
        std::vector<const T*> out;
        for (int m = 0; m < nsurf; m++) out.push_back(base + 16 * ((size_t)i * nsurf + m));
        return out;
    }

    CoefArgs<T> ca;
    T dt_ = 0, sigma_ = 0;
    int32_t roll_ = 0;
    int64_t next_step = 0;

    static std::vector<const T*> C(const std::vector<T*>& v) { return std::vector<const T*>(v.begin(), v.end()); }

    int run(double dt_d, int32_t roll, double sigma_d, cudaStream_t st) override {
        int rc = begin(dt_d, roll, sigma_d, st);
        if (rc) return rc;
        for (int64_t i = 0; i + 1 < t_steps; i++)
            if ((rc = step(st))) return rc;
        return GBVLM_OK;
    }

    int begin(double dt_d, int32_t roll, double sigma_d, cudaStream_t st) override {
        gbvlm_stream s = (gbvlm_stream)st;
        const T dt = (T)dt_d, sigma = (T)sigma_d;
        dt_ = dt;
        sigma_ = sigma;
        roll_ = roll;
        next_step = 0;
        GB_REQUIRE(!looping, "UVLM: a request loop advances this case (destroy it first)");
        int rc;
        // a new run refactors the AIC: the staged solve and the step graph are rebuilt on first use
        if (sexec) cudaGraphExecDestroy(sexec);
        if (sgraph) cudaGraphDestroy(sgraph);
        sexec = nullptr;
        sgraph = nullptr;
        if (lut) lu_solve_tables_free(lut);
        lut = nullptr;
        dev_idx = -1;
        // t = 0 placement (vlm.cpp:368-376): verts_pos = T(0) verts_init; metrics; colloc at t = 0 kept
        auto t0 = tr_at(Tm, 0);
        if ((rc = Ops2<T>::displace(nsurf, dims.data(), t0.data(), vpos.data(), C(vinit).data(), s))) return rc;
        for (int m = 0; m < nsurf; m++) {
            const int64_t nv = (dims[m].ns + 1) * (dims[m].nc + 1);
            GB_CUDA(cudaMemcpyAsync(verts[m], vpos[m], sizeof(T) * 4 * nv, cudaMemcpyDeviceToDevice, st));
        }
        if ((rc = Ops2<T>::metrics(nsurf, dims.data(), C(verts).data(), colloc.data(), normals.data(), areas.data(), s)))
            return rc;
        for (int m = 0; m < nsurf; m++) {
            const int64_t np = dims[m].ns * dims[m].nc;
            GB_CUDA(cudaMemcpyAsync(colloc0[m], colloc[m], sizeof(T) * 3 * np, cudaMemcpyDeviceToDevice, st));
        }
        // AIC without wake, factored once (vlm.cpp:401-403)
        GB_CUDA(cudaMemsetAsync(lhs, 0, sizeof(T) * n * n, st));
        if ((rc = Ops2<T>::lhs(lhs, n, nsurf, dims.data(), C(colloc).data(), C(normals).data(), C(verts).data(), sigma, s)))
            return rc;
        if ((rc = Ops2<T>::factor(lu, lhs, n, s))) return rc;
        memset(&ca, 0, sizeof(ca));
        ca.n = nsurf;
        for (int m = 0; m < nsurf; m++) {
            ca.ns[m] = dims[m].ns;
            ca.nc[m] = dims[m].nc;
            ca.forces[m] = forces[m];
            ca.verts[m] = verts[m];
            ca.areas[m] = areas[m];
        }
        GB_CUDA(cudaMemsetAsync(res, 0, sizeof(double) * 4 * t_steps, st));
        return GBVLM_OK;
    }

    // one time step (vlm.cpp:410-508); steps run in order 0, 1, ..., t_steps-2
    int step(cudaStream_t st) override {
        gbvlm_stream s = (gbvlm_stream)st;
        GB_REQUIRE(!looping, "UVLM: a request loop advances this case (destroy it first)");
        GB_REQUIRE(next_step + 1 < t_steps, "UVLM: all %lld steps done (wake capacity)", (long long)t_steps);
        const int64_t i = next_step++;
        const T dt = dt_, sigma = sigma_;
        const int32_t roll = roll_;
        int rc;
        {
            if ((rc = Ops2<T>::shed(nsurf, dims.data(), C(verts).data(), wake.data(), (int32_t)i, s))) return rc;
            for (int m = 0; m < nsurf; m++) {
                const int64_t np = dims[m].ns * dims[m].nc;
                k_dual_velocity<T><<<(unsigned)cdiv(np, 256), 256, 0, st>>>(Tdm + 16 * ((size_t)i * nsurf + m),
                                                                           colloc0[m], vel[m], np);
                GB_LAUNCH_CHECK();
            }
            GB_CUDA(cudaMemsetAsync(rhs, 0, sizeof(T) * n, st));
            if ((rc = Ops2<T>::rhsv(rhs, nsurf, dims.data(), C(normals).data(), C(vel).data(), s))) return rc;
            if ((rc = Ops2<T>::wake(rhs, nsurf, dims.data(), C(gwake).data(), C(colloc).data(), C(normals).data(),
                                    C(wake).data(), lifting.data(), (int32_t)i, sigma, s)))
                return rc;
            if ((rc = Ops2<T>::solve(lu, lhs, n, rhs, s))) return rc;
            int64_t off = 0;
            for (int m = 0; m < nsurf; m++) {
                const int64_t ns = dims[m].ns, nc = dims[m].nc;
                if ((rc = Ops2<T>::gupd(ns, nc, rhs + off, gamma[m], gdelta[m], gwake[m], t_steps - 2 - i, gprev[m],
                                        gdt[m], dt, s)))
                    return rc;
                off += ns * nc;
            }
            if (i > 0) {
                for (int m = 0; m < nsurf; m++) {
                    if ((rc = Ops2<T>::forces(dims[m].ns, dims[m].nc, verts[m], gdelta[m], gdt[m], vel[m], areas[m],
                                              normals[m], forces[m], s)))
                        return rc;
                }
                k_step_coeffs<T><<<1, 512, 0, st>>>(ca, fs, ref, i, 1.0, res + 4 * i);
                GB_LAUNCH_CHECK();
            }
            if (roll && i > 0) {
                if ((rc = Ops2<T>::rollup(nsurf, dims.data(), wake.data(), C(verts).data(), C(gamma).data(),
                                          C(gwake).data(), lifting.data(), sigma, dt, (int32_t)i, s)))
                    return rc;
            }
            for (int m = 0; m < nsurf; m++) {
                const int64_t np = dims[m].ns * dims[m].nc;
                GB_CUDA(cudaMemcpyAsync(gprev[m], gamma[m], sizeof(T) * np, cudaMemcpyDeviceToDevice, st));
            }
            auto tn = tr_at(Tm, i + 1);
            if ((rc = Ops2<T>::displace(nsurf, dims.data(), tn.data(), verts.data(), C(vpos).data(), s))) return rc;
            if ((rc = Ops2<T>::metrics(nsurf, dims.data(), C(verts).data(), colloc.data(), normals.data(), areas.data(),
                                       s)))
                return rc;
        }
        return GBVLM_OK;
    }

    // The step of step() with every step-dependent argument read from the
    // device (float, no roll-up, from step 1 on): captured into one graph on
    // first use and replayed, one launch per step.  Results equal step()'s
    // within float rounding (the wake sums are sliced for the run's last row
    // count, not the step's).
    int step_graph(cudaStream_t st) override {
        if constexpr (!std::is_same<T, float>::value) {
            set_error("UVLM graph step: float runs only");
            return GBVLM_ERR_ARG;
        } else {
            GB_REQUIRE(!looping, "UVLM: a request loop advances this case (destroy it first)");
            GB_REQUIRE(!roll_, "UVLM graph step: roll-up runs step on the host");
            GB_REQUIRE(next_step >= 1, "UVLM graph step: take the first step with gbvlm_uvlm_step");
            GB_REQUIRE(next_step + 1 < t_steps, "UVLM: all %lld steps done (wake capacity)", (long long)t_steps);
            int rc;
            if (!sexec && (rc = build_step_graph(st))) return rc;
            if (dev_idx != next_step) {
                GB_CUDA(cudaMemcpyAsync(d_idx, &next_step, sizeof(int64_t), cudaMemcpyHostToDevice, st));
                GB_CUDA(cudaStreamSynchronize(st));  // next_step is host memory that changes below
            }
            GB_CUDA(cudaGraphLaunch(sexec, st));
            next_step++;
            dev_idx = next_step;
            return GBVLM_OK;
        }
    }

    // the device-indexed step on stream c (captured by step_graph and by the
    // request loop of gbvlm_uvlm_loop_*)
    int enqueue_dev_step(cudaStream_t c) {
        gbvlm_stream cs = (gbvlm_stream)c;
        int r;
        k_uvlm_dev_pose<T><<<1, 128, 0, c>>>(d_idx, Tm, Tdm, fs, ref, nsurf, d_pose);
        GB_LAUNCH_CHECK();
        if ((r = wake_shed_dev_f32(nsurf, dims.data(), C(verts).data(), wake.data(), d_idx, c))) return r;
        for (int m = 0; m < nsurf; m++) {
            const int64_t np = dims[m].ns * dims[m].nc;
            k_dual_velocity<T><<<(unsigned)cdiv(np, 256), 256, 0, c>>>(d_pose + 16 * nsurf + 16 * m,
                                                                      colloc0[m], vel[m], np);
            GB_LAUNCH_CHECK();
        }
        GB_CUDA(cudaMemsetAsync(rhs, 0, sizeof(T) * n, c));
        if ((r = Ops2<T>::rhsv(rhs, nsurf, dims.data(), C(normals).data(), C(vel).data(), cs))) return r;
        if ((r = wake_influence_dev_f32(rhs, nsurf, dims.data(), C(gwake).data(), C(colloc).data(),
                                        C(normals).data(), C(wake).data(), lifting.data(), d_idx,
                                        (int32_t)(t_steps - 2), wsc, c)))
            return r;
        if ((r = lu_solve_prepared_f32(lu, lut, n, c))) return r;
        int64_t off = 0;
        for (int m = 0; m < nsurf; m++) {
            const int64_t ns = dims[m].ns, nc = dims[m].nc;
            if ((r = gamma_update_dev_f32(ns, nc, rhs + off, gamma[m], gdelta[m], gwake[m], t_steps - 2, d_idx,
                                          gprev[m], gdt[m], dt_, c)))
                return r;
            off += ns * nc;
        }
        for (int m = 0; m < nsurf; m++)
            if ((r = Ops2<T>::forces(dims[m].ns, dims[m].nc, verts[m], gdelta[m], gdt[m], vel[m], areas[m],
                                     normals[m], forces[m], cs)))
                return r;
        k_step_coeffs<T><<<1, 512, 0, c>>>(ca, d_pose + 32 * nsurf, d_pose + 32 * nsurf + 3, 0, 1.0, d_coef);
        GB_LAUNCH_CHECK();
        for (int m = 0; m < nsurf; m++) {
            const int64_t np = dims[m].ns * dims[m].nc;
            GB_CUDA(cudaMemcpyAsync(gprev[m], gamma[m], sizeof(T) * np, cudaMemcpyDeviceToDevice, c));
        }
        std::vector<const T*> tn(nsurf);
        for (int m = 0; m < nsurf; m++) tn[m] = d_pose + 16 * m;
        if ((r = Ops2<T>::displace(nsurf, dims.data(), tn.data(), verts.data(), C(vpos).data(), cs))) return r;
        if ((r = Ops2<T>::metrics(nsurf, dims.data(), C(verts).data(), colloc.data(), normals.data(),
                                  areas.data(), cs)))
            return r;
        k_uvlm_dev_end<<<1, 32, 0, c>>>(d_idx, d_coef, res);
        GB_LAUNCH_CHECK();
        return GBVLM_OK;
    }

    // device buffers of the device-indexed step and the staged LU solve
    int prepare_dev(cudaStream_t st) {
        if (!dmem) {
            const size_t pose = sizeof(T) * (32 * nsurf + 6), wb = sizeof(float) * WAKE_DEV_MAX_SLICES * n;
            GB_CUDA(cudaMalloc(&dmem, 256 + 256 + (pose + 255) / 256 * 256 + wb));
            d_idx = (int64_t*)dmem;
            d_coef = (double*)((char*)dmem + 256);
            d_pose = (T*)((char*)dmem + 512);
            wsc = (float*)((char*)dmem + 512 + (pose + 255) / 256 * 256);
        }
        if constexpr (std::is_same<T, float>::value) {
            if (!lut) {
                int rc = lu_solve_prepare_f32(lu, lhs, n, rhs, &lut, st);
                if (rc) return rc;
            }
        }
        return GBVLM_OK;
    }

    int build_step_graph(cudaStream_t st) {
        if constexpr (std::is_same<T, float>::value) {
            int rc = prepare_dev(st);
            if (rc) return rc;
            if (!scap) GB_CUDA(cudaStreamCreateWithFlags(&scap, cudaStreamNonBlocking));
            GB_CUDA(cudaStreamSynchronize(st));
            GB_CUDA(cudaStreamBeginCapture(scap, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_dev_step(scap);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(scap, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            GB_CUDA(e);
            sgraph = g;
            GB_CUDA(cudaGraphInstantiate(&sexec, sgraph, 0));
            dev_idx = -1;
            return GBVLM_OK;
        } else {
            (void)st;
            return GBVLM_ERR_ARG;
        }
    }

    int64_t last_step() const override { return next_step - 1; }

    int step_result(int64_t i, double* cl, double* cm, cudaStream_t st) override {
        GB_REQUIRE(i >= 0 && i < t_steps, "step index outside the run");
        double h[4];
        GB_CUDA(cudaMemcpyAsync(h, res + 4 * i, sizeof(h), cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        if (cl) *cl = h[0];
        if (cm) for (int k = 0; k < 3; k++) cm[k] = h[1 + k];
        return lu_solve_check(lu, st);  // the steps' solves finished their bounded waits
    }

    int results(double* cl, double* cm, double* gamma_last, cudaStream_t st) override {
        std::vector<double> h(4 * t_steps);
        GB_CUDA(cudaMemcpyAsync(h.data(), res, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
        std::vector<T> g(n);
        if (gamma_last) {
            int64_t off = 0;
            for (int m = 0; m < nsurf; m++) {
                const int64_t np = dims[m].ns * dims[m].nc;
                GB_CUDA(cudaMemcpyAsync(g.data() + off, gamma[m], sizeof(T) * np, cudaMemcpyDeviceToHost, st));
                off += np;
            }
        }
        GB_CUDA(cudaStreamSynchronize(st));
        for (int64_t i = 0; i < t_steps; i++) {
            if (cl) cl[i] = h[4 * i];
            if (cm)
                for (int k = 0; k < 3; k++) cm[3 * i + k] = h[4 * i + 1 + k];
        }
        if (gamma_last)
            for (int64_t q = 0; q < n; q++) gamma_last[q] = (double)g[q];
        return lu_solve_check(lu, st);  // the steps' solves finished their bounded waits
    }
};

// ===========================================================================
// Coupled aeroelastic 2-DOF (pitch-plunge) UVLM, tests/uvlm_2dof.cpp:437-808
// (COUPLED branch).  Aerodynamics in float as the reference; structure in
// double on the device (Newmark-beta, gbvlm_struct.cu).  Per time step i a
// Newton loop on the load increment: Newmark step -> state at i+1 -> pose
// fs(t+dt).heave.pitch (value and time derivative) -> displaced wing,
// metrics, wake shed, panel velocities, RHS with the wake, solve with the
// AIC factored at t = 0 -> gamma, wing-flap delta coupling, forces, CL/CM ->
// loads F(i+1) and their increment -> converged when |du_prev - du| <= eps.
// Each iteration is a fixed chain of launches; the host reads one flag per
// iteration to end the loop.
// ===========================================================================
struct A2Dev {
    double M[4], C[4], K[4];
    double du[2], dv[2], da[2], dF[2], du_prev[2];
    double coef[4];  // CL, CM x, y, z of the iterate
    float T[16], dT[16], ref[3], fs[3];
    int converged;
    int32_t iter, max_iter;  // Newton iterations of the current step, and their limit
    int64_t step;            // the step being advanced: state i -> i + 1
    int64_t wit;             // wake rows of that step's solve (step + 1)
};

// state at i+1 from the Newmark increments, the pose and the moment point
__global__ void k_a2_pose(A2Dev* d, double* u, double* v, double* a, float dtf, double a_h, int32_t nsurf,
                          float* T_all, float* dT_all) {
    if (threadIdx.x != 0) return;
    const int64_t i = d->step;
    const double t_next = (double)((float)i * dtf + dtf);
    double* u1 = u + 2 * (i + 1);
    double* v1 = v + 2 * (i + 1);
    double* a1 = a + 2 * (i + 1);
    for (int k = 0; k < 2; k++) {
        u1[k] = u[2 * i + k] + d->du[k];
        v1[k] = v[2 * i + k] + d->dv[k];
        a1[k] = a[2 * i + k] + d->da[k];
    }
    const double h = u1[0], al = u1[1], hd = v1[0], ad = v1[1];
    const double px = 1.0 + a_h;
    // pitch: rotation about y through (px, 0, 0) (vlm_kinematics.hpp:184-201), and d/dt = dR/dalpha * alpha'
    const double c = cos(al), sn = sin(al);
    double P[16] = {c, 0, -sn, 0, 0, 1, 0, 0, sn, 0, c, 0, px - c * px, 0, sn * px, 1};   // column-major
    double dP[16] = {-sn * ad, 0, -c * ad, 0, 0, 0, 0, 0, c * ad, 0, -sn * ad, 0, sn * px * ad, 0, c * px * ad, 0};
    // heave: translation (0, 0, -h), d/dt (0, 0, -h'); freestream: translation (-t, 0, 0), d/dt (-1, 0, 0)
    double H[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, -h, 1};
    double dH[16] = {0};
    dH[14] = -hd;
    double Fm[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, -t_next, 0, 0, 1};
    double dFm[16] = {0};
    dFm[12] = -1.0;
    auto mul = [](const double* A, const double* B, double* R) {
        for (int cc = 0; cc < 4; cc++)
            for (int r = 0; r < 4; r++) {
                double s_ = 0;
                for (int k = 0; k < 4; k++) s_ += A[r + 4 * k] * B[k + 4 * cc];
                R[r + 4 * cc] = s_;
            }
    };
    double HP[16], dHP[16], t1[16], t2[16], TT[16], dTT[16];
    mul(H, P, HP);
    mul(dH, P, t1);
    mul(H, dP, t2);
    for (int q = 0; q < 16; q++) dHP[q] = t1[q] + t2[q];
    mul(Fm, HP, TT);
    mul(dFm, HP, t1);
    mul(Fm, dHP, t2);
    for (int q = 0; q < 16; q++) dTT[q] = t1[q] + t2[q];
    for (int q = 0; q < 16; q++) {
        d->T[q] = (float)TT[q];
        d->dT[q] = (float)dTT[q];
    }
    for (int r = 0; r < 3; r++) d->ref[r] = (float)(TT[r] * px + TT[r + 12]);
    for (int m = 0; m < nsurf; m++)
        for (int q = 0; q < 16; q++) {
            T_all[16 * m + q] = (float)TT[q];
            dT_all[16 * m + q] = (float)dTT[q];
        }
}

// the reference's wing-flap coupling: the flap's first chordwise row of
// gamma_delta also subtracts the wing's trailing-edge gamma (uvlm_2dof.cpp:578-584)
__global__ void k_a2_flap(float* gdelta1, const float* gamma0, int64_t ns, int64_t nc0) {
    const int64_t s_ = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s_ < ns) gdelta1[s_] -= gamma0[s_ + (nc0 - 1) * ns];
}

__host__ __device__ inline double torsional_cubic(double al) { return 0.1 * al + 40.0 * al * al * al; }

// loads of the iterate (uvlm_2dof.cpp:728-744) and the Newton test; the
// loop of the time step's graph continues while the test fails and at most
// max_iter iterations have run (the reference's loop, :639-807)
__global__ void k_a2_loads(A2Dev* d, double* u, double* F, double mu, double r_a, double om, double Ua, double eps,
                           cudaGraphConditionalHandle loop) {
    if (threadIdx.x != 0) return;
    const int64_t i = d->step;
    const double pi_f = (double)3.141593f;
    F[2 * (i + 1)] = -d->coef[0] / (pi_f * mu);
    F[2 * (i + 1) + 1] = (2.0 * d->coef[2]) / (pi_f * mu * r_a * r_a);
    d->dF[0] = F[2 * (i + 1)] - F[2 * i] - (om / Ua) * (om / Ua) * d->du[0];
    d->dF[1] = F[2 * (i + 1) + 1] - F[2 * i + 1] -
               1.0 / (Ua * Ua) * (torsional_cubic(u[2 * (i + 1) + 1]) - torsional_cubic(u[2 * i + 1]));
    const double k0 = d->du_prev[0] - d->du[0], k1 = d->du_prev[1] - d->du[1];
    d->converged = sqrt(k0 * k0 + k1 * k1) <= eps ? 1 : 0;
    d->iter += 1;
    cudaGraphSetConditional(loop, (!d->converged && d->iter <= d->max_iter) ? 1u : 0u);
}

// start of a time step: the previous circulation kept, increments and the
// iteration count cleared
struct A2Copy {
    int32_t n;
    const float* src[GBVLM_MAX_SURFACES];
    float* dst[GBVLM_MAX_SURFACES];
    int64_t cnt[GBVLM_MAX_SURFACES];
};
__global__ void k_a2_step_begin(A2Dev* d, A2Copy c) {
    for (int m = 0; m < c.n; m++)
        for (int64_t e = threadIdx.x; e < c.cnt[m]; e += blockDim.x) c.dst[m][e] = c.src[m][e];
    if (threadIdx.x == 0) {
        d->dF[0] = d->dF[1] = 0.0;
        d->du[0] = d->du[1] = 0.0;
        d->iter = 0;
    }
}
// end of a time step: its iteration count recorded, the next step's indices
__global__ void k_a2_step_end(A2Dev* d, int32_t* iters) {
    if (threadIdx.x != 0) return;
    iters[d->step] = d->iter;
    d->step += 1;
    d->wit = d->step + 1;
}
__global__ void k_a2_set(A2Dev* d, int64_t step, int32_t max_iter) {
    if (threadIdx.x != 0) return;
    d->step = step;
    d->wit = step + 1;
    d->max_iter = max_iter;
}

struct Aero2Dof {
    int32_t nsurf = 0;
    std::vector<gbvlm_dims> dims;
    std::vector<int32_t> lifting;
    gbvlm_2dof_vars vars{};
    double dt = 0;
    int64_t t_steps = 0, n = 0, done = 0;  // steps advanced
    void* mem = nullptr;
    std::vector<float*> vinit, verts, wake, colloc, colloch, normals, areas, gamma, gprev, gdelta, gdt, gwake, vel,
        forces;
    float *lhs = nullptr, *rhs = nullptr, *T_all = nullptr, *dT_all = nullptr;
    double *u = nullptr, *v = nullptr, *a = nullptr, *F = nullptr;
    A2Dev* dev = nullptr;
    gbvlm_lu lu = nullptr;
    gbvlm_newmark nm = nullptr;
    std::vector<int32_t> iters;
    CoefArgs<float> ca;
    // one time step as a CUDA graph: the Newton iterations in a conditional
    // while node, replayed step after step without host round trips
    void* aux = nullptr;             // iteration counts per step, wake-influence scratch
    int32_t* iters_dev = nullptr;
    float* wscratch = nullptr;
    void* lut = nullptr;             // the staged LU solve of the factored AIC
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;

    ~Aero2Dof() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
        if (lut) lu_solve_tables_free(lut);
        if (aux) cudaFree(aux);
        if (lu) gbvlm_lu_destroy(lu);
        if (nm) gbvlm_newmark_destroy(nm);
        if (mem) cudaFree(mem);
    }

    static std::vector<const float*> C(const std::vector<float*>& x) { return std::vector<const float*>(x.begin(), x.end()); }

    int init(int32_t ns_, const gbvlm_dims* d, const float* const* vh, const int32_t* lift, const gbvlm_2dof_vars& vr,
             double t_final, cudaStream_t st) {
        nsurf = ns_;
        vars = vr;
        dims.assign(d, d + ns_);
        lifting.assign(lift, lift + ns_);
        // nondimensional vertices (uvlm_2dof.cpp:428-435) and the time step: the chord of the last
        // chordwise panel of the last surface at the first spanwise station (:473-480), in float
        std::vector<std::vector<float>> vnd(nsurf);
        for (int m = 0; m < nsurf; m++) {
            const int64_t nv = (dims[m].ns + 1) * (dims[m].nc + 1);
            vnd[m].assign(vh[m], vh[m] + 4 * nv);
            for (int64_t q = 0; q < 3 * nv; q++) vnd[m][q] = (float)(vnd[m][q] / (float)vars.b);
        }
        {
            const gbvlm_dims& L = dims[nsurf - 1];
            const int64_t nv = (L.ns + 1) * (L.nc + 1), lastj = L.nc * (L.ns + 1), prevj = (L.nc - 1) * (L.ns + 1);
            const std::vector<float>& w = vnd[nsurf - 1];
            const float dx = w[lastj] - w[prevj], dy = w[nv + lastj] - w[nv + prevj];
            const float dz = w[2 * nv + lastj] - w[2 * nv + prevj];
            const float dtf = sqrtf(dx * dx + dy * dy + dz * dz);
            dt = (double)dtf;
            t_steps = (int64_t)((float)t_final / dtf);
        }
        GB_REQUIRE(t_steps >= 3, "aeroelastic 2-DOF: t_final %.3g gives %lld steps of %.3g", t_final,
                   (long long)t_steps, dt);
        size_t bytes = 0;
        auto al = [](size_t b) { return (b + 255) / 256 * 256; };
        n = 0;
        for (auto& x : dims) {
            x.nwv = t_steps;
            const int64_t np = x.ns * x.nc, nv = (x.ns + 1) * (x.nc + 1);
            n += np;
            bytes += al(4 * 4 * nv) * 2 + al(4 * 4 * (x.ns + 1) * t_steps) + al(4 * 3 * np) * 5 + al(4 * np) * 5 +
                     al(4 * x.ns * (t_steps - 1));
        }
        bytes += al(4 * n * n) + al(4 * n) + 2 * al(4 * 16 * nsurf) + 4 * al(8 * 2 * t_steps) + al(sizeof(A2Dev));
        GB_CUDA(cudaMalloc(&mem, bytes));
        GB_CUDA(cudaMemset(mem, 0, bytes));
        char* p = (char*)mem;
        auto take = [&](size_t b) {
            void* r = p;
            p += al(b);
            return r;
        };
        lhs = (float*)take(4 * n * n);
        rhs = (float*)take(4 * n);
        T_all = (float*)take(4 * 16 * nsurf);
        dT_all = (float*)take(4 * 16 * nsurf);
        u = (double*)take(8 * 2 * t_steps);
        v = (double*)take(8 * 2 * t_steps);
        a = (double*)take(8 * 2 * t_steps);
        F = (double*)take(8 * 2 * t_steps);
        dev = (A2Dev*)take(sizeof(A2Dev));
        {
            const size_t ib = (sizeof(int32_t) * t_steps + 255) / 256 * 256;
            GB_CUDA(cudaMalloc(&aux, ib + sizeof(float) * WAKE_DEV_MAX_SLICES * n));
            iters_dev = (int32_t*)aux;
            wscratch = (float*)((char*)aux + ib);
        }
        for (auto& x : dims) {
            const int64_t np = x.ns * x.nc, nv = (x.ns + 1) * (x.nc + 1);
            vinit.push_back((float*)take(4 * 4 * nv));
            verts.push_back((float*)take(4 * 4 * nv));
            wake.push_back((float*)take(4 * 4 * (x.ns + 1) * t_steps));
            colloc.push_back((float*)take(4 * 3 * np));
            colloch.push_back((float*)take(4 * 3 * np));
            normals.push_back((float*)take(4 * 3 * np));
            vel.push_back((float*)take(4 * 3 * np));
            forces.push_back((float*)take(4 * 3 * np));
            areas.push_back((float*)take(4 * np));
            gamma.push_back((float*)take(4 * np));
            gprev.push_back((float*)take(4 * np));
            gdelta.push_back((float*)take(4 * np));
            gdt.push_back((float*)take(4 * np));
            gwake.push_back((float*)take(4 * x.ns * (t_steps - 1)));
        }
        for (int m = 0; m < nsurf; m++) {
            GB_CUDA(cudaMemcpy(vinit[m], vnd[m].data(), 4 * vnd[m].size(), cudaMemcpyHostToDevice));
            std::vector<float> ones((dims[m].ns + 1) * t_steps, 1.f);  // wake w plane
            GB_CUDA(cudaMemcpy(wake[m] + 3 * (dims[m].ns + 1) * t_steps, ones.data(), 4 * ones.size(),
                               cudaMemcpyHostToDevice));
        }
        // structure (uvlm_2dof.cpp:352-416): K = 0, the linear stiffness is in the load
        A2Dev h{};
        const double xa = vars.x_a, ra = vars.r_a, om = vars.omega, Ua = vars.U_a;
        h.M[0] = 1.0;
        h.M[1] = xa / (ra * ra);
        h.M[2] = xa;
        h.M[3] = 1.0;
        h.C[0] = 2.0 * vars.zeta_h * (om / Ua);
        h.C[3] = 2.0 * vars.zeta_a / Ua;
        h.fs[0] = 1.f;  // -d/dt of the freestream translation (-t, 0, 0)
        GB_CUDA(cudaMemcpy(dev, &h, sizeof(h), cudaMemcpyHostToDevice));
        {
            const double u0[2] = {0.0, 3.0 * M_PI / 180.0}, v0[2] = {0.0, 0.0};
            const double r0[2] = {-(om / Ua) * (om / Ua) * u0[0], -1.0 / (Ua * Ua) * torsional_cubic(u0[1])};
            // M a0 = r0 - C v0 - K u0 (2 x 2, column-major M)
            const double det = h.M[0] * h.M[3] - h.M[2] * h.M[1];
            const double a0[2] = {(h.M[3] * r0[0] - h.M[2] * r0[1]) / det, (-h.M[1] * r0[0] + h.M[0] * r0[1]) / det};
            GB_CUDA(cudaMemcpy(u, u0, sizeof(u0), cudaMemcpyHostToDevice));
            GB_CUDA(cudaMemcpy(v, v0, sizeof(v0), cudaMemcpyHostToDevice));
            GB_CUDA(cudaMemcpy(a, a0, sizeof(a0), cudaMemcpyHostToDevice));
        }
        int rc = gbvlm_newmark_create(&nm, 0.25, 0.5);
        if (rc) return rc;
        if ((rc = gbvlm_newmark_init(nm, 2, dev->M, dev->C, dev->K, dt, (gbvlm_stream)st))) return rc;
        if ((rc = gbvlm_lu_create(&lu))) return rc;
        if ((rc = gbvlm_lu_init(lu, n))) return rc;
        memset(&ca, 0, sizeof(ca));
        ca.n = nsurf;
        for (int m = 0; m < nsurf; m++) {
            ca.ns[m] = dims[m].ns;
            ca.nc[m] = dims[m].nc;
            ca.forces[m] = forces[m];
            ca.verts[m] = verts[m];
            ca.areas[m] = areas[m];
        }
        return start(st);
    }

    // initial pose, AIC factored once, the t = 0 solve (uvlm_2dof.cpp:453-515)
    int start(cudaStream_t st) {
        gbvlm_stream s = (gbvlm_stream)st;
        const double px = 1.0 + vars.a_h, th = 3.0 * M_PI / 180.0, c = cos(th), sn = sin(th);
        float T0[16] = {(float)c, 0, (float)-sn, 0, 0, 1, 0, 0, (float)sn, 0, (float)c, 0,
                        (float)(px - c * px), 0, (float)(sn * px), 1};
        float dT0[16] = {0};
        dT0[12] = -1.f;
        std::vector<float> ta(16 * nsurf), tb(16 * nsurf);
        for (int m = 0; m < nsurf; m++)
            for (int q = 0; q < 16; q++) {
                ta[16 * m + q] = T0[q];
                tb[16 * m + q] = dT0[q];
            }
        GB_CUDA(cudaMemcpyAsync(T_all, ta.data(), 4 * ta.size(), cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(dT_all, tb.data(), 4 * tb.size(), cudaMemcpyHostToDevice, st));
        std::vector<const float*> tr(nsurf);
        for (int m = 0; m < nsurf; m++) tr[m] = T_all + 16 * m;
        int rc;
        if ((rc = Ops2<float>::displace(nsurf, dims.data(), tr.data(), verts.data(), C(vinit).data(), s))) return rc;
        if ((rc = Ops2<float>::metrics(nsurf, dims.data(), C(verts).data(), colloc.data(), normals.data(),
                                       areas.data(), s)))
            return rc;
        for (int m = 0; m < nsurf; m++)
            GB_CUDA(cudaMemcpyAsync(colloch[m], colloc[m], 4 * 3 * dims[m].ns * dims[m].nc, cudaMemcpyDeviceToDevice,
                                    st));
        GB_CUDA(cudaMemsetAsync(lhs, 0, 4 * n * n, st));
        if ((rc = Ops2<float>::lhs(lhs, n, nsurf, dims.data(), C(colloc).data(), C(normals).data(), C(verts).data(),
                                   0.f, s)))
            return rc;
        if ((rc = Ops2<float>::factor(lu, lhs, n, s))) return rc;
        if (!lut && (rc = lu_solve_prepare_f32(lu, lhs, n, rhs, &lut, st))) return rc;
        if ((rc = Ops2<float>::shed(nsurf, dims.data(), C(verts).data(), wake.data(), 0, s))) return rc;
        if ((rc = aero_solve(0, st))) return rc;
        done = 0;
        iters.clear();
        return GBVLM_OK;
    }

    // velocities, RHS, solve and circulation of the current pose (wake rows 0..it)
    int aero_solve(int64_t it, cudaStream_t st) {
        gbvlm_stream s = (gbvlm_stream)st;
        int rc;
        for (int m = 0; m < nsurf; m++) {
            const int64_t np = dims[m].ns * dims[m].nc;
            k_dual_velocity<float><<<(unsigned)cdiv(np, 256), 256, 0, st>>>(dT_all + 16 * m, colloch[m], vel[m], np);
            GB_LAUNCH_CHECK();
        }
        GB_CUDA(cudaMemsetAsync(rhs, 0, 4 * n, st));
        if ((rc = Ops2<float>::rhsv(rhs, nsurf, dims.data(), C(normals).data(), C(vel).data(), s))) return rc;
        if ((rc = Ops2<float>::wake(rhs, nsurf, dims.data(), C(gwake).data(), C(colloc).data(), C(normals).data(),
                                    C(wake).data(), lifting.data(), (int32_t)it, 0.f, s)))
            return rc;
        if ((rc = Ops2<float>::solve(lu, lhs, n, rhs, s))) return rc;
        int64_t off = 0;
        for (int m = 0; m < nsurf; m++) {
            const int64_t ns = dims[m].ns, nc = dims[m].nc;
            if ((rc = Ops2<float>::gupd(ns, nc, rhs + off, gamma[m], gdelta[m], gwake[m], t_steps - 2 - it, gprev[m],
                                        gdt[m], (float)dt, s)))
                return rc;
            off += ns * nc;
        }
        if (nsurf > 1 && dims[1].ns == dims[0].ns) {
            k_a2_flap<<<(unsigned)cdiv(dims[1].ns, 128), 128, 0, st>>>(gdelta[1], gamma[0], dims[0].ns, dims[0].nc);
            GB_LAUNCH_CHECK();
        }
        return GBVLM_OK;
    }

    // one Newton iteration of the step dev->step (uvlm_2dof.cpp:639-751), with
    // every step-dependent index read on the device: captured into the body
    // of the step graph's while node
    int iterate_dev(cudaStream_t st, cudaGraphConditionalHandle loop) {
        gbvlm_stream s = (gbvlm_stream)st;
        int rc;
        GB_CUDA(cudaMemcpyAsync(dev->du_prev, dev->du, sizeof(double) * 2, cudaMemcpyDeviceToDevice, st));
        if ((rc = newmark_step_dev(nm, dev->M, dev->C, v, a, &dev->step, dev->du, dev->dv, dev->da, dev->dF, dt, st)))
            return rc;
        k_a2_pose<<<1, 32, 0, st>>>(dev, u, v, a, (float)dt, vars.a_h, nsurf, T_all, dT_all);
        GB_LAUNCH_CHECK();
        std::vector<const float*> tr(nsurf);
        for (int m = 0; m < nsurf; m++) tr[m] = T_all + 16 * m;
        if ((rc = Ops2<float>::displace(nsurf, dims.data(), tr.data(), verts.data(), C(vinit).data(), s))) return rc;
        if ((rc = Ops2<float>::metrics(nsurf, dims.data(), C(verts).data(), colloc.data(), normals.data(),
                                       areas.data(), s)))
            return rc;
        if ((rc = wake_shed_dev_f32(nsurf, dims.data(), C(verts).data(), wake.data(), &dev->wit, st))) return rc;
        // velocities, RHS, solve and circulation of the pose (wake rows 0..step+1)
        for (int m = 0; m < nsurf; m++) {
            const int64_t np = dims[m].ns * dims[m].nc;
            k_dual_velocity<float><<<(unsigned)cdiv(np, 256), 256, 0, st>>>(dT_all + 16 * m, colloch[m], vel[m], np);
            GB_LAUNCH_CHECK();
        }
        GB_CUDA(cudaMemsetAsync(rhs, 0, 4 * n, st));
        if ((rc = Ops2<float>::rhsv(rhs, nsurf, dims.data(), C(normals).data(), C(vel).data(), s))) return rc;
        if ((rc = wake_influence_dev_f32(rhs, nsurf, dims.data(), C(gwake).data(), C(colloc).data(),
                                         C(normals).data(), C(wake).data(), lifting.data(), &dev->wit,
                                         (int32_t)(t_steps - 2), wscratch, st)))
            return rc;
        if ((rc = lu_solve_prepared_f32(lu, lut, n, st))) return rc;
        int64_t off = 0;
        for (int m = 0; m < nsurf; m++) {
            const int64_t ns = dims[m].ns, nc = dims[m].nc;
            if ((rc = gamma_update_dev_f32(ns, nc, rhs + off, gamma[m], gdelta[m], gwake[m], t_steps - 2, &dev->wit,
                                           gprev[m], gdt[m], (float)dt, st)))
                return rc;
            off += ns * nc;
        }
        if (nsurf > 1 && dims[1].ns == dims[0].ns) {
            k_a2_flap<<<(unsigned)cdiv(dims[1].ns, 128), 128, 0, st>>>(gdelta[1], gamma[0], dims[0].ns, dims[0].nc);
            GB_LAUNCH_CHECK();
        }
        for (int m = 0; m < nsurf; m++)
            if ((rc = Ops2<float>::forces(dims[m].ns, dims[m].nc, verts[m], gdelta[m], gdt[m], vel[m], areas[m],
                                          normals[m], forces[m], s)))
                return rc;
        k_step_coeffs<float><<<1, 512, 0, st>>>(ca, dev->fs, dev->ref, 0, vars.rho, dev->coef);
        GB_LAUNCH_CHECK();
        k_a2_loads<<<1, 32, 0, st>>>(dev, u, F, vars.mu, vars.r_a, vars.omega, vars.U_a,
                                     (double)1.1920928955078125e-07, loop);
        GB_LAUNCH_CHECK();
        return GBVLM_OK;
    }

    // the step graph: begin (previous circulation, cleared increments) ->
    // while (Newton test fails and iterations <= max_iter) { iteration } -> end
    int build_graph() {
        if (exec) return GBVLM_OK;
        GB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        GB_CUDA(cudaGraphCreate(&graph, 0));
        cudaGraphConditionalHandle loop;
        GB_CUDA(cudaGraphConditionalHandleCreate(&loop, graph, 1, cudaGraphCondAssignDefault));
        A2Copy cp{};
        cp.n = nsurf;
        for (int m = 0; m < nsurf; m++) {
            cp.src[m] = gamma[m];
            cp.dst[m] = gprev[m];
            cp.cnt[m] = dims[m].ns * dims[m].nc;
        }
        cudaGraphNode_t nb, nw, ne;
        {
            void* args[] = {&dev, &cp};
            cudaKernelNodeParams kp = {};
            kp.func = (void*)k_a2_step_begin;
            kp.gridDim = dim3(1);
            kp.blockDim = dim3(256);
            kp.kernelParams = args;
            GB_CUDA(cudaGraphAddKernelNode(&nb, graph, nullptr, 0, &kp));
        }
        cudaGraphNodeParams wp = {};
        wp.type = cudaGraphNodeTypeConditional;
        wp.conditional.handle = loop;
        wp.conditional.type = cudaGraphCondTypeWhile;
        wp.conditional.size = 1;
        GB_CUDA(cudaGraphAddNode(&nw, graph, &nb, nullptr, 1, &wp));
        cudaGraph_t body = wp.conditional.phGraph_out[0];
        GB_CUDA(cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        int rc = iterate_dev(cap, loop);
        cudaGraph_t got = nullptr;
        const cudaError_t e = cudaStreamEndCapture(cap, &got);
        if (rc) return rc;
        GB_CUDA(e);
        {
            void* args[] = {&dev, &iters_dev};
            cudaKernelNodeParams kp = {};
            kp.func = (void*)k_a2_step_end;
            kp.gridDim = dim3(1);
            kp.blockDim = dim3(32);
            kp.kernelParams = args;
            GB_CUDA(cudaGraphAddKernelNode(&ne, graph, &nw, 1, &kp));
        }
        GB_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        return GBVLM_OK;
    }

    int run(int64_t steps, int32_t max_iter, cudaStream_t st) {
        GB_REQUIRE(done + steps <= t_steps - 2, "aeroelastic 2-DOF: %lld steps requested, %lld left",
                   (long long)steps, (long long)(t_steps - 2 - done));
        GB_REQUIRE(max_iter >= 0, "aeroelastic 2-DOF: max_iter must be non-negative");
        if (steps <= 0) return GBVLM_OK;
        int rc = build_graph();
        if (rc) return rc;
        k_a2_set<<<1, 32, 0, st>>>(dev, done, max_iter);
        GB_LAUNCH_CHECK();
        for (int64_t k = 0; k < steps; k++) GB_CUDA(cudaGraphLaunch(exec, st));
        std::vector<int32_t> h(steps);
        GB_CUDA(cudaMemcpyAsync(h.data(), iters_dev + done, sizeof(int32_t) * steps, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        iters.insert(iters.end(), h.begin(), h.end());
        done += steps;
        return GBVLM_OK;
    }
};

}  // namespace gbvlm

using namespace gbvlm;

struct gbvlm_uvlm_s {
    UvlmBase* impl = nullptr;
};

// ===========================================================================
// Device-resident request loop over a resident UVLM case.  One CUDA graph: a
// while node whose body is the device-indexed step followed by
// k_uvlm_loop_next.  The host submits a request by raising a counter in
// mapped host memory; the running graph takes one step per request, writes
// each step's coefficients into a mapped record and raises the done
// counter, then waits (bounded) for the next request.  After poll_ns
// without one it marks itself stopped and ends; the next submit launches
// the graph again.  Between requests no CUDA call is made.
// ===========================================================================
namespace gbvlm {

struct LoopCtl {
    int64_t enq;    // requests submitted (host)
    int64_t done;   // requests completed (device)
    int32_t state;  // 0: no graph running or about to run, 1: running (both sides, system-scope atomics)
    int32_t stop;   // host: end the loop
    int32_t error;  // device: 1 = the wake is full
    int32_t pad;
};
struct LoopRec {
    int64_t step;
    double c[4];  // CL, CM x, y, z
};

__device__ __forceinline__ uint64_t loop_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// last_idx: the largest step index the wake holds
__global__ void k_uvlm_loop_next(LoopCtl* ctl, LoopRec* rec, const int64_t* idx, const double* res, int64_t last_idx,
                                 uint64_t poll_ns, cudaGraphConditionalHandle loop) {
    if (threadIdx.x != 0) return;
    volatile LoopCtl* vc = ctl;
    const int64_t i = idx[0] - 1;  // the step this iteration took
    const int64_t t = vc->done;
    rec[t].step = i;
    for (int k = 0; k < 4; k++) rec[t].c[k] = res[4 * i + k];
    __threadfence_system();
    vc->done = t + 1;
    __threadfence_system();
    unsigned cont = 0;
    bool released = false;
    if (idx[0] > last_idx) {
        vc->error = 1;
    } else {
        const uint64_t t0 = loop_ns();
        while (true) {
            if (vc->stop) break;
            if (vc->enq > t + 1) {
                cont = 1;
                break;
            }
            if (loop_ns() - t0 > poll_ns) {
                // stop, unless a request came in meanwhile and the host has
                // not already taken the running state to launch a new graph
                atomicExch_system(&ctl->state, 0);
                released = true;
                __threadfence_system();
                if (vc->enq > t + 1 && atomicCAS_system(&ctl->state, 0, 1) == 0) {
                    cont = 1;
                    released = false;
                }
                break;
            }
            __nanosleep(2000);
        }
    }
    if (!cont && !released) atomicExch_system(&ctl->state, 0);
    cudaGraphSetConditional(loop, cont);
}

}  // namespace gbvlm

struct gbvlm_uvlm_loop_s {
    gbvlm_uvlm owner = nullptr;
    UvlmState<float>* u = nullptr;
    LoopCtl* ctl = nullptr;  // mapped host memory
    LoopRec* rec = nullptr;
    LoopCtl* ctl_d = nullptr;
    LoopRec* rec_d = nullptr;
    int64_t cap = 0, base_step = 0, enq = 0, launches = 0;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::mutex mu;
    ~gbvlm_uvlm_loop_s() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (st) cudaStreamDestroy(st);
        if (ctl) cudaFreeHost(ctl);
        if (rec) cudaFreeHost(rec);
    }
};

extern "C" {

int gbvlm_uvlm_create(gbvlm_uvlm* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                      const int32_t* lifting, int64_t t_steps, int32_t precision) {
    GB_REQUIRE(out && dims && verts_init && lifting, "null argument");
    GB_REQUIRE(nsurf >= 1 && nsurf <= GBVLM_MAX_SURFACES, "nsurf=%d outside [1, %d]", nsurf, GBVLM_MAX_SURFACES);
    GB_REQUIRE(t_steps >= 2, "t_steps must be at least 2");
    GB_REQUIRE(precision == 32 || precision == 64, "precision must be 32 or 64");
    for (int m = 0; m < nsurf; m++) GB_REQUIRE(verts_init[m] && dims[m].ns >= 1 && dims[m].nc >= 1, "surface %d", m);
    auto* h = new gbvlm_uvlm_s();
    int rc;
    if (precision == 32) {
        auto* s = new UvlmState<float>();
        h->impl = s;
        rc = s->init(nsurf, dims, verts_init, lifting, t_steps);
    } else {
        auto* s = new UvlmState<double>();
        h->impl = s;
        rc = s->init(nsurf, dims, verts_init, lifting, t_steps);
    }
    if (rc) {
        delete h->impl;
        delete h;
        return rc;
    }
    *out = h;
    return GBVLM_OK;
}

int gbvlm_uvlm_destroy(gbvlm_uvlm h) {
    if (!h) return GBVLM_OK;
    GB_REQUIRE(!h->impl || !h->impl->looping, "UVLM: destroy its request loop first");
    delete h->impl;
    delete h;
    return GBVLM_OK;
}

int gbvlm_uvlm_set_kinematics(gbvlm_uvlm h, const double* transforms, const double* dtransforms,
                              const double* freestream, const double* ref_pt) {
    GB_REQUIRE(h && h->impl && transforms && dtransforms && freestream, "null argument");
    return h->impl->set_kinematics(transforms, dtransforms, freestream, ref_pt);
}

int gbvlm_uvlm_run(gbvlm_uvlm h, double dt, int32_t rollup, double sigma, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl && dt > 0, "bad arguments");
    return h->impl->run(dt, rollup, sigma, to_cuda(stream));
}

int gbvlm_uvlm_begin(gbvlm_uvlm h, double dt, int32_t rollup, double sigma, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl && dt > 0, "bad arguments");
    return h->impl->begin(dt, rollup, sigma, to_cuda(stream));
}

int gbvlm_uvlm_step(gbvlm_uvlm h, int64_t* step_index, double* cl, double* cm, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl, "null argument");
    int rc = h->impl->step(to_cuda(stream));
    if (rc) return rc;
    auto* u = h->impl;
    const int64_t i = u->last_step();
    if (step_index) *step_index = i;
    if (cl || cm) return u->step_result(i, cl, cm, to_cuda(stream));
    return GBVLM_OK;
}

int gbvlm_uvlm_step_graph(gbvlm_uvlm h, int64_t* step_index, double* cl, double* cm, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl, "null argument");
    int rc = h->impl->step_graph(to_cuda(stream));
    if (rc) return rc;
    auto* u = h->impl;
    const int64_t i = u->last_step();
    if (step_index) *step_index = i;
    if (cl || cm) return u->step_result(i, cl, cm, to_cuda(stream));
    return GBVLM_OK;
}

int gbvlm_uvlm_loop_create(gbvlm_uvlm_loop* out, gbvlm_uvlm h, double poll_s) {
    GB_REQUIRE(out && h && h->impl, "null argument");
    GB_REQUIRE(poll_s > 0 && poll_s <= 1.0, "poll_s=%g outside (0, 1] s", poll_s);
    auto* u = dynamic_cast<UvlmState<float>*>(h->impl);
    GB_REQUIRE(u, "UVLM request loop: float runs only");
    GB_REQUIRE(!u->looping, "UVLM request loop: this case already has one");
    GB_REQUIRE(!u->roll_, "UVLM request loop: roll-up runs step on the host");
    GB_REQUIRE(u->next_step >= 1, "UVLM request loop: take the first step with gbvlm_uvlm_step");
    GB_REQUIRE(u->next_step + 1 < u->t_steps, "UVLM: all %lld steps done (wake capacity)", (long long)u->t_steps);
    int dev = 0, native = 0;
    GB_CUDA(cudaGetDevice(&dev));
    GB_CUDA(cudaDeviceGetAttribute(&native, cudaDevAttrHostNativeAtomicSupported, dev));
    GB_REQUIRE(native, "UVLM request loop: the device has no native atomics on host memory");
    auto* l = new gbvlm_uvlm_loop_s();
    l->owner = h;
    l->u = u;
    l->base_step = u->next_step;
    l->cap = u->t_steps - 1 - u->next_step;
    auto fail = [&](int rc) {
        delete l;
        return rc;
    };
    int rc = u->prepare_dev(0);
    if (rc) return fail(rc);
    cudaError_t e = cudaStreamCreateWithFlags(&l->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&l->ctl, sizeof(LoopCtl), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&l->rec, sizeof(LoopRec) * (size_t)l->cap, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&l->ctl_d, l->ctl, 0);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&l->rec_d, l->rec, 0);
    if (e != cudaSuccess) return fail(cuda_fail(e, "UVLM request loop set-up", __FILE__, __LINE__));
    memset(l->ctl, 0, sizeof(LoopCtl));
    memset(l->rec, 0, sizeof(LoopRec) * (size_t)l->cap);
    // the device step counter at the case's next step
    e = cudaMemcpy(u->d_idx, &u->next_step, sizeof(int64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(cuda_fail(e, "UVLM request loop set-up", __FILE__, __LINE__));
    u->dev_idx = u->next_step;
    // graph: while (cond) { device-indexed step; next }
    cudaGraphConditionalHandle cond;
    cudaGraphNode_t nw;
    cudaGraphNodeParams wp = {};
    e = cudaGraphCreate(&l->graph, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&cond, l->graph, 1, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) {
        wp.type = cudaGraphNodeTypeConditional;
        wp.conditional.handle = cond;
        wp.conditional.type = cudaGraphCondTypeWhile;
        wp.conditional.size = 1;
        e = cudaGraphAddNode(&nw, l->graph, nullptr, nullptr, 0, &wp);
    }
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(l->st, wp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail(cuda_fail(e, "UVLM request loop graph", __FILE__, __LINE__));
    rc = u->enqueue_dev_step(l->st);
    if (rc == GBVLM_OK) {
        const uint64_t poll_ns = (uint64_t)(poll_s * 1e9);
        k_uvlm_loop_next<<<1, 32, 0, l->st>>>(l->ctl_d, l->rec_d, u->d_idx, u->res, u->t_steps - 2, poll_ns, cond);
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) rc = cuda_fail(le, "k_uvlm_loop_next", __FILE__, __LINE__);
    }
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(l->st, &got);
    if (rc) return fail(rc);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&l->exec, l->graph, 0);
    if (e != cudaSuccess) return fail(cuda_fail(e, "UVLM request loop graph", __FILE__, __LINE__));
    u->looping = true;
    *out = l;
    return GBVLM_OK;
}

int gbvlm_uvlm_loop_submit(gbvlm_uvlm_loop l, int64_t* ticket) {
    GB_REQUIRE(l && ticket, "null argument");
    std::lock_guard<std::mutex> g(l->mu);
    GB_REQUIRE(l->enq < l->cap, "UVLM request loop: the wake holds %lld more steps", (long long)l->cap);
    GB_REQUIRE(!__atomic_load_n(&l->ctl->stop, __ATOMIC_SEQ_CST), "UVLM request loop: stopped");
    const int64_t t = ++l->enq;
    __atomic_store_n(&l->ctl->enq, t, __ATOMIC_SEQ_CST);
    std::atomic_thread_fence(std::memory_order_seq_cst);
    int32_t idle = 0;
    if (__atomic_load_n(&l->ctl->state, __ATOMIC_SEQ_CST) == 0 &&
        __atomic_compare_exchange_n(&l->ctl->state, &idle, 1, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
        GB_CUDA(cudaGraphLaunch(l->exec, l->st));
        l->launches++;
    }
    *ticket = t;
    return GBVLM_OK;
}

int gbvlm_uvlm_loop_wait(gbvlm_uvlm_loop l, int64_t ticket, double timeout_s, int64_t* step_index, double* cl,
                         double* cm) {
    GB_REQUIRE(l && ticket >= 1 && timeout_s >= 0, "bad arguments");
    GB_REQUIRE(ticket <= l->enq, "UVLM request loop: ticket %lld not submitted", (long long)ticket);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (__atomic_load_n(&l->ctl->done, __ATOMIC_ACQUIRE) < ticket) {
        if (__atomic_load_n(&l->ctl->error, __ATOMIC_ACQUIRE)) {
            set_error("UVLM request loop: the wake is full");
            return GBVLM_ERR_ARG;
        }
        const cudaError_t q = cudaStreamQuery(l->st);
        if (q != cudaSuccess && q != cudaErrorNotReady) return cuda_fail(q, "UVLM request loop", __FILE__, __LINE__);
        if (std::chrono::steady_clock::now() > deadline) {
            set_error("UVLM request loop: ticket %lld not done within %g s", (long long)ticket, timeout_s);
            return GBVLM_ERR_CUDA;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    const LoopRec& r = l->rec[ticket - 1];
    if (step_index) *step_index = r.step;
    if (cl) *cl = r.c[0];
    if (cm)
        for (int k = 0; k < 3; k++) cm[k] = r.c[1 + k];
    return GBVLM_OK;
}

int gbvlm_uvlm_loop_stats(gbvlm_uvlm_loop l, int64_t* submitted, int64_t* completed, int64_t* launches) {
    GB_REQUIRE(l, "null argument");
    std::lock_guard<std::mutex> g(l->mu);
    if (submitted) *submitted = l->enq;
    if (completed) *completed = __atomic_load_n(&l->ctl->done, __ATOMIC_ACQUIRE);
    if (launches) *launches = l->launches;
    return GBVLM_OK;
}

int gbvlm_uvlm_loop_destroy(gbvlm_uvlm_loop l) {
    if (!l) return GBVLM_OK;
    int rc = GBVLM_OK;
    {
        std::lock_guard<std::mutex> g(l->mu);
        __atomic_store_n(&l->ctl->stop, 1, __ATOMIC_SEQ_CST);
    }
    // a running graph sees the stop flag within its poll wait and ends
    cudaError_t e = cudaStreamSynchronize(l->st);
    if (e != cudaSuccess) rc = cuda_fail(e, "UVLM request loop", __FILE__, __LINE__);
    // the case continues host-stepped from where the loop left it
    const int64_t done = __atomic_load_n(&l->ctl->done, __ATOMIC_ACQUIRE);
    l->u->next_step = l->base_step + done;
    l->u->dev_idx = l->u->next_step;
    l->u->looping = false;
    delete l;
    return rc;
}

int gbvlm_uvlm_results(gbvlm_uvlm h, double* cl, double* cm, double* gamma_last, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl, "null argument");
    return h->impl->results(cl, cm, gamma_last, to_cuda(stream));
}

int gbvlm_aero2dof_create(gbvlm_aero2dof* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                          const int32_t* lifting, const gbvlm_2dof_vars* vars, double t_final, int64_t* t_steps,
                          double* dt, gbvlm_stream stream) {
    GB_REQUIRE(out && dims && verts_init && lifting && vars, "null argument");
    GB_REQUIRE(nsurf >= 1 && nsurf <= GBVLM_MAX_SURFACES, "nsurf=%d outside [1, %d]", nsurf, GBVLM_MAX_SURFACES);
    GB_REQUIRE(vars->b > 0 && vars->mu > 0 && vars->r_a > 0 && vars->U_a > 0, "aeroelastic 2-DOF: bad parameters");
    for (int m = 0; m < nsurf; m++) GB_REQUIRE(verts_init[m] && dims[m].ns >= 1 && dims[m].nc >= 1, "surface %d", m);
    GB_REQUIRE(dims[nsurf - 1].nc >= 2, "aeroelastic 2-DOF: the last surface needs two chordwise panels (time step)");
    auto* h = new Aero2Dof();
    int rc = h->init(nsurf, dims, verts_init, lifting, *vars, t_final, to_cuda(stream));
    if (rc) {
        delete h;
        return rc;
    }
    if (t_steps) *t_steps = h->t_steps;
    if (dt) *dt = h->dt;
    *out = (gbvlm_aero2dof)h;
    return GBVLM_OK;
}

int gbvlm_aero2dof_destroy(gbvlm_aero2dof h) {
    delete (Aero2Dof*)h;
    return GBVLM_OK;
}

int gbvlm_aero2dof_run(gbvlm_aero2dof h, int64_t steps, int32_t max_iter, gbvlm_stream stream) {
    GB_REQUIRE(h && steps >= 0 && max_iter >= 1, "bad arguments");
    return ((Aero2Dof*)h)->run(steps, max_iter, to_cuda(stream));
}

int gbvlm_aero2dof_results(gbvlm_aero2dof h, int64_t* steps_done, double* u, double* v, double* a, double* F,
                           int32_t* iters, gbvlm_stream stream) {
    GB_REQUIRE(h, "null argument");
    Aero2Dof* s = (Aero2Dof*)h;
    cudaStream_t st = to_cuda(stream);
    const size_t nb = sizeof(double) * 2 * (size_t)(s->done + 1);
    if (u) GB_CUDA(cudaMemcpyAsync(u, s->u, nb, cudaMemcpyDeviceToHost, st));
    if (v) GB_CUDA(cudaMemcpyAsync(v, s->v, nb, cudaMemcpyDeviceToHost, st));
    if (a) GB_CUDA(cudaMemcpyAsync(a, s->a, nb, cudaMemcpyDeviceToHost, st));
    if (F) GB_CUDA(cudaMemcpyAsync(F, s->F, nb, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (steps_done) *steps_done = s->done;
    if (iters)
        for (int64_t k = 0; k < s->done; k++) iters[k] = s->iters[k];
    return GBVLM_OK;
}

}  // extern "C"
