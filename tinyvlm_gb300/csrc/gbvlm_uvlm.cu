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
#include <string.h>

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

struct UvlmBase {
    virtual ~UvlmBase() = default;
    virtual int set_kinematics(const double* T, const double* Td, const double* fs, const double* ref) = 0;
    virtual int run(double dt, int32_t rollup, double sigma, cudaStream_t st) = 0;
    virtual int begin(double dt, int32_t rollup, double sigma, cudaStream_t st) = 0;
    virtual int step(cudaStream_t st) = 0;
    virtual int step_result(int64_t i, double* cl, double* cm, cudaStream_t st) = 0;
    virtual int64_t last_step() const = 0;
    virtual int results(double* cl, double* cm, double* gamma_last, cudaStream_t st) = 0;
    int64_t t_steps = 0, n = 0;
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

    ~UvlmState() override {
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
        int rc;
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

    int64_t last_step() const override { return next_step - 1; }

    int step_result(int64_t i, double* cl, double* cm, cudaStream_t st) override {
        GB_REQUIRE(i >= 0 && i < t_steps, "step index outside the run");
        double h[4];
        GB_CUDA(cudaMemcpyAsync(h, res + 4 * i, sizeof(h), cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        if (cl) *cl = h[0];
        if (cm) for (int k = 0; k < 3; k++) cm[k] = h[1 + k];
        return GBVLM_OK;
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
        return GBVLM_OK;
    }
};

}  // namespace gbvlm

using namespace gbvlm;

struct gbvlm_uvlm_s {
    UvlmBase* impl = nullptr;
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

int gbvlm_uvlm_results(gbvlm_uvlm h, double* cl, double* cm, double* gamma_last, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl, "null argument");
    return h->impl->results(cl, cm, gamma_last, to_cuda(stream));
}

}  // extern "C"
