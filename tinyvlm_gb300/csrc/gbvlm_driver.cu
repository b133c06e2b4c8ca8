// Host drivers above the operator C ABI: the steady VLM simulation
// (vlm/src/vlm.cpp:17-151), the nonlinear VLM (vlm.cpp:153-295) and the
// plot3d reader (vlm/src/vlm_mesh.cpp).
// These are the "plain per-solve" paths: one operator call per reference
// backend call, scalars read back synchronously, in float (the reference's
// semantics) or double.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <fstream>
#include <string>
#include <vector>

#include "gbvlm_internal.h"

namespace gbvlm {

template <class T>
__global__ void k_fill3(T* v, int64_t np, T x, T y, T z) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    v[p] = x;
    v[np + p] = y;
    v[2 * np + p] = z;
}

template <class T>
__global__ void k_cast(const float* in, T* out, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (T)in[i];
}

template <class T>
struct Ops;
#define OPS(T, sfx)                                                                                                  \
    template <>                                                                                                      \
    struct Ops<T> {                                                                                                  \
        static int lhs(T* a, int64_t ld, int32_t ns, const gbvlm_dims* d, const T* const* c, const T* const* n,      \
                       const T* const* vw, const T* const* vk, int32_t it, T sg, gbvlm_stream s) {                    \
            return gbvlm_lhs_assemble_##sfx(a, ld, ns, d, c, n, vw, vk, it, sg, s);                                  \
        }                                                                                                            \
        static int rhsv(T* r, int32_t ns, const gbvlm_dims* d, const T* const* n, const T* const* v, gbvlm_stream s) { \
            return gbvlm_rhs_assemble_velocities_##sfx(r, ns, d, n, v, s);                                          \
        }                                                                                                            \
        static int metrics(T a, int32_t ns, const gbvlm_dims* d, const T* const* v, T* const* c, T* const* n,        \
                           T* const* ar, gbvlm_stream s) {                                                           \
            return gbvlm_mesh_metrics_##sfx(a, ns, d, v, c, n, ar, s);                                              \
        }                                                                                                            \
        static int displace(int32_t ns, const gbvlm_dims* d, const T* const* t, T* const* v, const T* const* vi,     \
                            gbvlm_stream s) {                                                                        \
            return gbvlm_displace_wing_##sfx(ns, d, t, v, vi, s);                                                   \
        }                                                                                                            \
        static int shed(int32_t ns, const gbvlm_dims* d, const T* const* v, T* const* k, int32_t it, gbvlm_stream s) { \
            return gbvlm_wake_shed_##sfx(ns, d, v, k, it, s);                                                       \
        }                                                                                                            \
        static int factor(gbvlm_lu h, T* a, int64_t n, gbvlm_stream s) { return gbvlm_lu_factor_##sfx(h, a, n, n, s); } \
        static int solve(gbvlm_lu h, const T* a, int64_t n, T* x, gbvlm_stream s) {                                  \
            return gbvlm_lu_solve_##sfx(h, a, n, n, x, n, 1, s);                                                     \
        }                                                                                                            \
        static int gupd(int64_t ns, int64_t nc, const T* x, T* g, T* gd, T* gw, gbvlm_stream s) {                    \
            return gbvlm_gamma_update_##sfx(ns, nc, x, g, gd, gw, 0, nullptr, nullptr, (T)0, s);                     \
        }                                                                                                            \
        static int forces(int64_t ns, int64_t nc, const T* v, const T* gd, const T* vel, T* f, gbvlm_stream s) {     \
            return gbvlm_forces_steady_##sfx(ns, nc, v, gd, vel, f, s);                                             \
        }                                                                                                            \
        static int sum(const T* x, int64_t n, T* o, gbvlm_stream s) { return gbvlm_sum_##sfx(x, n, o, s); }          \
        static int cl(int64_t ns, int64_t nc, const T* f, const T* la, const T* fs, T rho, T area, T* o,             \
                      gbvlm_stream s) {                                                                              \
            return gbvlm_coeff_cl_##sfx(ns, nc, f, la, fs, rho, area, o, s);                                        \
        }                                                                                                            \
        static int cm(int64_t ns, int64_t nc, const T* f, const T* v, const T* r, const T* fs, T rho, T area, T mac, \
                      T* o, gbvlm_stream s) {                                                                        \
            return gbvlm_coeff_cm_##sfx(ns, nc, f, v, r, fs, rho, area, mac, o, s);                                 \
        }                                                                                                            \
        static int mac(int64_t ns, int64_t nc, const T* v, const T* a, T* o, gbvlm_stream s) {                       \
            return gbvlm_mesh_mac_##sfx(ns, nc, v, a, o, s);                                                        \
        }                                                                                                            \
        static int cd(int64_t ns, int64_t nwv, const T* vk, const T* gw, const T* fs, T area, T sg, T* o,            \
                      gbvlm_stream s) {                                                                              \
            return gbvlm_trefftz_cd_##sfx(ns, nwv, vk, gw, fs, area, sg, o, s);                                     \
        }                                                                                                            \
    };
OPS(float, f32)
OPS(double, f64)

// Per-precision simulation state of a steady VLM (vlm/src/vlm.cpp:60-95).
struct VlmBase {
    virtual ~VlmBase() = default;
    virtual int run(double alpha, double beta, double u_inf, double rho, const double* ref_pt, gbvlm_coeffs* out,
                    double* gamma_out, cudaStream_t st) = 0;
    virtual int run_shared(int32_t nalpha, const double* alphas, double u_inf, double rho, const double* ref_pt,
                           gbvlm_coeffs* out, double* gamma_out, cudaStream_t st) = 0;
};

template <class T>
struct VlmState : VlmBase {
    int32_t nsurf = 0;
    std::vector<gbvlm_dims> dims;
    int64_t n = 0;
    void* mem = nullptr;
    std::vector<T*> verts_init, verts, wake, colloc, normals, areas, gamma, gdelta, gwake, vel, forces, transform;
    T* lhs = nullptr;
    T* rhs = nullptr;
    gbvlm_lu lu = nullptr;
    T sigma = 0;

    ~VlmState() override {
        if (lu) gbvlm_lu_destroy(lu);
        if (mem) cudaFree(mem);
    }

    int init(int32_t ns_, const gbvlm_dims* d, const float* const* vinit_host) {
        nsurf = ns_;
        dims.assign(d, d + ns_);
        size_t bytes = 0;
        n = 0;
        for (auto& x : dims) {
            x.nwv = 2;  // single row of wake panels (vlm.cpp:73)
            int64_t np = x.ns * x.nc, nv = (x.ns + 1) * (x.nc + 1);
            n += np;
            bytes += sizeof(T) * (2 * 4 * nv + 4 * (x.ns + 1) * 2 + 3 * 3 * np + 3 * np + 3 * np + x.ns + 16 + 3 * np);
        }
        bytes += sizeof(T) * (n * n + n) + 4096 * 8;
        GB_CUDA(cudaMalloc(&mem, bytes));
        GB_CUDA(cudaMemset(mem, 0, bytes));
        char* p = (char*)mem;
        auto take = [&](int64_t cnt) {
            T* r = (T*)p;
            p += ((sizeof(T) * cnt + 255) / 256) * 256;
            return r;
        };
        lhs = take(n * n);
        rhs = take(n);
        for (auto& x : dims) {
            int64_t np = x.ns * x.nc, nv = (x.ns + 1) * (x.nc + 1);
            verts_init.push_back(take(4 * nv));
            verts.push_back(take(4 * nv));
            wake.push_back(take(4 * (x.ns + 1) * 2));
            colloc.push_back(take(3 * np));
            normals.push_back(take(3 * np));
            areas.push_back(take(np));
            gamma.push_back(take(np));
            gdelta.push_back(take(np));
            gwake.push_back(take(x.ns));
            vel.push_back(take(3 * np));
            forces.push_back(take(3 * np));
            transform.push_back(take(16));
        }
        // upload initial vertices (float host) and set wake w = 1
        for (int m = 0; m < nsurf; m++) {
            int64_t nv = (dims[m].ns + 1) * (dims[m].nc + 1);
            float* tmp = nullptr;
            GB_CUDA(cudaMalloc(&tmp, sizeof(float) * 4 * nv));
            GB_CUDA(cudaMemcpy(tmp, vinit_host[m], sizeof(float) * 4 * nv, cudaMemcpyHostToDevice));
            k_cast<T><<<(unsigned)cdiv(4 * nv, 256), 256>>>(tmp, verts_init[m], 4 * nv);
            GB_LAUNCH_CHECK();
            GB_CUDA(cudaDeviceSynchronize());
            cudaFree(tmp);
            std::vector<T> ones(2 * (dims[m].ns + 1), (T)1);
            GB_CUDA(cudaMemcpy(wake[m] + 3 * 2 * (dims[m].ns + 1), ones.data(), sizeof(T) * ones.size(),
                               cudaMemcpyHostToDevice));
        }
        int rc = gbvlm_lu_create(&lu);
        if (rc) return rc;
        return gbvlm_lu_init(lu, n);
    }

    // FlowData (vlm_utils.cpp:5-19): free stream and lift axis
    static void flow(T alpha, T beta, T u, T* fs, T* la) {
        fs[0] = u * (T)cos(alpha) * (T)cos(beta);
        fs[1] = -(u * (T)cos(alpha) * (T)sin(beta));
        fs[2] = u * (T)sin(alpha);
        la[0] = -fs[2];
        la[1] = (T)0;
        la[2] = fs[0];
        T ll = (T)sqrt(la[0] * la[0] + la[1] * la[1] + la[2] * la[2]);
        la[0] /= ll; la[1] /= ll; la[2] /= ll;
    }

    // Geometry, AIC and its factorisation for the angle alpha (vlm.cpp:97-126):
    // the 100-chord wake row along the free stream, collocation points with the
    // high-AoA factor of alpha; `tr` receives the wake translation.
    int assemble(T alpha, T u, T* tr, gbvlm_stream s, cudaStream_t st) {
        GB_CUDA(cudaMemsetAsync(lhs, 0, sizeof(T) * n * n, st));
        for (int m = 0; m < nsurf; m++) {
            int64_t nv = (dims[m].ns + 1) * (dims[m].nc + 1);
            GB_CUDA(cudaMemcpyAsync(verts[m], verts_init[m], sizeof(T) * 4 * nv, cudaMemcpyDeviceToDevice, st));
        }
        // 100-chord wake (vlm.cpp:104-114)
        const T t16[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, (T)-100 * u * (T)cos(alpha), 0,
                           (T)-100 * u * (T)sin(alpha), 1};
        for (int k = 0; k < 16; k++) tr[k] = t16[k];
        for (int m = 0; m < nsurf; m++)
            GB_CUDA(cudaMemcpyAsync(transform[m], t16, sizeof(t16), cudaMemcpyHostToDevice, st));
        std::vector<const T*> cverts(verts.begin(), verts.end()), cinit(verts_init.begin(), verts_init.end()),
            ctr(transform.begin(), transform.end()), ccol(colloc.begin(), colloc.end()),
            cnor(normals.begin(), normals.end()), cwake(wake.begin(), wake.end());
        int rc;
        if ((rc = Ops<T>::shed(nsurf, dims.data(), cverts.data(), wake.data(), 0, s))) return rc;
        if ((rc = Ops<T>::displace(nsurf, dims.data(), ctr.data(), verts.data(), cinit.data(), s))) return rc;
        if ((rc = Ops<T>::shed(nsurf, dims.data(), cverts.data(), wake.data(), 1, s))) return rc;
        if ((rc = Ops<T>::metrics(alpha, nsurf, dims.data(), cverts.data(), colloc.data(), normals.data(), areas.data(), s)))
            return rc;
        if ((rc = Ops<T>::lhs(lhs, n, nsurf, dims.data(), ccol.data(), cnor.data(), cverts.data(), cwake.data(), 1, sigma, s)))
            return rc;
        return Ops<T>::factor(lu, lhs, n, s);
    }

    // Right-hand side for the free stream fs, the solve, the circulation
    // update and the loads (vlm.cpp:115-151) on the factored AIC.
    int solve_loads(const T* fs, const T* la, T rho, const T* tr, const double* ref_pt, gbvlm_coeffs* out,
                    double* gamma_out, gbvlm_stream s, cudaStream_t st) {
        GB_CUDA(cudaMemsetAsync(rhs, 0, sizeof(T) * n, st));
        std::vector<const T*> cnor(normals.begin(), normals.end()), cvel(vel.begin(), vel.end());
        int rc;
        for (int m = 0; m < nsurf; m++) {
            int64_t np = dims[m].ns * dims[m].nc;
            k_fill3<T><<<(unsigned)cdiv(np, 256), 256, 0, st>>>(vel[m], np, fs[0], fs[1], fs[2]);
            GB_LAUNCH_CHECK();
        }
        if ((rc = Ops<T>::rhsv(rhs, nsurf, dims.data(), cnor.data(), cvel.data(), s))) return rc;
        if ((rc = Ops<T>::solve(lu, lhs, n, rhs, s))) return rc;
        int64_t off = 0;
        for (int m = 0; m < nsurf; m++) {
            if ((rc = Ops<T>::gupd(dims[m].ns, dims[m].nc, rhs + off, gamma[m], gdelta[m], gwake[m], s))) return rc;
            if ((rc = Ops<T>::forces(dims[m].ns, dims[m].nc, verts[m], gdelta[m], vel[m], forces[m], s))) return rc;
            off += dims[m].ns * dims[m].nc;
        }
        // coefficient reductions (vlm_backend.cpp:72-139) + Trefftz drag
        // the wing sits displaced by the wake translation; move the moment
        // reference with it so CM is the body-frame moment about ref_pt
        T ref[3] = {(T)(ref_pt ? ref_pt[0] : 0) + tr[12], (T)(ref_pt ? ref_pt[1] : 0) + tr[13],
                    (T)(ref_pt ? ref_pt[2] : 0) + tr[14]};
        T cl = 0, ta = 0, tm = 0, cdn = 0;
        T cm[3] = {0, 0, 0};
        for (int m = 0; m < nsurf; m++) {
            int64_t ns = dims[m].ns, nc = dims[m].nc;
            T area, clm, mac, cmm[3], cdm;
            if ((rc = Ops<T>::sum(areas[m], ns * nc, &area, s))) return rc;
            if ((rc = Ops<T>::cl(ns, nc, forces[m], la, fs, rho, area, &clm, s))) return rc;
            if ((rc = Ops<T>::mac(ns, nc, verts[m], areas[m], &mac, s))) return rc;
            if ((rc = Ops<T>::cm(ns, nc, forces[m], verts[m], ref, fs, rho, area, mac, cmm, s))) return rc;
            if ((rc = Ops<T>::cd(ns, 2, wake[m], gwake[m], fs, area, sigma, &cdm, s))) return rc;
            cl += clm * area;
            cdn += cdm * area;
            for (int k = 0; k < 3; k++) cm[k] += cmm[k] * area * mac;
            ta += area;
            tm += mac;
        }
        out->cl = (double)(cl / ta);
        out->cdi = (double)(cdn / ta);
        for (int k = 0; k < 3; k++) out->cm[k] = (double)(cm[k] / (ta * tm));
        if (gamma_out) {
            std::vector<T> h(n);
            GB_CUDA(cudaMemcpyAsync(h.data(), rhs, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
            GB_CUDA(cudaStreamSynchronize(st));
            for (int64_t i = 0; i < n; i++) gamma_out[i] = (double)h[i];
        }
        return lu_solve_check(lu, st);  // the solve finished its bounded waits
    }

    int run(double alpha_d, double beta_d, double u_inf_d, double rho_d, const double* ref_pt, gbvlm_coeffs* out,
            double* gamma_out, cudaStream_t st) override {
        gbvlm_stream s = (gbvlm_stream)st;
        const T alpha = (T)alpha_d, beta = (T)beta_d, u = (T)u_inf_d, rho = (T)rho_d;
        T fs[3], la[3], tr[16];
        flow(alpha, beta, u, fs, la);
        int rc = assemble(alpha, u, tr, s, st);
        if (rc) return rc;
        return solve_loads(fs, la, rho, tr, ref_pt, out, gamma_out, s, st);
    }

    int run_shared(int32_t nalpha, const double* alphas, double u_inf_d, double rho_d, const double* ref_pt,
                   gbvlm_coeffs* out, double* gamma_out, cudaStream_t st) override {
        gbvlm_stream s = (gbvlm_stream)st;
        const T u = (T)u_inf_d, rho = (T)rho_d;
        T tr[16];
        int rc = assemble((T)0, u, tr, s, st);
        if (rc) return rc;
        for (int32_t k = 0; k < nalpha; k++) {
            T fs[3], la[3];
            flow((T)alphas[k], (T)0, u, fs, la);
            rc = solve_loads(fs, la, rho, tr, ref_pt, out + k, gamma_out ? gamma_out + (int64_t)k * n : nullptr, s, st);
            if (rc) return rc;
        }
        return GBVLM_OK;
    }
};

// ---------------------------------------------------------------------------
// Nonlinear VLM (vlm/src/vlm.cpp:153-295): strip-wise correction of the
// angle of attack toward a 2D lift polar (van Dam's method).  The AIC of the
// wing with its 100-chord wake row is factored once; each iteration runs on
// the device (panel velocities from the strip angles, RHS, solve, gamma
// deltas, forces, strip correction) and the host reads one error per
// surface to decide whether to continue, as the reference's loop does.
// ---------------------------------------------------------------------------

// Akima interpolant (headeronly/tinyinterpolate.hpp:26-73): lower_bound on
// x, the cubic of that interval, the end segment's line outside the table
template <class T>
__device__ T akima_at(const T* x, const T* y, const T* m, const T* s, int n, T xq) {
    int lo = 0, hi = n;  // first index with x[i] >= xq
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (x[mid] < xq) lo = mid + 1;
        else hi = mid;
    }
    if (lo == 0) return y[0] - m[0] * (x[0] - xq);
    if (lo == n) return y[n - 1] + m[n - 2] * (xq - x[n - 1]);
    const int i = lo - 1;
    const T dx = x[i + 1] - x[i], dxx = xq - x[i];
    const T c = ((T)3 * m[i] - (T)2 * s[i] - s[i + 1]) / dx;
    const T d = (s[i] + s[i + 1] - (T)2 * m[i]) / (dx * dx);
    return y[i] + s[i] * dxx + c * dxx * dxx + d * dxx * dxx * dxx;
}

// panel velocities of a surface from its strip angles (vlm.cpp:186-196:
// freestream(u_inf, alpha_strip, 0), one value per spanwise strip)
template <class T>
__global__ void k_strip_vel(T* vel, const T* strip, int64_t ns, int64_t nc, T u) {
    const int64_t np = ns * nc, p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= np) return;
    const T a = strip[p % ns];
    vel[p] = u * cos(a);
    vel[np + p] = (T)0;
    vel[2 * np + p] = u * sin(a);
}

// one CTA per surface: for every spanwise strip its CL about the strip's own
// lift axis, the effective angle and the correction toward the polar
// (vlm.cpp:257-276); err_out = the surface's sum of |correction|
template <class T>
__global__ void __launch_bounds__(256) k_strip_correct(T* strip, const T* forces, const T* areas, int64_t ns, int64_t nc,
                                                       T alpha, T beta, T u, T rho, const T* tx, const T* ty,
                                                       const T* tm, const T* ts, int ntab, double* err_out) {
    __shared__ double red[256];
    const int64_t np = ns * nc;
    const T two_pi = (T)(2.0f * 3.141593f);  // 2 PI_f with the reference's float pi (vlm_types.hpp:22)
    double e = 0;
    for (int64_t i = threadIdx.x; i < ns; i += blockDim.x) {
        const T a = strip[i];
        // FlowData of the strip (vlm_utils.cpp:5-19): freestream and lift axis
        const T fx = u * cos(a) * cos(beta), fy = -(u * cos(a) * sin(beta)), fz = u * sin(a);
        T lx = -fz, lz = fx;
        const T ll = sqrt(lx * lx + lz * lz);
        lx /= ll;
        lz /= ll;
        T fl = 0, area = 0;
        for (int64_t j = 0; j < nc; j++) {
            const int64_t p = i + j * ns;
            fl += forces[p] * lx + forces[2 * np + p] * lz;  // the lift axis has no y component
            area += areas[p];
        }
        const T cl = fl / ((T)0.5 * rho * (fx * fx + fy * fy + fz * fz) * area);
        const T eff = cl / two_pi - a + alpha;
        const T corr = (akima_at<T>(tx, ty, tm, ts, ntab, eff) - cl) / two_pi;
        strip[i] = a + corr;
        e += fabs((double)corr);
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *err_out = red[0];
}

struct NlvlmBase {
    virtual ~NlvlmBase() = default;
    virtual int run(double alpha, double beta, double u_inf, double rho, const float* db_alpha, const float* db_cl,
                    int32_t ndb, double tol, int32_t max_iter, double* cl, int32_t* iters, double* err,
                    float* strip_out, cudaStream_t st) = 0;
};

template <class T>
struct NlvlmState : NlvlmBase {
    VlmState<T> w;  // wing, wake, AIC and per-panel buffers of the steady simulation
    void* mem = nullptr;
    std::vector<T*> strip;
    double* d_err = nullptr;
    T* tab = nullptr;  // x, y, m, s of the polar
    int32_t tab_cap = 0;

    ~NlvlmState() override {
        if (mem) cudaFree(mem);
        if (tab) cudaFree(tab);
    }

    int init(int32_t ns_, const gbvlm_dims* d, const float* const* vinit) {
        int rc = w.init(ns_, d, vinit);
        if (rc) return rc;
        int64_t strips = 0;
        for (auto& x : w.dims) strips += x.ns;
        GB_CUDA(cudaMalloc(&mem, sizeof(T) * strips + sizeof(double) * w.nsurf + 256));
        d_err = (double*)mem;
        T* p = (T*)((char*)mem + ((sizeof(double) * w.nsurf + 255) / 256) * 256);
        for (auto& x : w.dims) {
            strip.push_back(p);
            p += x.ns;
        }
        return GBVLM_OK;
    }

    int run(double alpha_d, double beta_d, double u_inf_d, double rho_d, const float* db_alpha, const float* db_cl,
            int32_t ndb, double tol, int32_t max_iter, double* cl_out, int32_t* iters_out, double* err_out,
            float* strip_out, cudaStream_t st) override {
        gbvlm_stream s = (gbvlm_stream)st;
        const int32_t nsurf = w.nsurf;
        const T alpha = (T)alpha_d, beta = (T)beta_d, u = (T)u_inf_d, rho = (T)rho_d;
        // the polar's Akima coefficients (tinyinterpolate.hpp:29-54), as the reference builds them on the host
        std::vector<T> tx(ndb), ty(ndb), tm(ndb - 1), ts(ndb);
        for (int i = 0; i < ndb; i++) {
            tx[i] = (T)db_alpha[i];
            ty[i] = (T)db_cl[i];
            GB_REQUIRE(i == 0 || tx[i] > tx[i - 1], "NLVLM: polar angles must increase");
        }
        for (int i = 0; i + 1 < ndb; i++) tm[i] = (ty[i + 1] - ty[i]) / (tx[i + 1] - tx[i]);
        ts[0] = tm[0];
        ts[1] = (T)0.5 * (tm[0] + tm[1]);
        for (int i = 2; i < ndb - 2; i++) {
            const T d1 = std::abs(tm[i + 1] - tm[i]), d2 = std::abs(tm[i - 1] - tm[i - 2]);
            ts[i] = d1 + d2 > (T)0 ? (d1 * tm[i - 1] + d2 * tm[i]) / (d1 + d2) : (T)0.5 * (tm[i] + tm[i - 1]);
        }
        ts[ndb - 2] = (T)0.5 * (tm[ndb - 3] + tm[ndb - 2]);
        ts[ndb - 1] = tm[ndb - 2];
        if (tab_cap < ndb) {
            if (tab) cudaFree(tab);
            tab = nullptr;
            GB_CUDA(cudaMalloc(&tab, sizeof(T) * 4 * ndb));
            tab_cap = ndb;
        }
        T* dx = tab;
        T* dy = tab + ndb;
        T* dm = tab + 2 * ndb;
        T* dsp = tab + 3 * ndb;
        GB_CUDA(cudaMemcpyAsync(dx, tx.data(), sizeof(T) * ndb, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(dy, ty.data(), sizeof(T) * ndb, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(dm, tm.data(), sizeof(T) * (ndb - 1), cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(dsp, ts.data(), sizeof(T) * ndb, cudaMemcpyHostToDevice, st));
        // the wing with its 100-chord wake row and the factored AIC (vlm.cpp:201-217)
        GB_CUDA(cudaMemsetAsync(w.lhs, 0, sizeof(T) * w.n * w.n, st));
        for (int m = 0; m < nsurf; m++) {
            const int64_t nv = (w.dims[m].ns + 1) * (w.dims[m].nc + 1);
            GB_CUDA(cudaMemcpyAsync(w.verts[m], w.verts_init[m], sizeof(T) * 4 * nv, cudaMemcpyDeviceToDevice, st));
        }
        T tr[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, (T)-100 * u * (T)cos(alpha), 0, (T)-100 * u * (T)sin(alpha), 1};
        for (int m = 0; m < nsurf; m++)
            GB_CUDA(cudaMemcpyAsync(w.transform[m], tr, sizeof(tr), cudaMemcpyHostToDevice, st));
        std::vector<const T*> cverts(w.verts.begin(), w.verts.end()), cinit(w.verts_init.begin(), w.verts_init.end()),
            ctr(w.transform.begin(), w.transform.end()), ccol(w.colloc.begin(), w.colloc.end()),
            cnor(w.normals.begin(), w.normals.end()), cwake(w.wake.begin(), w.wake.end()),
            cvel(w.vel.begin(), w.vel.end());
        int rc;
        if ((rc = Ops<T>::shed(nsurf, w.dims.data(), cverts.data(), w.wake.data(), 0, s))) return rc;
        if ((rc = Ops<T>::displace(nsurf, w.dims.data(), ctr.data(), w.verts.data(), cinit.data(), s))) return rc;
        if ((rc = Ops<T>::shed(nsurf, w.dims.data(), cverts.data(), w.wake.data(), 1, s))) return rc;
        if ((rc = Ops<T>::metrics(alpha, nsurf, w.dims.data(), cverts.data(), w.colloc.data(), w.normals.data(),
                                  w.areas.data(), s)))
            return rc;
        if ((rc = Ops<T>::lhs(w.lhs, w.n, nsurf, w.dims.data(), ccol.data(), cnor.data(), cverts.data(),
                              cwake.data(), 1, (T)0, s)))
            return rc;
        if ((rc = Ops<T>::factor(w.lu, w.lhs, w.n, s))) return rc;
        for (int m = 0; m < nsurf; m++) {
            std::vector<T> a0(w.dims[m].ns, alpha);
            GB_CUDA(cudaMemcpyAsync(strip[m], a0.data(), sizeof(T) * a0.size(), cudaMemcpyHostToDevice, st));
            GB_CUDA(cudaStreamSynchronize(st));  // a0 goes out of scope
        }
        auto velocities = [&]() -> int {
            for (int m = 0; m < nsurf; m++) {
                const int64_t np = w.dims[m].ns * w.dims[m].nc;
                k_strip_vel<T><<<(unsigned)cdiv(np, 256), 256, 0, st>>>(w.vel[m], strip[m], w.dims[m].ns,
                                                                        w.dims[m].nc, u);
                GB_LAUNCH_CHECK();
            }
            return GBVLM_OK;
        };
        std::vector<double> herr(nsurf);
        double err = 1.0;
        int32_t it = 0;
        for (; it < max_iter && err > tol; it++) {
            if ((rc = velocities())) return rc;
            GB_CUDA(cudaMemsetAsync(w.rhs, 0, sizeof(T) * w.n, st));
            if ((rc = Ops<T>::rhsv(w.rhs, nsurf, w.dims.data(), cnor.data(), cvel.data(), s))) return rc;
            if ((rc = Ops<T>::solve(w.lu, w.lhs, w.n, w.rhs, s))) return rc;
            int64_t off = 0;
            for (int m = 0; m < nsurf; m++) {
                const int64_t ns = w.dims[m].ns, nc = w.dims[m].nc;
                if ((rc = Ops<T>::gupd(ns, nc, w.rhs + off, w.gamma[m], w.gdelta[m], w.gwake[m], s))) return rc;
                if ((rc = Ops<T>::forces(ns, nc, w.verts[m], w.gdelta[m], w.vel[m], w.forces[m], s))) return rc;
                k_strip_correct<T><<<1, 256, 0, st>>>(strip[m], w.forces[m], w.areas[m], ns, nc, alpha, beta, u, rho,
                                                      dx, dy, dm, dsp, ndb, d_err + m);
                GB_LAUNCH_CHECK();
                off += ns * nc;
            }
            GB_CUDA(cudaMemcpyAsync(herr.data(), d_err, sizeof(double) * nsurf, cudaMemcpyDeviceToHost, st));
            GB_CUDA(cudaStreamSynchronize(st));
            err = 0;
            for (int m = 0; m < nsurf; m++) err += herr[m];
            err /= (double)w.n;  // per panel, as the reference normalises
        }
        if (strip_out) {
            int64_t o = 0;
            for (int m = 0; m < nsurf; m++) {
                std::vector<T> h(w.dims[m].ns);
                GB_CUDA(cudaMemcpyAsync(h.data(), strip[m], sizeof(T) * h.size(), cudaMemcpyDeviceToHost, st));
                GB_CUDA(cudaStreamSynchronize(st));
                for (auto v : h) strip_out[o++] = (float)v;
            }
        }
        // final loads with the strips back at alpha (vlm.cpp:281-291)
        for (int m = 0; m < nsurf; m++) {
            std::vector<T> a0(w.dims[m].ns, alpha);
            GB_CUDA(cudaMemcpyAsync(strip[m], a0.data(), sizeof(T) * a0.size(), cudaMemcpyHostToDevice, st));
            GB_CUDA(cudaStreamSynchronize(st));
        }
        if ((rc = velocities())) return rc;
        T fs[3] = {u * (T)cos(alpha) * (T)cos(beta), -(u * (T)cos(alpha) * (T)sin(beta)), u * (T)sin(alpha)};
        T la[3] = {-fs[2], (T)0, fs[0]};
        const T ll = (T)sqrt(la[0] * la[0] + la[2] * la[2]);
        la[0] /= ll;
        la[2] /= ll;
        T cl = 0, ta = 0;
        for (int m = 0; m < nsurf; m++) {
            const int64_t ns = w.dims[m].ns, nc = w.dims[m].nc;
            if ((rc = Ops<T>::forces(ns, nc, w.verts[m], w.gdelta[m], w.vel[m], w.forces[m], s))) return rc;
            T area, clm;
            if ((rc = Ops<T>::sum(w.areas[m], ns * nc, &area, s))) return rc;
            if ((rc = Ops<T>::cl(ns, nc, w.forces[m], la, fs, rho, area, &clm, s))) return rc;
            cl += clm * area;
            ta += area;
        }
        *cl_out = (double)(cl / ta);
        if (iters_out) *iters_out = it;
        if (err_out) *err_out = err;
        return GBVLM_OK;
    }
};

}  // namespace gbvlm

using namespace gbvlm;

struct gbvlm_vlm_s {
    VlmBase* impl = nullptr;
};

struct gbvlm_nlvlm_s {
    NlvlmBase* impl = nullptr;
};

extern "C" {

int gbvlm_vlm_create(gbvlm_vlm* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                     int32_t precision) {
    GB_REQUIRE(out && dims && verts_init, "null argument");
    GB_REQUIRE(nsurf >= 1 && nsurf <= GBVLM_MAX_SURFACES, "nsurf=%d outside [1, %d]", nsurf, GBVLM_MAX_SURFACES);
    GB_REQUIRE(precision == 32 || precision == 64, "precision must be 32 or 64");
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(verts_init[m], "verts_init[%d] is null", m);
        GB_REQUIRE(dims[m].ns >= 1 && dims[m].nc >= 1, "surface %d has bad sizes", m);
    }
    auto* h = new gbvlm_vlm_s();
    int rc;
    if (precision == 32) {
        auto* s = new VlmState<float>();
        h->impl = s;
        rc = s->init(nsurf, dims, verts_init);
    } else {
        auto* s = new VlmState<double>();
        h->impl = s;
        rc = s->init(nsurf, dims, verts_init);
    }
    if (rc) {
        delete h->impl;
        delete h;
        return rc;
    }
    *out = h;
    return GBVLM_OK;
}

int gbvlm_vlm_destroy(gbvlm_vlm h) {
    if (!h) return GBVLM_OK;
    delete h->impl;
    delete h;
    return GBVLM_OK;
}

int gbvlm_vlm_run(gbvlm_vlm h, double alpha, double beta, double u_inf, double rho, const double* ref_pt,
                  gbvlm_coeffs* out, double* gamma_out, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl && out, "null argument");
    return h->impl->run(alpha, beta, u_inf, rho, ref_pt, out, gamma_out, to_cuda(stream));
}

int gbvlm_vlm_run_shared(gbvlm_vlm h, int32_t nalpha, const double* alphas, double u_inf, double rho,
                         const double* ref_pt, gbvlm_coeffs* out, double* gamma_out, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl && out && alphas, "null argument");
    GB_REQUIRE(nalpha >= 1, "nalpha=%d < 1", nalpha);
    return h->impl->run_shared(nalpha, alphas, u_inf, rho, ref_pt, out, gamma_out, to_cuda(stream));
}

int gbvlm_nlvlm_create(gbvlm_nlvlm* out, int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_init,
                       int32_t precision) {
    GB_REQUIRE(out && dims && verts_init, "null argument");
    GB_REQUIRE(nsurf >= 1 && nsurf <= GBVLM_MAX_SURFACES, "nsurf=%d outside [1, %d]", nsurf, GBVLM_MAX_SURFACES);
    GB_REQUIRE(precision == 32 || precision == 64, "precision must be 32 or 64");
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(verts_init[m], "verts_init[%d] is null", m);
        GB_REQUIRE(dims[m].ns >= 1 && dims[m].nc >= 1, "surface %d has bad sizes", m);
    }
    auto* h = new gbvlm_nlvlm_s();
    int rc;
    if (precision == 32) {
        auto* st = new NlvlmState<float>();
        h->impl = st;
        rc = st->init(nsurf, dims, verts_init);
    } else {
        auto* st = new NlvlmState<double>();
        h->impl = st;
        rc = st->init(nsurf, dims, verts_init);
    }
    if (rc) {
        delete h->impl;
        delete h;
        return rc;
    }
    *out = h;
    return GBVLM_OK;
}

int gbvlm_nlvlm_destroy(gbvlm_nlvlm h) {
    if (!h) return GBVLM_OK;
    delete h->impl;
    delete h;
    return GBVLM_OK;
}

int gbvlm_nlvlm_run(gbvlm_nlvlm h, double alpha, double beta, double u_inf, double rho, const float* db_alpha,
                    const float* db_cl, int32_t n_db, double tol, int32_t max_iter, double* cl, int32_t* iters,
                    double* err, float* strip_alpha, gbvlm_stream stream) {
    GB_REQUIRE(h && h->impl && db_alpha && db_cl && cl, "null argument");
    GB_REQUIRE(n_db >= 4, "NLVLM: the polar needs at least 4 points (Akima), got %d", n_db);
    GB_REQUIRE(max_iter >= 0, "NLVLM: max_iter must be non-negative");
    return h->impl->run(alpha, beta, u_inf, rho, db_alpha, db_cl, n_db, tol, max_iter, cl, iters, err, strip_alpha,
                        to_cuda(stream));
}

int gbvlm_read_plot3d(const char* path, int32_t quarter_chord, gbvlm_dims* dims, float* verts) {
    GB_REQUIRE(path && dims, "null argument");
    std::ifstream f(path);
    if (!f.is_open()) {
        set_error("Failed to open mesh file %s", path);
        return GBVLM_ERR_IO;
    }
    long long blocks = 0, ni = 0, nj = 0, nk = 0;
    f >> blocks;
    if (blocks != 1) {
        set_error("Only single block plot3d mesh is supported");
        return GBVLM_ERR_IO;
    }
    f >> ni >> nj >> nk;
    if (nk != 1 || ni < 2 || nj < 2 || !f) {
        set_error("Only 2D plot3d mesh is supported");
        return GBVLM_ERR_IO;
    }
    dims->nc = ni - 1;
    dims->ns = nj - 1;
    dims->nwv = 0;
    if (!verts) return GBVLM_OK;
    // reference tensor (nj, ni, 4): span index fastest (vlm_mesh.cpp:61-78)
    const int64_t nv = ni * nj;
    for (int k = 0; k < 3; k++) {
        for (long long j = 0; j < nj; j++) {
            for (long long i = 0; i < ni; i++) {
                double x;
                if (!(f >> x)) {
                    set_error("plot3d file %s ended early", path);
                    return GBVLM_ERR_IO;
                }
                verts[k * nv + j + i * nj] = (float)x;
            }
        }
    }
    for (int64_t q = 0; q < nv; q++) verts[3 * nv + q] = 1.0f;
    const float first_y = verts[nv];
    for (long long i = 1; i < ni; i++) {
        if (verts[nv + i * nj] != first_y) {
            set_error("Mesh vertices should be ordered in chordwise direction");
            return GBVLM_ERR_IO;
        }
    }
    if (quarter_chord) {
        // vlm_mesh.cpp:16-32
        for (long long i = 0; i + 1 < ni; i++)
            for (long long j = 0; j < nj; j++)
                for (int k = 0; k < 3; k++) {
                    float* a = &verts[k * nv + j + i * nj];
                    a[0] = 0.75f * a[0] + 0.25f * a[nj];
                }
        const long long i = ni - 2;
        for (long long j = 0; j < nj; j++)
            for (int k = 0; k < 3; k++) {
                float* a = &verts[k * nv + j + i * nj];
                a[nj] = (4.f / 3.f) * a[nj] - (1.f / 3.f) * a[0];
            }
    }
    return GBVLM_OK;
}

}  // extern "C"
