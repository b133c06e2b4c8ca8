// BackendGB300: vlm::Backend over the gbvlm C ABI (see vlm_backend_gb300.hpp).
#include "vlm_backend_gb300.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbvlm.h"

using namespace vlm;

namespace {

// The reference's error convention: print and exit (vlm_backend_cuda.cu:21-29).
void check(int rc, const char* what) {
    if (rc != GBVLM_OK) {
        std::fprintf(stderr, "gbvlm error in %s: %s\n", what, gbvlm_last_error());
        std::exit(EXIT_FAILURE);
    }
}
#define GB(call) check((call), #call)

constexpr gbvlm_stream kStream = nullptr;  // the legacy default stream, like BackendCUDA's kernels

template <class V>
gbvlm_dims panel_dims(const V& panels, int64_t nwv = 0) {
    return gbvlm_dims{panels.shape(0), panels.shape(1), nwv};
}

template <class T>
struct Ptrs {
    std::vector<T*> p;
    template <class MV>
    explicit Ptrs(const MV& views) {
        for (const auto& v : views) p.push_back(v.ptr());
    }
    T* const* get() const { return p.data(); }
    const T* const* cget() const { return const_cast<const T* const*>(p.data()); }
};

// ---- precision dispatch onto the f32 / f64 entry points ---------------------
template <class T>
struct Abi;

#define GB_ABI(T, sfx)                                                                                           \
    template <>                                                                                                  \
    struct Abi<T> {                                                                                              \
        static int lhs(T* a, int64_t ld, int32_t ns, const gbvlm_dims* d, const T* const* c, const T* const* n,   \
                       const T* const* vw, const T* const* vk, int32_t it, T s) {                                \
            return gbvlm_lhs_assemble_##sfx(a, ld, ns, d, c, n, vw, vk, it, s, kStream);                         \
        }                                                                                                        \
        static int rhsv(T* r, int32_t ns, const gbvlm_dims* d, const T* const* n, const T* const* v) {          \
            return gbvlm_rhs_assemble_velocities_##sfx(r, ns, d, n, v, kStream);                                 \
        }                                                                                                        \
        static int wake(T* r, int32_t ns, const gbvlm_dims* d, const T* const* g, const T* const* c,             \
                        const T* const* n, const T* const* w, const int32_t* l, int32_t it, T s) {               \
            return gbvlm_rhs_assemble_wake_influence_##sfx(r, ns, d, g, c, n, w, l, it, s, kStream);             \
        }                                                                                                        \
        static int fsteady(int64_t ns, int64_t nc, const T* v, const T* g, const T* u, T* f) {                  \
            return gbvlm_forces_steady_##sfx(ns, nc, v, g, u, f, kStream);                                       \
        }                                                                                                        \
        static int funsteady(int64_t ns, int64_t nc, const T* v, const T* g, const T* gd, const T* u,           \
                             const T* a, const T* n, T* f) {                                                      \
            return gbvlm_forces_unsteady_##sfx(ns, nc, v, g, gd, u, a, n, f, kStream);                           \
        }                                                                                                        \
        static int cl(int64_t ns, int64_t nc, const T* f, const T* la, const T* fs, T rho, T area, T* out) {    \
            return gbvlm_coeff_cl_##sfx(ns, nc, f, la, fs, rho, area, out, kStream);                             \
        }                                                                                                        \
        static int cm(int64_t ns, int64_t nc, const T* f, const T* v, const T* rp, const T* fs, T rho, T area,  \
                      T mac, T* out) {                                                                           \
            return gbvlm_coeff_cm_##sfx(ns, nc, f, v, rp, fs, rho, area, mac, out, kStream);                     \
        }                                                                                                        \
        static int metrics(T a, int32_t ns, const gbvlm_dims* d, const T* const* v, T* const* c, T* const* n,   \
                           T* const* ar) {                                                                       \
            return gbvlm_mesh_metrics_##sfx(a, ns, d, v, c, n, ar, kStream);                                     \
        }                                                                                                        \
        static int mac(int64_t ns, int64_t nc, const T* v, const T* a, T* out) {                                \
            return gbvlm_mesh_mac_##sfx(ns, nc, v, a, out, kStream);                                             \
        }                                                                                                        \
        static int gwake(T* g, int64_t ns, int64_t ncols, const T* co, int32_t h, T tn, T om, T dt, int64_t it) { \
            return gbvlm_gamma_wake_from_coeffs_##sfx(g, ns, ncols, co, h, tn, om, dt, it, kStream);             \
        }                                                                                                        \
        static int sum2d(const T* x, int64_t m, int64_t n, int64_t s0, int64_t s1, T* out) {                     \
            return gbvlm_sum2d_##sfx(x, m, n, s0, s1, out, kStream);                                             \
        }                                                                                                        \
        static int fill(int32_t loc, T* p, int64_t s, T v, int64_t n) {                                          \
            return gbvlm_mem_fill_##sfx(loc, p, s, v, n, kStream);                                               \
        }                                                                                                        \
        static int factor(gbvlm_lu h, T* a, int64_t n, int64_t ld) { return gbvlm_lu_factor_##sfx(h, a, n, ld, kStream); } \
        static int solve(gbvlm_lu h, const T* a, int64_t n, int64_t ld, T* x, int64_t ldx, int64_t nrhs) {       \
            return gbvlm_lu_solve_##sfx(h, a, n, ld, x, ldx, nrhs, kStream);                                     \
        }                                                                                                        \
        static int gemv(int32_t t, int64_t m, int64_t n, T al, const T* a, int64_t lda, const T* x, int64_t ix,  \
                        T be, T* y, int64_t iy) {                                                                \
            return gbvlm_blas_gemv_##sfx(t, m, n, al, a, lda, x, ix, be, y, iy, kStream);                        \
        }                                                                                                        \
        static int gemm(int32_t ta, int32_t tb, int64_t m, int64_t n, int64_t k, T al, const T* a, int64_t lda,  \
                        const T* b, int64_t ldb, T be, T* c, int64_t ldc) {                                      \
            return gbvlm_blas_gemm_##sfx(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc, kStream);              \
        }                                                                                                        \
        static int axpy2d(int64_t m, int64_t n, T al, const T* x, int64_t xs0, int64_t xs1, T* y, int64_t ys0,   \
                          int64_t ys1) {                                                                         \
            return gbvlm_blas_axpy2d_##sfx(m, n, al, x, xs0, xs1, y, ys0, ys1, kStream);                         \
        }                                                                                                        \
        static int scal(int64_t n, T al, T* x, int64_t ix) { return gbvlm_blas_scal_##sfx(n, al, x, ix, kStream); } \
        static int nrm2(int64_t n, const T* x, int64_t ix, T* out) {                                             \
            return gbvlm_blas_nrm2_##sfx(n, x, ix, out, kStream);                                                \
        }                                                                                                        \
        static int lsq(int64_t m, int64_t n, T* a, int64_t lda, T* b, int64_t nrhs, int64_t ldb) {               \
            return gbvlm_lsq_solve_##sfx(m, n, a, lda, b, nrhs, ldb, kStream);                                   \
        }                                                                                                        \
    };
GB_ABI(f32, f32)
GB_ABI(f64, f64)

// ---- operator bodies, both precisions ---------------------------------------
template <class T, class TV2, class MV3>
void lhs_impl(TV2& lhs, MV3& colloc, MV3& normals, MV3& verts_wing, MV3& verts_wake, std::vector<i32>& condition,
              i32 iteration, T sigma) {
    std::vector<gbvlm_dims> d;
    for (size_t m = 0; m < colloc.size(); m++)
        d.push_back(panel_dims(colloc[m], verts_wake.size() > m ? verts_wake[m].shape(1) : 0));
    Ptrs<T> c(colloc), n(normals), vw(verts_wing), vk(verts_wake);
    GB(Abi<T>::lhs(lhs.ptr(), lhs.stride(1), (int32_t)d.size(), d.data(), c.cget(), n.cget(), vw.cget(),
                   verts_wake.empty() ? nullptr : vk.cget(), iteration, sigma));
    // the reference's condition counters end at `iteration` for every surface pair (vlm_backend_cpu.cpp:121-139)
    std::fill(condition.begin(), condition.end(), iteration);
}

template <class T, class TV1, class MV3>
void rhsv_impl(TV1& rhs, MV3& normals, MV3& velocities) {
    std::vector<gbvlm_dims> d;
    for (const auto& n : normals) d.push_back(panel_dims(n));
    Ptrs<T> n(normals), v(velocities);
    GB(Abi<T>::rhsv(rhs.ptr(), (int32_t)d.size(), d.data(), n.cget(), v.cget()));
}

template <class T, class TV1, class MV2, class MV3>
void wake_impl(TV1& rhs, MV2& gamma_wake, MV3& colloc, MV3& normals, MV3& verts_wake, std::vector<bool>& lifting,
               i32 iteration, T sigma) {
    std::vector<gbvlm_dims> d;
    std::vector<int32_t> lf;
    for (size_t m = 0; m < normals.size(); m++) {
        d.push_back(panel_dims(normals[m], verts_wake[m].shape(1)));
        lf.push_back(lifting[m] ? 1 : 0);
    }
    Ptrs<T> g(gamma_wake), c(colloc), n(normals), w(verts_wake);
    GB(Abi<T>::wake(rhs.ptr(), (int32_t)d.size(), d.data(), g.cget(), c.cget(), n.cget(), w.cget(), lf.data(),
                    iteration, sigma));
}

template <class T, class MV3, class MV2>
void metrics_impl(T alpha, MV3& verts_wing, MV3& colloc, MV3& normals, MV2& areas) {
    std::vector<gbvlm_dims> d;
    for (const auto& c : colloc) d.push_back(panel_dims(c));
    Ptrs<T> v(verts_wing), c(colloc), n(normals), a(areas);
    GB(Abi<T>::metrics(alpha, (int32_t)d.size(), d.data(), v.cget(), c.get(), n.get(), a.get()));
}

template <class T, class TV2>
T sum2d_impl(TV2& t) {
    T out = 0;
    GB(Abi<T>::sum2d(t.ptr(), t.shape(0), t.shape(1), t.stride(0), t.stride(1), &out));
    return out;
}

template <class T, class TV1>
T sum1d_impl(TV1& t) {
    T out = 0;
    GB(Abi<T>::sum2d(t.ptr(), t.shape(0), 1, t.stride(0), 0, &out));
    return out;
}

// ---- Memory, LU, BLAS, LSQ -------------------------------------------------
class GB300Memory final : public Memory {
public:
    GB300Memory() : Memory(false) {}
    void* alloc(Location location, i64 size) const override {
        void* p = nullptr;
        GB(gbvlm_mem_alloc(location == Location::Device ? GBVLM_LOC_DEVICE : GBVLM_LOC_HOST, size, &p));
        return p;
    }
    void free(Location location, void* ptr) const override {
        GB(gbvlm_mem_free(location == Location::Device ? GBVLM_LOC_DEVICE : GBVLM_LOC_HOST, ptr));
    }
    void copy(Location dst_loc, void* dst, i64 dst_stride, Location src_loc, const void* src, i64 src_stride,
              i64 elem_size, i64 size) const override {
        GB(gbvlm_mem_copy(dst_loc == Location::Device ? GBVLM_LOC_DEVICE : GBVLM_LOC_HOST, dst, dst_stride,
                          src_loc == Location::Device ? GBVLM_LOC_DEVICE : GBVLM_LOC_HOST, src, src_stride, elem_size,
                          size, kStream));
    }
    void fill(Location loc, float* ptr, i64 stride, float value, i64 size) const override {
        GB(Abi<f32>::fill(loc == Location::Device ? GBVLM_LOC_DEVICE : GBVLM_LOC_HOST, ptr, stride, value, size));
    }
    void fill(Location loc, double* ptr, i64 stride, double value, i64 size) const override {
        GB(Abi<f64>::fill(loc == Location::Device ? GBVLM_LOC_DEVICE : GBVLM_LOC_HOST, ptr, stride, value, size));
    }
};

class GB300LU final : public LU {
public:
    explicit GB300LU(std::unique_ptr<Memory> memory) : LU(std::move(memory)) { GB(gbvlm_lu_create(&h_)); }
    ~GB300LU() override {
        if (h_) gbvlm_lu_destroy(h_);
    }
    void init(const TensorView2fD& A) override { GB(gbvlm_lu_init(h_, A.shape(0))); }
    void factorize(const TensorView2fD& A) override { GB(Abi<f32>::factor(h_, A.ptr(), A.shape(0), A.stride(1))); }
    void solve(const TensorView2fD& A, const TensorView2fD& x) override {
        GB(Abi<f32>::solve(h_, A.ptr(), A.shape(1), A.stride(1), x.ptr(), x.stride(1), x.shape(1)));
    }
    void init(const TensorView2dD& A) override { GB(gbvlm_lu_init(h_, A.shape(0))); }
    void factorize(const TensorView2dD& A) override { GB(Abi<f64>::factor(h_, A.ptr(), A.shape(0), A.stride(1))); }
    void solve(const TensorView2dD& A, const TensorView2dD& x) override {
        GB(Abi<f64>::solve(h_, A.ptr(), A.shape(1), A.stride(1), x.ptr(), x.stride(1), x.shape(1)));
    }

private:
    gbvlm_lu h_ = nullptr;
};

class GB300BLAS final : public BLAS {
    template <class T, class TV2, class TV1>
    static void gemv_t(T alpha, const TV2& A, const TV1& x, T beta, const TV1& y, Trans trans) {
        GB(Abi<T>::gemv(trans == Trans::Yes, A.shape(0), A.shape(1), alpha, A.ptr(), A.stride(1), x.ptr(),
                        x.stride(0), beta, y.ptr(), y.stride(0)));
    }
    template <class T, class TV2>
    static void gemm_t(T alpha, const TV2& A, const TV2& B, T beta, const TV2& C, Trans ta, Trans tb) {
        const i64 k = ta == Trans::No ? A.shape(1) : A.shape(0);
        GB(Abi<T>::gemm(ta == Trans::Yes, tb == Trans::Yes, C.shape(0), C.shape(1), k, alpha, A.ptr(), A.stride(1),
                        B.ptr(), B.stride(1), beta, C.ptr(), C.stride(1)));
    }

public:
    void gemv(const f32 alpha, const TensorView2fD& A, const TensorView1fD& x, const f32 beta, const TensorView1fD& y,
              Trans trans) override {
        gemv_t<f32>(alpha, A, x, beta, y, trans);
    }
    void gemm(const f32 alpha, const TensorView2fD& A, const TensorView2fD& B, const f32 beta, const TensorView2fD& C,
              Trans trans_a, Trans trans_b) override {
        gemm_t<f32>(alpha, A, B, beta, C, trans_a, trans_b);
    }
    void axpy(const f32 alpha, const TensorView1fD& x, const TensorView1fD& y) override {
        GB(Abi<f32>::axpy2d(x.shape(0), 1, alpha, x.ptr(), x.stride(0), 0, y.ptr(), y.stride(0), 0));
    }
    void axpy(const f32 alpha, const TensorView2fD& x, const TensorView2fD& y) override {
        GB(Abi<f32>::axpy2d(x.shape(0), x.shape(1), alpha, x.ptr(), x.stride(0), x.stride(1), y.ptr(), y.stride(0),
                            y.stride(1)));
    }
    void scal(const f32 alpha, const TensorView1fD& x) override {
        GB(Abi<f32>::scal(x.shape(0), alpha, x.ptr(), x.stride(0)));
    }
    f32 norm(const TensorView1fD& x) override {
        f32 out = 0;
        GB(Abi<f32>::nrm2(x.shape(0), x.ptr(), x.stride(0), &out));
        return out;
    }
    void gemv(const f64 alpha, const TensorView2dD& A, const TensorView1dD& x, const f64 beta, const TensorView1dD& y,
              Trans trans) override {
        gemv_t<f64>(alpha, A, x, beta, y, trans);
    }
    void gemm(const f64 alpha, const TensorView2dD& A, const TensorView2dD& B, const f64 beta, const TensorView2dD& C,
              Trans trans_a, Trans trans_b) override {
        gemm_t<f64>(alpha, A, B, beta, C, trans_a, trans_b);
    }
    void axpy(const f64 alpha, const TensorView1dD& x, const TensorView1dD& y) override {
        GB(Abi<f64>::axpy2d(x.shape(0), 1, alpha, x.ptr(), x.stride(0), 0, y.ptr(), y.stride(0), 0));
    }
    void axpy(const f64 alpha, const TensorView2dD& x, const TensorView2dD& y) override {
        GB(Abi<f64>::axpy2d(x.shape(0), x.shape(1), alpha, x.ptr(), x.stride(0), x.stride(1), y.ptr(), y.stride(0),
                            y.stride(1)));
    }
    void scal(const f64 alpha, const TensorView1dD& x) override {
        GB(Abi<f64>::scal(x.shape(0), alpha, x.ptr(), x.stride(0)));
    }
    f64 norm(const TensorView1dD& x) override {
        f64 out = 0;
        GB(Abi<f64>::nrm2(x.shape(0), x.ptr(), x.stride(0), &out));
        return out;
    }
};

class GB300LSQ final : public LSQ {
public:
    explicit GB300LSQ(std::unique_ptr<Memory> memory) : LSQ(std::move(memory)) {}
    void init(const TensorView2fD&, const TensorView2fD&) override {}  // no workspace to size
    void solve(const TensorView2fD& A, const TensorView2fD& B) override {
        GB(Abi<f32>::lsq(A.shape(0), A.shape(1), A.ptr(), A.stride(1), B.ptr(), B.shape(1), B.stride(1)));
    }
    void init(const TensorView2dD&, const TensorView2dD&) override {}
    void solve(const TensorView2dD& A, const TensorView2dD& B) override {
        GB(Abi<f64>::lsq(A.shape(0), A.shape(1), A.ptr(), A.stride(1), B.ptr(), B.shape(1), B.stride(1)));
    }
};

}  // namespace

// ---- BackendGB300 ------------------------------------------------------------
BackendGB300::BackendGB300() : Backend(std::make_unique<GB300Memory>(), std::make_unique<GB300BLAS>()) {
    name = "GB300";
    int32_t sms = 0;
    int64_t free_b = 0, total_b = 0;
    GB(gbvlm_device_info(&sms, &free_b, &total_b));
    std::printf("DEVICE: GB300 backend, libgbvlm %d (%d SMs, %.1f GB)\n", gbvlm_version(), sms, total_b / 1e9);
}

BackendGB300::~BackendGB300() = default;

std::unique_ptr<Memory> BackendGB300::create_memory_manager() { return std::make_unique<GB300Memory>(); }
std::unique_ptr<LU> BackendGB300::create_lu_solver() { return std::make_unique<GB300LU>(create_memory_manager()); }
std::unique_ptr<BLAS> BackendGB300::create_blas() { return std::make_unique<GB300BLAS>(); }
std::unique_ptr<LSQ> BackendGB300::create_lsq_solver() { return std::make_unique<GB300LSQ>(create_memory_manager()); }

#define GB_OPS(T, TV1, TV2, TV3, MTV2, MTV3, X3)                                                                  \
    void BackendGB300::lhs_assemble(TV2& lhs, MTV3& colloc, MTV3& normals, MTV3& verts_wing, MTV3& verts_wake,    \
                                    std::vector<i32>& condition, i32 iteration) {                                 \
        lhs_impl<T>(lhs, colloc, normals, verts_wing, verts_wake, condition, iteration, (T)sigma_vatistas);       \
    }                                                                                                             \
    void BackendGB300::rhs_assemble_velocities(TV1& rhs, MTV3& normals, MTV3& velocities) {                       \
        rhsv_impl<T>(rhs, normals, velocities);                                                                   \
    }                                                                                                             \
    void BackendGB300::rhs_assemble_wake_influence(TV1& rhs, MTV2& gamma_wake, MTV3& colloc, MTV3& normals,       \
                                                   MTV3& verts_wake, std::vector<bool>& lifting, i32 iteration) { \
        wake_impl<T>(rhs, gamma_wake, colloc, normals, verts_wake, lifting, iteration, (T)sigma_vatistas);        \
    }                                                                                                             \
    void BackendGB300::forces_steady(TV3& verts_wing, TV2& gamma_delta, TV3& velocities, TV3& forces) {           \
        GB(Abi<T>::fsteady(gamma_delta.shape(0), gamma_delta.shape(1), verts_wing.ptr(), gamma_delta.ptr(),       \
                           velocities.ptr(), forces.ptr()));                                                      \
    }                                                                                                             \
    void BackendGB300::forces_unsteady(TV3& verts_wing, TV2& gamma_delta, TV2& dgamma_dt, TV3& velocities,        \
                                       TV2& areas, TV3& normals, TV3& forces) {                                   \
        GB(Abi<T>::funsteady(gamma_delta.shape(0), gamma_delta.shape(1), verts_wing.ptr(), gamma_delta.ptr(),     \
                             dgamma_dt.ptr(), velocities.ptr(), areas.ptr(), normals.ptr(), forces.ptr()));       \
    }                                                                                                             \
    T BackendGB300::coeff_cl(TV3& forces, X3& lift_axis, X3& freestream, T rho, T area) {                         \
        const T la[3] = {lift_axis.x, lift_axis.y, lift_axis.z}, fs[3] = {freestream.x, freestream.y, freestream.z}; \
        T out = 0;                                                                                                \
        GB(Abi<T>::cl(forces.shape(0), forces.shape(1), forces.ptr(), la, fs, rho, area, &out));                  \
        return out;                                                                                               \
    }                                                                                                             \
    BackendGB300::X3 BackendGB300::coeff_cm(TV3& forces, TV3& verts_wing, X3& ref_pt, X3& freestream, T rho, T area, T mac) {   \
        const T rp[3] = {ref_pt.x, ref_pt.y, ref_pt.z}, fs[3] = {freestream.x, freestream.y, freestream.z};       \
        T out[3] = {0, 0, 0};                                                                                     \
        GB(Abi<T>::cm(forces.shape(0), forces.shape(1), forces.ptr(), verts_wing.ptr(), rp, fs, rho, area, mac,   \
                      out));                                                                                      \
        return X3{out[0], out[1], out[2]};                                                                        \
    }                                                                                                             \
    void BackendGB300::mesh_metrics(T alpha_rad, MTV3& verts_wing, MTV3& colloc, MTV3& normals, MTV2& areas) {    \
        metrics_impl<T>(alpha_rad, verts_wing, colloc, normals, areas);                                           \
    }                                                                                                             \
    T BackendGB300::mesh_mac(TV3& verts_wing, TV2& areas) {                                                       \
        T out = 0;                                                                                                \
        GB(Abi<T>::mac(areas.shape(0), areas.shape(1), verts_wing.ptr(), areas.ptr(), &out));                     \
        return out;                                                                                               \
    }                                                                                                             \
    void BackendGB300::gamma_wake_from_coeffs(TV2& gamma_wake, TV2& gamma_coeffs, i32 harmonics, T tn, T omega,   \
                                              T dt, i64 iteration) {                                              \
        GB(Abi<T>::gwake(gamma_wake.ptr(), gamma_wake.shape(0), gamma_wake.shape(1), gamma_coeffs.ptr(),          \
                         harmonics, tn, omega, dt, iteration));                                                   \
    }                                                                                                             \
    T BackendGB300::sum(TV1& tensor) { return sum1d_impl<T>(tensor); }                                            \
    T BackendGB300::sum(TV2& tensor) { return sum2d_impl<T>(tensor); }

GB_OPS(f32, TV1f, TV2f, TV3f, MTV2f, MTV3f, f32x3)
GB_OPS(f64, TV1d, TV2d, TV3d, MTV2d, MTV3d, f64x3)
