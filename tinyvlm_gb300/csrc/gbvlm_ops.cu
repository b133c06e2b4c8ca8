// Per-operator kernels of the vortex-lattice hot path (the vlm::Backend
// operator set) in float and double, and their C-ABI entry points.
//
// Layout contract: see include/gbvlm.h.  Kernels are templated on the
// precision T; the float instantiation keeps the reference's float
// semantics (cut-offs, 5000-row wake window), the double one the reference's
// double kernels (vlm_backend_cpu_kernels.ispc:383-502).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "gbvlm_internal.h"
#include "gbvlm_math.cuh"
#include "gbvlm_walk.cuh"

namespace gbvlm {

// ---------------------------------------------------------------------------
// error state
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), what, file, line);
    return e == cudaErrorMemoryAllocation ? GBVLM_ERR_NOMEM : GBVLM_ERR_CUDA;
}

void* host_scratch(size_t bytes) {
    static thread_local void* p = nullptr;
    static thread_local size_t cap = 0;
    if (bytes > cap) {
        if (p) cudaFreeHost(p);
        cap = bytes < 4096 ? 4096 : bytes;
        if (cudaMallocHost(&p, cap) != cudaSuccess) {
            p = nullptr;
            cap = 0;
        }
    }
    return p;
}

// Scratch for partial sums and small reductions, one buffer per (thread,
// device): calls from different host threads (each with its own stream) never
// share one, and a grow only has to wait for the calling thread's stream.
int device_scratch(size_t bytes, void** out, cudaStream_t s) {
    static thread_local std::vector<std::pair<void*, size_t>> per_dev(64, {nullptr, 0});
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    GB_REQUIRE(dev >= 0 && dev < 64, "device index %d out of range", dev);
    auto& slot = per_dev[dev];
    if (bytes > slot.second) {
        if (slot.first) {
            GB_CUDA(cudaStreamSynchronize(s));
            GB_CUDA(cudaFree(slot.first));
        }
        size_t cap = bytes < (1 << 20) ? (1 << 20) : bytes;
        GB_CUDA(cudaMalloc(&slot.first, cap));
        slot.second = cap;
    }
    *out = slot.first;
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// multi-surface argument table passed by value
// ---------------------------------------------------------------------------
template <class T>
struct Surfs {
    int32_t n;
    int64_t ns[GBVLM_MAX_SURFACES], nc[GBVLM_MAX_SURFACES], nwv[GBVLM_MAX_SURFACES];
    int64_t poff[GBVLM_MAX_SURFACES + 1];  // packed panel offsets
    const T* a[GBVLM_MAX_SURFACES];
    const T* b[GBVLM_MAX_SURFACES];
    const T* c[GBVLM_MAX_SURFACES];
    const T* d[GBVLM_MAX_SURFACES];
    T* o0[GBVLM_MAX_SURFACES];
    T* o1[GBVLM_MAX_SURFACES];
    T* o2[GBVLM_MAX_SURFACES];
    int32_t flag[GBVLM_MAX_SURFACES];
};

template <class T>
static int make_surfs(Surfs<T>& s, int32_t nsurf, const gbvlm_dims* dims) {
    GB_REQUIRE(nsurf >= 1 && nsurf <= GBVLM_MAX_SURFACES, "nsurf=%d outside [1, %d]", nsurf, GBVLM_MAX_SURFACES);
    GB_REQUIRE(dims != nullptr, "dims is null");
    memset(&s, 0, sizeof(s));
    s.n = nsurf;
    s.poff[0] = 0;
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(dims[m].ns >= 1 && dims[m].nc >= 1, "surface %d has ns=%lld nc=%lld", m, (long long)dims[m].ns,
                   (long long)dims[m].nc);
        s.ns[m] = dims[m].ns;
        s.nc[m] = dims[m].nc;
        s.nwv[m] = dims[m].nwv;
        s.poff[m + 1] = s.poff[m] + dims[m].ns * dims[m].nc;
    }
    return GBVLM_OK;
}

template <class T>
__device__ __forceinline__ int find_surf(const Surfs<T>& s, int64_t p) {
    int m = 0;
    while (m + 1 < s.n && p >= s.poff[m + 1]) m++;
    return m;
}

// ---------------------------------------------------------------------------
// a6: mesh metrics (vlm_backend_cpu.cpp:391-433)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_mesh_metrics(Surfs<T> s, T factor) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= s.poff[s.n]) return;
    int m = find_surf(s, g);
    int64_t p = g - s.poff[m], ns = s.ns[m], nc = s.nc[m];
    int64_t i = p % ns, j = p / ns;
    const T* v = s.a[m];
    int64_t vld = (ns + 1) * (nc + 1), np = ns * nc;
    int64_t a = i + j * (ns + 1), b = a + 1, c = b + (ns + 1), d = a + (ns + 1);
    V3<T> v0{v[a], v[vld + a], v[2 * vld + a]}, v1{v[b], v[vld + b], v[2 * vld + b]};
    V3<T> v2{v[c], v[vld + c], v[2 * vld + c]}, v3_{v[d], v[vld + d], v[2 * vld + d]};
    V3<T> nn = cross(v3_ - v1, v2 - v0);
    T l = dsqrt(len2(nn));
    T* col = s.o0[m];
    T* nor = s.o1[m];
    T* ar = s.o2[m];
    nor[p] = nn.x / l;
    nor[np + p] = nn.y / l;
    nor[2 * np + p] = nn.z / l;
    V3<T> f = v3_ - v0, bb = v2 - v0, e = v1 - v0;
    ar[p] = (T)0.5 * (dsqrt(len2(cross(f, bb))) + dsqrt(len2(cross(bb, e))));
    V3<T> ch = (T)0.5 * (((v2 + v3_) - v0) - v1);
    V3<T> cp = (T)0.5 * (v0 + v1) + factor * ch;
    col[p] = cp.x;
    col[np + p] = cp.y;
    col[2 * np + p] = cp.z;
}

template <class T>
static T aoa_factor(T alpha);
template <>
float aoa_factor<float>(float alpha) {
    return (alpha < EPS_F) ? 0.5f : 0.5f * (alpha / (sinf(alpha) + EPS_F));
}
template <>
double aoa_factor<double>(double alpha) {
    return (alpha < (double)EPS_F) ? 0.5 : 0.5 * (alpha / (sin(alpha) + (double)EPS_F));
}

template <class T>
static int mesh_metrics(T alpha, int32_t nsurf, const gbvlm_dims* dims, const T* const* verts, T* const* colloc,
                        T* const* normals, T* const* areas, cudaStream_t st) {
    Surfs<T> s;
    int rc = make_surfs(s, nsurf, dims);
    if (rc) return rc;
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(verts[m] && colloc[m] && normals[m] && areas[m], "null pointer for surface %d", m);
        s.a[m] = verts[m];
        s.o0[m] = colloc[m];
        s.o1[m] = normals[m];
        s.o2[m] = areas[m];
    }
    int64_t n = s.poff[nsurf];
    k_mesh_metrics<T><<<(unsigned)cdiv(n, 256), 256, 0, st>>>(s, aoa_factor<T>(alpha));
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// a1: AIC assembly, one launch per (influenced, influencing) surface pair
// (vlm_backend_cpu.cpp:84-148).  Block = 128 collocation points (one per
// thread, each with its y-mirror) x one chordwise ring row (chunked along
// the span) of the influencing surface; that row's two vertex lines are
// staged in shared memory and read as broadcasts.  Along the span a thread
// keeps the left vertex terms and left chordwise segment of the previous
// ring, so each ring costs two vertex terms and three segment terms per
// evaluation point.
// ---------------------------------------------------------------------------
constexpr int LHS_THREADS = 128;
constexpr int LHS_SCHUNK = 256;

template <class T>
struct LhsPair {
    T* lhs;
    int64_t ld;
    const T* colloc;
    const T* normals;
    int64_t np_i;
    const T* vw;
    int64_t ns, nc;
    const T* vk;
    int64_t nwv;
    int32_t iteration;
    T sigma2;
    int64_t row_off, col_off;
};

template <class T, bool SIGMA>
__global__ void __launch_bounds__(LHS_THREADS) k_lhs_pair(LhsPair<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sv = reinterpret_cast<T*>(smem_raw);
    constexpr int W = LHS_SCHUNK + 1;
    const int64_t c = blockIdx.y;
    const int64_t s0 = (int64_t)blockIdx.z * LHS_SCHUNK;
    const int64_t s1 = min(s0 + (int64_t)LHS_SCHUNK, a.ns);
    const int nv = (int)(s1 - s0 + 1);
    const int64_t vld = (a.ns + 1) * (a.nc + 1);
    for (int t = threadIdx.x; t < 2 * nv; t += blockDim.x) {
        int r = t / nv, sl = t - r * nv;
        int64_t vi = (s0 + sl) + (c + r) * (a.ns + 1);
        sv[(r * 3 + 0) * W + sl] = a.vw[vi];
        sv[(r * 3 + 1) * W + sl] = a.vw[vld + vi];
        sv[(r * 3 + 2) * W + sl] = a.vw[2 * vld + vi];
    }
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * LHS_THREADS + threadIdx.x;
    if (i >= a.np_i) return;
    const T px = a.colloc[i], py = a.colloc[a.np_i + i], pz = a.colloc[2 * a.np_i + i];
    const T nx = a.normals[i], ny = a.normals[a.np_i + i], nz = a.normals[2 * a.np_i + i];
    const T sg = a.sigma2;
    const bool te = (c == a.nc - 1) && a.iteration > 0;
    const int64_t wk_ld = (a.ns + 1) * a.nwv;
    T* out = a.lhs + (a.row_off + i) + (a.col_off + c * a.ns) * a.ld;
    strip_normal<T, SIGMA>(sv, sv + 3 * W, W, nv, px, py, pz, nx, ny, nz, sg, [&](int kk, T val) {
        const int64_t s = s0 + kk;
        if (te) {
            for (int32_t it = 0; it < a.iteration; it++) {
                const int64_t r0 = a.nwv - 2 - it;
                const int64_t i0 = s + r0 * (a.ns + 1), i1 = i0 + 1, i2 = i1 + (a.ns + 1), i3 = i0 + (a.ns + 1);
                V3<T> q[4] = {{a.vk[i0], a.vk[wk_ld + i0], a.vk[2 * wk_ld + i0]},
                              {a.vk[i1], a.vk[wk_ld + i1], a.vk[2 * wk_ld + i1]},
                              {a.vk[i2], a.vk[wk_ld + i2], a.vk[2 * wk_ld + i2]},
                              {a.vk[i3], a.vk[wk_ld + i3], a.vk[2 * wk_ld + i3]}};
                val += ring_normal_full<T, SIGMA>(px, py, pz, nx, ny, nz, q, sg);
            }
        }
        out[s * a.ld] += val * inv_four_pi<T>();
    });
}

template <class T>
static int lhs_assemble(T* lhs, int64_t ld, int32_t nsurf, const gbvlm_dims* dims, const T* const* colloc,
                        const T* const* normals, const T* const* verts_wing, const T* const* verts_wake,
                        int32_t iteration, T sigma, cudaStream_t st) {
    Surfs<T> s;
    int rc = make_surfs(s, nsurf, dims);
    if (rc) return rc;
    GB_REQUIRE(lhs != nullptr, "lhs is null");
    GB_REQUIRE(iteration >= 0, "iteration < 0");
    const int64_t n = s.poff[nsurf];
    GB_REQUIRE(ld >= n, "ld=%lld < n=%lld", (long long)ld, (long long)n);
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(colloc[m] && normals[m] && verts_wing[m], "null pointer for surface %d", m);
        if (iteration > 0) {
            GB_REQUIRE(verts_wake && verts_wake[m], "wake of surface %d is null", m);
            GB_REQUIRE(dims[m].nwv >= iteration + 1, "surface %d: nwv=%lld < iteration+1", m, (long long)dims[m].nwv);
        }
    }
    const size_t smem = 2 * 3 * (LHS_SCHUNK + 1) * sizeof(T);
    for (int mj = 0; mj < nsurf; mj++) {
        for (int mi = 0; mi < nsurf; mi++) {
            LhsPair<T> a;
            a.lhs = lhs;
            a.ld = ld;
            a.colloc = colloc[mi];
            a.normals = normals[mi];
            a.np_i = s.ns[mi] * s.nc[mi];
            a.vw = verts_wing[mj];
            a.ns = s.ns[mj];
            a.nc = s.nc[mj];
            a.vk = iteration > 0 ? verts_wake[mj] : nullptr;
            a.nwv = dims[mj].nwv;
            a.iteration = iteration;
            a.sigma2 = sigma * sigma;
            a.row_off = s.poff[mi];
            a.col_off = s.poff[mj];
            dim3 grid((unsigned)cdiv(a.np_i, LHS_THREADS), (unsigned)a.nc, (unsigned)cdiv(a.ns, LHS_SCHUNK));
            if (sigma != (T)0)
                k_lhs_pair<T, true><<<grid, LHS_THREADS, smem, st>>>(a);
            else
                k_lhs_pair<T, false><<<grid, LHS_THREADS, smem, st>>>(a);
            GB_LAUNCH_CHECK();
        }
    }
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// a2: rhs += -(V . n) (vlm_backend_cpu.cpp:156-179)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_rhs_velocities(Surfs<T> s, T* rhs) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= s.poff[s.n]) return;
    int m = find_surf(s, g);
    int64_t p = g - s.poff[m], np = s.ns[m] * s.nc[m];
    const T* n = s.a[m];
    const T* v = s.b[m];
    rhs[g] += -(v[p] * n[p] + v[np + p] * n[np + p] + v[2 * np + p] * n[2 * np + p]);
}

template <class T>
static int rhs_velocities(T* rhs, int32_t nsurf, const gbvlm_dims* dims, const T* const* normals,
                          const T* const* velocities, cudaStream_t st) {
    Surfs<T> s;
    int rc = make_surfs(s, nsurf, dims);
    if (rc) return rc;
    GB_REQUIRE(rhs != nullptr, "rhs is null");
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(normals[m] && velocities[m], "null pointer for surface %d", m);
        s.a[m] = normals[m];
        s.b[m] = velocities[m];
    }
    int64_t n = s.poff[nsurf];
    k_rhs_velocities<T><<<(unsigned)cdiv(n, 256), 256, 0, st>>>(s, rhs);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// a3: wake influence on the RHS (vlm_backend_cpu.cpp:181-224), N-body tiled.
// Grid x: blocks of 128 target panels (all surfaces packed); grid y: slices
// of the active wake ring rows (split-K).  Each block stages WK_ROWS ring rows
// (vertex lines + gammas) of one lifting wake in shared memory and every
// thread walks them span-wise with the shared vertex/segment chain, keeping
// a scalar sum of gamma_r (v_r . n) for its point and its mirror.  Partial
// sums go to a scratch buffer [slice][target] and a second kernel reduces
// them in a fixed order into rhs, so results do not depend on scheduling.
// ---------------------------------------------------------------------------
constexpr int WK_THREADS = 128;
constexpr int WK_ROWS = 8;
constexpr int WK_MAXSPAN = 512;  // spanwise vertices staged per row chunk

template <class T>
struct WakeArgs {
    Surfs<T> s;          // a=colloc, b=normals (targets); c=verts_wake, d=gamma_wake, flag=lifting
    int32_t iteration;
    int32_t window;      // 0 = no window
    T sigma2;
    int64_t total_rows;  // sum over lifting surfaces of active ring rows
    int64_t rows_per_slice;
    T* partial;          // [slices][n_targets]
    int32_t sc;          // spanwise rings staged per chunk (<= WK_MAXSPAN)
    const int64_t* it_dev;  // if set: the iteration, read on the device (the grid covers up to `iteration`)
};

// number of active ring rows of surface m and the first one
template <class T>
__device__ __forceinline__ void wake_rows(const WakeArgs<T>& w, int m, int64_t& first, int64_t& count) {
    const int64_t v_m = w.s.nwv[m];
    const int64_t it = w.it_dev ? *w.it_dev : w.iteration;
    first = v_m - it - 1;
    int64_t end = v_m - 1;
    if (w.window > 0 && it > w.window) end = v_m - 1 - it + w.window;
    count = end - first;
    if (count < 0) count = 0;
}

template <class T, bool SIGMA>
__global__ void __launch_bounds__(WK_THREADS) k_wake_influence(WakeArgs<T> w) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int SC = w.sc, W = SC + 1;
    T* sv = reinterpret_cast<T*>(smem_raw);  // [(WK_ROWS+1) rows][3][W]
    T* sg = sv + (WK_ROWS + 1) * 3 * W;      // [WK_ROWS][SC]
    const int64_t ntg = w.s.poff[w.s.n];
    const int64_t g = (int64_t)blockIdx.x * WK_THREADS + threadIdx.x;
    const bool active = g < ntg;
    T px = 0, py = 0, pz = 0, nx = 0, ny = 0, nz = 0;
    if (active) {
        int m = find_surf(w.s, g);
        int64_t p = g - w.s.poff[m], np = w.s.ns[m] * w.s.nc[m];
        px = w.s.a[m][p]; py = w.s.a[m][np + p]; pz = w.s.a[m][2 * np + p];
        nx = w.s.b[m][p]; ny = w.s.b[m][np + p]; nz = w.s.b[m][2 * np + p];
    }
    // this block's global row range [R0, R1) over the concatenation of lifting wakes
    int64_t total_rows = w.total_rows;
    if (w.it_dev) {  // rows of the current iteration; slices past them contribute zero
        total_rows = 0;
        for (int m = 0; m < w.s.n; m++)
            if (w.s.flag[m]) {
                int64_t f_, c_;
                wake_rows(w, m, f_, c_);
                total_rows += c_;
            }
    }
    // the device-iteration form spreads the current rows over all its slices
    // (its grid is sized for the largest row count, at capture)
    const int64_t rps = w.it_dev ? max((total_rows + gridDim.y - 1) / gridDim.y, (int64_t)WK_ROWS) : w.rows_per_slice;
    const int64_t R0 = (int64_t)blockIdx.y * rps;
    const int64_t R1 = min(R0 + rps, total_rows);
    T acc = 0;
    int64_t base = 0;
    for (int m = 0; m < w.s.n && base < R1; m++) {
        if (!w.s.flag[m]) continue;
        int64_t first, count;
        wake_rows(w, m, first, count);
        const int64_t lo = max(R0, base), hi = min(R1, base + count);
        if (lo < hi) {
            const int64_t n = w.s.ns[m] + 1;  // spanwise vertices
            const int64_t vld = n * w.s.nwv[m];
            const T* vk = w.s.c[m];
            const T* gk = w.s.d[m];
            for (int64_t sc0 = 0; sc0 < n - 1; sc0 += SC) {
                const int64_t sc1 = min(sc0 + (int64_t)SC, n - 1);  // rings [sc0, sc1)
                const int nvs = (int)(sc1 - sc0 + 1);
                for (int64_t r0 = lo; r0 < hi; r0 += WK_ROWS) {
                    const int nr = (int)min((int64_t)WK_ROWS, hi - r0);
                    const int64_t row0 = first + (r0 - base);  // first ring row of this chunk
                    __syncthreads();
                    for (int t = threadIdx.x; t < (nr + 1) * nvs; t += blockDim.x) {
                        int r = t / nvs, sl = t - r * nvs;
                        int64_t vi = (sc0 + sl) + (row0 + r) * n;
                        sv[(r * 3 + 0) * W + sl] = vk[vi];
                        sv[(r * 3 + 1) * W + sl] = vk[vld + vi];
                        sv[(r * 3 + 2) * W + sl] = vk[2 * vld + vi];
                    }
                    for (int t = threadIdx.x; t < nr * (nvs - 1); t += blockDim.x) {
                        int r = t / (nvs - 1), sl = t - r * (nvs - 1);
                        sg[r * SC + sl] = gk[(row0 + r) * (n - 1) + sc0 + sl];
                    }
                    __syncthreads();
                    if (active) {
                        for (int r = 0; r < nr; r++) {
                            const T* gr = sg + r * SC;
                            strip_normal<T, SIGMA>(sv + r * 3 * W, sv + (r + 1) * 3 * W, W, nvs, px, py, pz, nx, ny, nz,
                                                   w.sigma2, [&](int kk, T val) { acc += gr[kk] * val; });
                        }
                    }
                }
            }
        }
        base += count;
    }
    if (active) w.partial[(int64_t)blockIdx.y * ntg + g] = acc;
}

template <class T>
__global__ void k_wake_reduce(const T* partial, int64_t slices, int64_t ntg, T* rhs) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= ntg) return;
    T s = 0;
    for (int64_t k = 0; k < slices; k++) s += partial[k * ntg + g];
    rhs[g] -= s * inv_four_pi<T>();
}

template <class T>
static int wake_influence(T* rhs, int32_t nsurf, const gbvlm_dims* dims, const T* const* gamma_wake,
                          const T* const* colloc, const T* const* normals, const T* const* verts_wake,
                          const int32_t* lifting, int32_t iteration, T sigma, int32_t window, T* scratch,
                          size_t scratch_elems, cudaStream_t st, const int64_t* it_dev = nullptr) {
    WakeArgs<T> w;
    int rc = make_surfs(w.s, nsurf, dims);
    if (rc) return rc;
    GB_REQUIRE(rhs != nullptr, "rhs is null");
    GB_REQUIRE(lifting != nullptr, "lifting is null");
    GB_REQUIRE(iteration >= 0, "iteration < 0");
    w.it_dev = it_dev;
    w.iteration = iteration;
    w.window = window;
    w.sigma2 = sigma * sigma;
    int64_t total = 0;
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(colloc[m] && normals[m], "null pointer for surface %d", m);
        w.s.a[m] = colloc[m];
        w.s.b[m] = normals[m];
        w.s.flag[m] = lifting[m] ? 1 : 0;
        if (lifting[m] && iteration > 0) {
            GB_REQUIRE(verts_wake && verts_wake[m] && gamma_wake && gamma_wake[m], "wake of surface %d is null", m);
            GB_REQUIRE(dims[m].nwv >= iteration + 1, "surface %d: nwv=%lld < iteration+1", m, (long long)dims[m].nwv);
            w.s.c[m] = verts_wake[m];
            w.s.d[m] = gamma_wake[m];
            int64_t end = dims[m].nwv - 1;
            if (window > 0 && iteration > window) end = dims[m].nwv - 1 - iteration + window;
            total += end - (dims[m].nwv - iteration - 1);
        } else {
            w.s.flag[m] = 0;
        }
    }
    if (total == 0) return GBVLM_OK;
    const int64_t ntg = w.s.poff[nsurf];
    const int64_t xblocks = cdiv(ntg, WK_THREADS);
    // enough slices to cover about `wake.waves` waves of the device's SMs
    // (tuned per shape), at least WK_ROWS rows each; a caller-owned scratch
    // caps the slice count at what it holds
    int64_t want = cdiv(tune().wake_waves * sm_count(), xblocks);
    if (scratch != nullptr) want = std::min<int64_t>(want, (int64_t)(scratch_elems / (size_t)ntg));
    int64_t slices = want < 1 ? 1 : want;
    int64_t rps = cdiv(total, slices);
    if (rps < WK_ROWS) rps = WK_ROWS;
    slices = cdiv(total, rps);
    if (scratch == nullptr) {
        GB_REQUIRE(it_dev == nullptr, "the device-iteration form needs its own scratch");
        void* p = nullptr;
        rc = device_scratch(sizeof(T) * slices * ntg, &p, st);
        if (rc) return rc;
        scratch = (T*)p;
    } else {
        GB_REQUIRE((size_t)(slices * ntg) <= scratch_elems, "scratch too small: need %lld elements",
                   (long long)(slices * ntg));
    }
    w.total_rows = total;
    w.rows_per_slice = rps;
    w.partial = scratch;
    int64_t maxs = 1;
    for (int m = 0; m < nsurf; m++)
        if (w.s.flag[m] && dims[m].ns > maxs) maxs = dims[m].ns;
    w.sc = (int32_t)(maxs < WK_MAXSPAN ? maxs : WK_MAXSPAN);
    const size_t smem = ((WK_ROWS + 1) * 3 * (w.sc + 1) + WK_ROWS * w.sc) * sizeof(T);
    dim3 grid((unsigned)xblocks, (unsigned)slices);
    if (sigma != (T)0) {
        GB_CUDA(cudaFuncSetAttribute(k_wake_influence<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_wake_influence<T, true><<<grid, WK_THREADS, smem, st>>>(w);
    } else {
        GB_CUDA(cudaFuncSetAttribute(k_wake_influence<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_wake_influence<T, false><<<grid, WK_THREADS, smem, st>>>(w);
    }
    GB_LAUNCH_CHECK();
    k_wake_reduce<T><<<(unsigned)cdiv(ntg, 256), 256, 0, st>>>(scratch, slices, ntg, rhs);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// a17: free-wake roll-up (ispc:215-271).  One thread per moving wake vertex;
// block-stages chunks of source ring rows.  Sources: every wing lattice
// (all ring rows) and every lifting wake (its active ring rows).  New
// positions go to `out` (a copy of the wake) so that all reads see the old
// positions; the host then swaps/copies.
// ---------------------------------------------------------------------------
constexpr int RU_THREADS = 128;

template <class T>
struct RollArgs {
    Surfs<T> s;  // a=verts_wing, b=gamma_wing, c=verts_wake(old), d=gamma_wake, flag=lifting; o0=out wake
    int32_t iteration;
    T sigma2, dt;
    int64_t voff[GBVLM_MAX_SURFACES + 1];  // packed moving-vertex offsets
    int32_t sc;                             // spanwise rings staged per chunk
};

template <class T, bool SIGMA>
__device__ __forceinline__ void lattice_vel(T px, T py, T pz, const T* v, int64_t vld, int64_t n, int64_t r0, int64_t r1,
                                            const T* gam, T sigma2, T* sv, T* sgm, int SC, V3<T>& vel) {
    const int W = SC + 1;
    for (int64_t sc0 = 0; sc0 < n - 1; sc0 += SC) {
        const int64_t sc1 = min(sc0 + (int64_t)SC, n - 1);
        const int nvs = (int)(sc1 - sc0 + 1);
        for (int64_t rr = r0; rr < r1; rr += WK_ROWS) {
            const int nr = (int)min((int64_t)WK_ROWS, r1 - rr);
            __syncthreads();
            for (int t = threadIdx.x; t < (nr + 1) * nvs; t += blockDim.x) {
                int r = t / nvs, sl = t - r * nvs;
                int64_t vi = (sc0 + sl) + (rr + r) * n;
                sv[(r * 3 + 0) * W + sl] = v[vi];
                sv[(r * 3 + 1) * W + sl] = v[vld + vi];
                sv[(r * 3 + 2) * W + sl] = v[2 * vld + vi];
            }
            for (int t = threadIdx.x; t < nr * (nvs - 1); t += blockDim.x) {
                int r = t / (nvs - 1), sl = t - r * (nvs - 1);
                sgm[r * SC + sl] = gam[(rr + r) * (n - 1) + sc0 + sl];
            }
            __syncthreads();
            for (int r = 0; r < nr; r++) {
                const T* gr = sgm + r * SC;
                strip_vec<T, SIGMA>(sv + r * 3 * W, sv + (r + 1) * 3 * W, W, nvs, px, py, pz, sigma2,
                                    [&](int kk, V3<T> v) {
                                        const T gm = gr[kk];
                                        vel.x += gm * v.x;
                                        vel.y += gm * v.y;
                                        vel.z += gm * v.z;
                                    });
            }
        }
    }
}

template <class T, bool SIGMA>
__global__ void __launch_bounds__(RU_THREADS) k_rollup(RollArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sv = reinterpret_cast<T*>(smem_raw);
    T* sgm = sv + (WK_ROWS + 1) * 3 * (a.sc + 1);
    const int64_t total = a.voff[a.s.n];
    const int64_t g = (int64_t)blockIdx.x * RU_THREADS + threadIdx.x;
    const bool active = g < total;
    int m = 0;
    int64_t vi = 0, vld = 0;
    T px = 0, py = 0, pz = 0;
    if (active) {
        while (m + 1 < a.s.n && g >= a.voff[m + 1]) m++;
        const int64_t n = a.s.ns[m] + 1;
        vld = n * a.s.nwv[m];
        vi = (a.s.nwv[m] - a.iteration) * n + (g - a.voff[m]);
        px = a.s.c[m][vi]; py = a.s.c[m][vld + vi]; pz = a.s.c[m][2 * vld + vi];
    }
    V3<T> vel{0, 0, 0};
    for (int k = 0; k < a.s.n; k++) {
        const int64_t n = a.s.ns[k] + 1;
        lattice_vel<T, SIGMA>(px, py, pz, a.s.a[k], n * (a.s.nc[k] + 1), n, 0, a.s.nc[k], a.s.b[k], a.sigma2, sv, sgm, a.sc, vel);
        if (!a.s.flag[k]) continue;
        const int64_t nw = a.s.nwv[k];
        lattice_vel<T, SIGMA>(px, py, pz, a.s.c[k], n * nw, n, nw - a.iteration - 1, nw - 1, a.s.d[k], a.sigma2, sv, sgm, a.sc, vel);
    }
    if (active) {
        const T sc = a.dt * inv_four_pi<T>();
        a.s.o0[m][vi] = px + vel.x * sc;
        a.s.o0[m][vld + vi] = py + vel.y * sc;
        a.s.o0[m][2 * vld + vi] = pz + vel.z * sc;
    }
}

template <class T>
static int wake_rollup(int32_t nsurf, const gbvlm_dims* dims, T* const* verts_wake, const T* const* verts_wing,
                       const T* const* gamma_wing, const T* const* gamma_wake, const int32_t* lifting, T sigma, T dt,
                       int32_t iteration, cudaStream_t st) {
    RollArgs<T> a;
    int rc = make_surfs(a.s, nsurf, dims);
    if (rc) return rc;
    GB_REQUIRE(lifting != nullptr, "lifting is null");
    GB_REQUIRE(iteration >= 0, "iteration < 0");
    if (iteration == 0) return GBVLM_OK;
    size_t wake_bytes = 0;
    a.voff[0] = 0;
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(verts_wake[m] && verts_wing[m] && gamma_wing[m], "null pointer for surface %d", m);
        GB_REQUIRE(dims[m].nwv >= iteration + 1, "surface %d: nwv=%lld < iteration+1", m, (long long)dims[m].nwv);
        a.s.a[m] = verts_wing[m];
        a.s.b[m] = gamma_wing[m];
        a.s.c[m] = verts_wake[m];
        a.s.d[m] = gamma_wake ? gamma_wake[m] : nullptr;
        a.s.flag[m] = lifting[m] ? 1 : 0;
        if (lifting[m]) GB_REQUIRE(gamma_wake && gamma_wake[m], "gamma_wake of surface %d is null", m);
        a.voff[m + 1] = a.voff[m] + (int64_t)iteration * (dims[m].ns + 1);
        wake_bytes += sizeof(T) * 3 * (dims[m].ns + 1) * dims[m].nwv;
    }
    void* scratch = nullptr;
    rc = device_scratch(wake_bytes, &scratch, st);
    if (rc) return rc;
    size_t off = 0;
    for (int m = 0; m < nsurf; m++) {
        a.s.o0[m] = (T*)((char*)scratch + off);
        off += sizeof(T) * 3 * (dims[m].ns + 1) * dims[m].nwv;
    }
    a.iteration = iteration;
    a.sigma2 = sigma * sigma;
    a.dt = dt;
    int64_t maxs = 1;
    for (int m = 0; m < nsurf; m++)
        if (dims[m].ns > maxs) maxs = dims[m].ns;
    a.sc = (int32_t)(maxs < WK_MAXSPAN ? maxs : WK_MAXSPAN);
    const size_t smem = ((WK_ROWS + 1) * 3 * (a.sc + 1) + WK_ROWS * a.sc) * sizeof(T);
    const int64_t total = a.voff[nsurf];
    if (sigma != (T)0) {
        GB_CUDA(cudaFuncSetAttribute(k_rollup<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_rollup<T, true><<<(unsigned)cdiv(total, RU_THREADS), RU_THREADS, smem, st>>>(a);
    } else {
        GB_CUDA(cudaFuncSetAttribute(k_rollup<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_rollup<T, false><<<(unsigned)cdiv(total, RU_THREADS), RU_THREADS, smem, st>>>(a);
    }
    GB_LAUNCH_CHECK();
    for (int m = 0; m < nsurf; m++) {
        const int64_t n = dims[m].ns + 1, vld = n * dims[m].nwv, begin = (dims[m].nwv - iteration) * n;
        for (int k = 0; k < 3; k++) {
            GB_CUDA(cudaMemcpyAsync(verts_wake[m] + k * vld + begin, a.s.o0[m] + k * vld + begin,
                                    sizeof(T) * iteration * n, cudaMemcpyDeviceToDevice, st));
        }
    }
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// a9: panel forces (vlm_backend_cpu.cpp:276-321), rho = 1
// ---------------------------------------------------------------------------
template <class T, bool UNSTEADY>
__global__ void k_forces(int64_t ns, int64_t nc, const T* vw, const T* gd, const T* dg, const T* vel, const T* ar,
                         const T* nor, T* f) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t np = ns * nc;
    if (p >= np) return;
    int64_t i = p % ns, j = p / ns, vld = (ns + 1) * (nc + 1);
    int64_t a = i + j * (ns + 1), b = a + 1;
    const T rho = 1;
    V3<T> V{vel[p], vel[np + p], vel[2 * np + p]};
    V3<T> v0{vw[a], vw[vld + a], vw[2 * vld + a]}, v1{vw[b], vw[vld + b], vw[2 * vld + b]};
    V3<T> F = (rho * gd[p]) * cross(V, v1 - v0);
    if (UNSTEADY) {
        V3<T> n{nor[p], nor[np + p], nor[2 * np + p]};
        F = F + (rho * dg[p] * ar[p]) * n;
    }
    f[p] = F.x;
    f[np + p] = F.y;
    f[2 * np + p] = F.z;
}

// ---------------------------------------------------------------------------
// a10/a11/a12: reductions in double with compensation, one block
// ---------------------------------------------------------------------------
constexpr int RED_THREADS = 512;

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0;
    if (threadIdx.x == 0) {
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];
    }
    __syncthreads();
    return r;
}

// kind 0: cl = sum F.L ; kind 1: cm = sum (0.5(v0+v1) - ref) x F ; kind 2: sum x ; kind 3: mac numerator
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_reduce(int kind, int64_t ns, int64_t nc, const T* x, const T* vw,
                                                        double ax, double ay, double az, double* out) {
    __shared__ double sh[32];
    CSum s0, s1, s2;
    const int64_t np = ns * nc, vld = (ns + 1) * (nc + 1);
    if (kind == 0) {
        for (int64_t p = threadIdx.x; p < np; p += blockDim.x)
            s0.add((double)x[p] * ax + (double)x[np + p] * ay + (double)x[2 * np + p] * az);
    } else if (kind == 1) {
        for (int64_t p = threadIdx.x; p < np; p += blockDim.x) {
            int64_t i = p % ns, j = p / ns, a = i + j * (ns + 1), b = a + 1;
            double lx = 0.5 * ((double)vw[a] + (double)vw[b]) - ax;
            double ly = 0.5 * ((double)vw[vld + a] + (double)vw[vld + b]) - ay;
            double lz = 0.5 * ((double)vw[2 * vld + a] + (double)vw[2 * vld + b]) - az;
            double fx = x[p], fy = x[np + p], fz = x[2 * np + p];
            s0.add(ly * fz - lz * fy);
            s1.add(lz * fx - lx * fz);
            s2.add(lx * fy - ly * fx);
        }
    } else if (kind == 2) {
        for (int64_t p = threadIdx.x; p < ns; p += blockDim.x) s0.add((double)x[p]);
    } else {
        const int64_t last = nc * (ns + 1);
        for (int64_t i = threadIdx.x; i < ns; i += blockDim.x) {
            double dx0 = (double)vw[i] - vw[last + i], dy0 = (double)vw[vld + i] - vw[vld + last + i];
            double dz0 = (double)vw[2 * vld + i] - vw[2 * vld + last + i];
            double dx1 = (double)vw[i + 1] - vw[last + i + 1], dy1 = (double)vw[vld + i + 1] - vw[vld + last + i + 1];
            double dz1 = (double)vw[2 * vld + i + 1] - vw[2 * vld + last + i + 1];
            double c0 = sqrt(dx0 * dx0 + dy0 * dy0 + dz0 * dz0), c1 = sqrt(dx1 * dx1 + dy1 * dy1 + dz1 * dz1);
            double dx3 = (double)vw[i + 1] - vw[i], dy3 = (double)vw[vld + i + 1] - vw[vld + i];
            double dz3 = (double)vw[2 * vld + i + 1] - vw[2 * vld + i];
            s0.add(0.5 * (c0 * c0 + c1 * c1) * sqrt(dx3 * dx3 + dy3 * dy3 + dz3 * dz3));
        }
        // areas sum in s1 (x = areas)
        for (int64_t p = threadIdx.x; p < np; p += blockDim.x) s1.add((double)x[p]);
    }
    double r0 = block_sum(s0.value(), sh), r1 = block_sum(s1.value(), sh), r2 = block_sum(s2.value(), sh);
    if (threadIdx.x == 0) {
        out[0] = r0;
        out[1] = r1;
        out[2] = r2;
    }
}

template <class T>
static int reduce_sync(int kind, int64_t ns, int64_t nc, const T* x, const T* vw, double ax, double ay, double az,
                       double* host_out, cudaStream_t st) {
    void* d = nullptr;
    int rc = device_scratch(4 * sizeof(double), &d, st);
    if (rc) return rc;
    k_reduce<T><<<1, RED_THREADS, 0, st>>>(kind, ns, nc, x, vw, ax, ay, az, (double*)d);
    GB_LAUNCH_CHECK();
    double* h = (double*)host_scratch(4 * sizeof(double));
    GB_REQUIRE(h != nullptr, "pinned host allocation failed");
    GB_CUDA(cudaMemcpyAsync(h, d, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    host_out[0] = h[0];
    host_out[1] = h[1];
    host_out[2] = h[2];
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// a13: wake gamma from trailing-edge Fourier coefficients (cpu.cpp:470-503)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_gamma_wake(T* gw, int64_t ns, int64_t ncols, const T* co, int32_t H, T tn, T omega, T dt, int64_t it) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g >= ns * it) return;
    const int64_t start = ncols - it;
    int64_t i = g % ns, j = start + g / ns;
    const int32_t U = 2 * H + 1;
    const T s0 = (T)1 / dsqrt((T)U), s2 = dsqrt((T)2 / (T)U);
    T v = co[i] * s0;
    for (int32_t h = 0; h < H; h++) {
        const T wk = omega * (T)(h + 1);
        T ph = wk * (tn - (T)(j - start + 1) * dt);
        T sn, cs;
        if constexpr (sizeof(T) == 4) {
            sincosf(ph, &sn, &cs);
        } else {
            sincos(ph, &sn, &cs);
        }
        v += co[i + (2 * h + 1) * ns] * cs * s2;
        v += co[i + (2 * h + 2) * ns] * sn * s2;
    }
    gw[i + j * ns] = v;
}

// ---------------------------------------------------------------------------
// a5 / a4: displacement and wake shedding
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_displace(Surfs<T> s) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    // vertex offsets in poff-like packing: reuse nwv as vertex counts
    int m = 0;
    int64_t base = 0;
    while (m < s.n) {
        int64_t nv = (s.ns[m] + 1) * (s.nc[m] + 1);
        if (g < base + nv) break;
        base += nv;
        m++;
    }
    if (m >= s.n) return;
    int64_t r = g - base, nv = (s.ns[m] + 1) * (s.nc[m] + 1);
    const T* tr = s.a[m];
    const T* in = s.b[m];
    T* out = s.o0[m];
    T x[4] = {in[r], in[nv + r], in[2 * nv + r], in[3 * nv + r]};
#pragma unroll
    for (int c = 0; c < 4; c++) {
        T acc = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) acc += x[k] * tr[c + 4 * k];
        out[c * nv + r] = acc;
    }
}

template <class T>
__global__ void k_wake_shed(Surfs<T> s, int32_t it) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int m = 0;
    int64_t base = 0;
    while (m < s.n) {
        int64_t cnt = 4 * (s.ns[m] + 1);
        if (g < base + cnt) break;
        base += cnt;
        m++;
    }
    if (m >= s.n) return;
    int64_t r = g - base, n = s.ns[m] + 1;
    int64_t k = r / n, i = r % n;
    const T* vw = s.a[m];
    T* vk = s.o0[m];
    int64_t vld = n * (s.nc[m] + 1), kld = n * s.nwv[m];
    vk[k * kld + i + (s.nwv[m] - 1 - it) * n] = vw[k * vld + i + s.nc[m] * n];
}

// ---------------------------------------------------------------------------
// a8: fused circulation update (vlm.cpp:442-458)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_gamma_update(int64_t ns, int64_t nc, const T* x, T* g, T* gd, T* gw, int64_t wcol, const T* gp,
                               T* dgdt, T inv_dt) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= ns * nc) return;
    int64_t i = p % ns, j = p / ns;
    T v = x[p];
    g[p] = v;
    gd[p] = (j > 0) ? v - x[p - ns] : v;
    if (gw && j == nc - 1) gw[i + wcol * ns] = v;
    if (dgdt) dgdt[p] = (v - gp[p]) * inv_dt;
}

// the same two with the iteration read on the device (graph replay)
template <class T>
__global__ void k_wake_shed_dev(Surfs<T> s, const int64_t* it_dev) {
    int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int m = 0;
    int64_t base = 0;
    while (m < s.n) {
        int64_t cnt = 4 * (s.ns[m] + 1);
        if (g < base + cnt) break;
        base += cnt;
        m++;
    }
    if (m >= s.n) return;
    const int64_t it = *it_dev;
    if (it < 0 || it >= s.nwv[m]) return;
    int64_t r = g - base, n = s.ns[m] + 1;
    int64_t k = r / n, i = r % n;
    int64_t vld = n * (s.nc[m] + 1), kld = n * s.nwv[m];
    s.o0[m][k * kld + i + (s.nwv[m] - 1 - it) * n] = s.a[m][k * vld + i + s.nc[m] * n];
}

template <class T>
__global__ void k_gamma_update_dev(int64_t ns, int64_t nc, const T* x, T* g, T* gd, T* gw, int64_t col_base,
                                   const int64_t* it_dev, const T* gp, T* dgdt, T inv_dt, int64_t ncols) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= ns * nc) return;
    int64_t i = p % ns, j = p / ns;
    T v = x[p];
    g[p] = v;
    gd[p] = (j > 0) ? v - x[p - ns] : v;
    const int64_t wcol = col_base - *it_dev;
    if (gw && j == nc - 1 && wcol >= 0 && wcol < ncols) gw[i + wcol * ns] = v;
    if (dgdt) dgdt[p] = (v - gp[p]) * inv_dt;
}

// ---------------------------------------------------------------------------
// Trefftz-plane drag (ispc:273-323): one block per spanwise ring
// ---------------------------------------------------------------------------
template <class T, bool SIGMA>
__global__ void k_trefftz(int64_t nv, int64_t nwv, const T* v, const T* gam, T sigma2, double* partial) {
    __shared__ double sh[32];
    const int64_t i = nwv - 2, ld = nv * nwv;
    const int64_t j = blockIdx.x;
    auto P = [&](int64_t idx) { return V3<T>{v[idx], v[ld + idx], v[2 * ld + idx]}; };
    V3<T> a = P(i * nv + j), b = P(i * nv + j + 1), d = P((i + 1) * nv + j + 1), e = P((i + 1) * nv + j);
    V3<T> c = (T)0.25 * (((a + b) + d) + e);
    V3<T> nn = cross(e - b, d - a);
    T l = dsqrt(len2(nn));
    V3<T> n{nn.x / l, nn.y / l, nn.z / l};
    double acc = 0;
    for (int64_t jj = threadIdx.x; jj < nv - 1; jj += blockDim.x) {
        V3<T> w0 = P(i * nv + jj), w1 = P(i * nv + jj + 1), w2 = P((i + 1) * nv + jj + 1), w3 = P((i + 1) * nv + jj);
        V3<T> inf2{0, 0, 0};
        symmetry_ref(inf2, c, w1, w2, (T)sqrt((double)sigma2));
        symmetry_ref(inf2, c, w3, w0, (T)sqrt((double)sigma2));
        acc += (double)gam[i * (nv - 1) + jj] * (double)dot(inf2, n);
    }
    double iv = block_sum(acc, sh);
    if (threadIdx.x == 0) {
        V3<T> dl = b - a;
        partial[j] = -(double)gam[i * (nv - 1) + j] * iv * sqrt((double)len2(dl));
    }
}

__global__ void k_sum_partials(const double* p, int64_t n, double* out) {
    __shared__ double sh[32];
    CSum s;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) s.add(p[k]);
    double r = block_sum(s.value(), sh);
    if (threadIdx.x == 0) out[0] = r;
}

template <class T>
static int trefftz(int64_t ns, int64_t nwv, const T* vk, const T* gw, const T* fs, T area, T sigma, T* out,
                   cudaStream_t st) {
    GB_REQUIRE(ns >= 1 && nwv >= 2, "trefftz needs ns>=1 and nwv>=2");
    GB_REQUIRE(vk && gw && fs && out, "null pointer");
    void* d = nullptr;
    int rc = device_scratch(sizeof(double) * (ns + 2), &d, st);
    if (rc) return rc;
    double* part = (double*)d;
    if (sigma != (T)0)
        k_trefftz<T, true><<<(unsigned)ns, 128, 0, st>>>(ns + 1, nwv, vk, gw, sigma * sigma, part);
    else
        k_trefftz<T, false><<<(unsigned)ns, 128, 0, st>>>(ns + 1, nwv, vk, gw, (T)0, part);
    GB_LAUNCH_CHECK();
    k_sum_partials<<<1, 256, 0, st>>>(part, ns, part + ns);
    GB_LAUNCH_CHECK();
    double* h = (double*)host_scratch(sizeof(double));
    GB_CUDA(cudaMemcpyAsync(h, part + ns, sizeof(double), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    double v2 = (double)fs[0] * fs[0] + (double)fs[1] * fs[1] + (double)fs[2] * fs[2];
    *out = (T)(h[0] / (v2 * (double)area));
    return GBVLM_OK;
}

}  // namespace gbvlm

using namespace gbvlm;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* gbvlm_last_error(void) { return g_err; }
int gbvlm_version(void) { return 10000; }

#define GB_BOTH(MACRO) MACRO(f32, float) MACRO(f64, double)

#define DEF_LHS(sfx, T)                                                                                       \
    int gbvlm_lhs_assemble_##sfx(T* lhs, int64_t ld, int32_t nsurf, const gbvlm_dims* dims,                 \
                                 const T* const* colloc, const T* const* normals, const T* const* verts_wing, \
                                 const T* const* verts_wake, int32_t iteration, T sigma, gbvlm_stream stream) { \
        GB_REQUIRE(colloc && normals && verts_wing, "null surface array");                                   \
        return lhs_assemble<T>(lhs, ld, nsurf, dims, colloc, normals, verts_wing, verts_wake, iteration, sigma, \
                               to_cuda(stream));                                                              \
    }
GB_BOTH(DEF_LHS)

#define DEF_RHSV(sfx, T)                                                                                  \
    int gbvlm_rhs_assemble_velocities_##sfx(T* rhs, int32_t nsurf, const gbvlm_dims* dims,               \
                                            const T* const* normals, const T* const* velocities,         \
                                            gbvlm_stream stream) {                                       \
        GB_REQUIRE(normals && velocities, "null surface array");                                         \
        return rhs_velocities<T>(rhs, nsurf, dims, normals, velocities, to_cuda(stream));                \
    }
GB_BOTH(DEF_RHSV)

int gbvlm_rhs_assemble_wake_influence_f32(float* rhs, int32_t nsurf, const gbvlm_dims* dims,
                                          const float* const* gamma_wake, const float* const* colloc,
                                          const float* const* normals, const float* const* verts_wake,
                                          const int32_t* lifting, int32_t iteration, float sigma,
                                          gbvlm_stream stream) {
    GB_REQUIRE(colloc && normals, "null surface array");
    return wake_influence<float>(rhs, nsurf, dims, gamma_wake, colloc, normals, verts_wake, lifting, iteration, sigma,
                                 5000, nullptr, 0, to_cuda(stream));
}
}  // extern "C"

namespace gbvlm {

int wake_influence_dev_f32(float* rhs, int32_t nsurf, const gbvlm_dims* dims, const float* const* gamma_wake,
                           const float* const* colloc, const float* const* normals, const float* const* verts_wake,
                           const int32_t* lifting, const int64_t* it_dev, int32_t it_max, float* scratch,
                           cudaStream_t st) {
    GB_REQUIRE(colloc && normals && it_dev && scratch, "null argument");
    int64_t ntg = 0;
    for (int m = 0; m < nsurf; m++) ntg += dims[m].ns * dims[m].nc;
    return wake_influence<float>(rhs, nsurf, dims, gamma_wake, colloc, normals, verts_wake, lifting, it_max, 0.f, 5000,
                                 scratch, (size_t)(WAKE_DEV_MAX_SLICES * ntg), st, it_dev);
}

int wake_shed_dev_f32(int32_t nsurf, const gbvlm_dims* dims, const float* const* verts_wing, float* const* verts_wake,
                      const int64_t* it_dev, cudaStream_t st) {
    Surfs<float> s;
    int rc = make_surfs(s, nsurf, dims);
    if (rc) return rc;
    int64_t total = 0;
    for (int m = 0; m < nsurf; m++) {
        GB_REQUIRE(verts_wing[m] && verts_wake[m], "null pointer surface %d", m);
        s.a[m] = verts_wing[m];
        s.o0[m] = verts_wake[m];
        total += 4 * (dims[m].ns + 1);
    }
    k_wake_shed_dev<float><<<(unsigned)cdiv(total, 256), 256, 0, st>>>(s, it_dev);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

int gamma_update_dev_f32(int64_t ns, int64_t nc, const float* x, float* gamma, float* gamma_delta, float* gamma_wake,
                         int64_t col_base, const int64_t* it_dev, const float* gamma_prev, float* dgamma_dt, float dt,
                         cudaStream_t st) {
    GB_REQUIRE(ns >= 1 && nc >= 1 && x && gamma && gamma_delta && it_dev, "bad arguments");
    GB_REQUIRE(!dgamma_dt || (gamma_prev && dt != 0.f), "dgamma_dt needs gamma_prev and dt != 0");
    k_gamma_update_dev<float><<<(unsigned)cdiv(ns * nc, 256), 256, 0, st>>>(
        ns, nc, x, gamma, gamma_delta, gamma_wake, col_base, it_dev, gamma_prev, dgamma_dt, dgamma_dt ? 1.f / dt : 0.f,
        col_base + 1);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

}  // namespace gbvlm

extern "C" {

int gbvlm_rhs_assemble_wake_influence_f64(double* rhs, int32_t nsurf, const gbvlm_dims* dims,
                                          const double* const* gamma_wake, const double* const* colloc,
                                          const double* const* normals, const double* const* verts_wake,
                                          const int32_t* lifting, int32_t iteration, double sigma,
                                          gbvlm_stream stream) {
    GB_REQUIRE(colloc && normals, "null surface array");
    return wake_influence<double>(rhs, nsurf, dims, gamma_wake, colloc, normals, verts_wake, lifting, iteration,
                                  sigma, 0, nullptr, 0, to_cuda(stream));
}

#define DEF_FORCES(sfx, T)                                                                                    \
    int gbvlm_forces_steady_##sfx(int64_t ns, int64_t nc, const T* verts_wing, const T* gamma_delta,         \
                                  const T* velocities, T* forces, gbvlm_stream stream) {                     \
        GB_REQUIRE(ns >= 1 && nc >= 1, "bad sizes");                                                         \
        GB_REQUIRE(verts_wing && gamma_delta && velocities && forces, "null pointer");                       \
        k_forces<T, false><<<(unsigned)cdiv(ns * nc, 256), 256, 0, to_cuda(stream)>>>(                        \
            ns, nc, verts_wing, gamma_delta, nullptr, velocities, nullptr, nullptr, forces);                 \
        GB_LAUNCH_CHECK();                                                                                   \
        return GBVLM_OK;                                                                                     \
    }                                                                                                        \
    int gbvlm_forces_unsteady_##sfx(int64_t ns, int64_t nc, const T* verts_wing, const T* gamma_delta,       \
                                    const T* dgamma_dt, const T* velocities, const T* areas, const T* normals, \
                                    T* forces, gbvlm_stream stream) {                                        \
        GB_REQUIRE(ns >= 1 && nc >= 1, "bad sizes");                                                         \
        GB_REQUIRE(verts_wing && gamma_delta && dgamma_dt && velocities && areas && normals && forces,       \
                   "null pointer");                                                                          \
        k_forces<T, true><<<(unsigned)cdiv(ns * nc, 256), 256, 0, to_cuda(stream)>>>(                         \
            ns, nc, verts_wing, gamma_delta, dgamma_dt, velocities, areas, normals, forces);                 \
        GB_LAUNCH_CHECK();                                                                                   \
        return GBVLM_OK;                                                                                     \
    }
GB_BOTH(DEF_FORCES)

#define DEF_COEFF(sfx, T)                                                                                     \
    int gbvlm_coeff_cl_##sfx(int64_t ns, int64_t nc, const T* forces, const T* lift_axis, const T* freestream, \
                             T rho, T area, T* out, gbvlm_stream stream) {                                    \
        GB_REQUIRE(ns >= 1 && nc >= 1 && forces && lift_axis && freestream && out, "bad arguments");          \
        double r[3];                                                                                          \
        int rc = reduce_sync<T>(0, ns, nc, forces, nullptr, lift_axis[0], lift_axis[1], lift_axis[2], r,      \
                                to_cuda(stream));                                                            \
        if (rc) return rc;                                                                                    \
        T v2 = freestream[0] * freestream[0] + freestream[1] * freestream[1] + freestream[2] * freestream[2];   \
        *out = (T)(r[0] / ((double)((T)0.5 * rho * v2 * area)));                                              \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_coeff_cm_##sfx(int64_t ns, int64_t nc, const T* forces, const T* verts_wing, const T* ref_pt,   \
                             const T* freestream, T rho, T area, T mac, T* out, gbvlm_stream stream) {        \
        GB_REQUIRE(ns >= 1 && nc >= 1 && forces && verts_wing && ref_pt && freestream && out, "bad arguments"); \
        double r[3];                                                                                          \
        int rc = reduce_sync<T>(1, ns, nc, forces, verts_wing, ref_pt[0], ref_pt[1], ref_pt[2], r,            \
                                to_cuda(stream));                                                            \
        if (rc) return rc;                                                                                    \
        T v2 = freestream[0] * freestream[0] + freestream[1] * freestream[1] + freestream[2] * freestream[2];   \
        double d = (double)((T)0.5 * rho * v2 * area * mac);                                                  \
        out[0] = (T)(r[0] / d);                                                                               \
        out[1] = (T)(r[1] / d);                                                                               \
        out[2] = (T)(r[2] / d);                                                                               \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_mesh_mac_##sfx(int64_t ns, int64_t nc, const T* verts_wing, const T* areas, T* out,            \
                             gbvlm_stream stream) {                                                           \
        GB_REQUIRE(ns >= 1 && nc >= 1 && verts_wing && areas && out, "bad arguments");                       \
        double r[3];                                                                                          \
        int rc = reduce_sync<T>(3, ns, nc, areas, verts_wing, 0, 0, 0, r, to_cuda(stream));                  \
        if (rc) return rc;                                                                                    \
        *out = (T)(r[0] / r[1]);                                                                              \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_sum_##sfx(const T* x, int64_t n, T* out, gbvlm_stream stream) {                                 \
        GB_REQUIRE(x && out && n >= 0, "bad arguments");                                                     \
        double r[3];                                                                                          \
        int rc = reduce_sync<T>(2, n, 1, x, nullptr, 0, 0, 0, r, to_cuda(stream));                           \
        if (rc) return rc;                                                                                    \
        *out = (T)r[0];                                                                                       \
        return GBVLM_OK;                                                                                      \
    }
GB_BOTH(DEF_COEFF)

#define DEF_METRICS(sfx, T)                                                                                   \
    int gbvlm_mesh_metrics_##sfx(T alpha_rad, int32_t nsurf, const gbvlm_dims* dims, const T* const* verts_wing, \
                                 T* const* colloc, T* const* normals, T* const* areas, gbvlm_stream stream) {  \
        GB_REQUIRE(verts_wing && colloc && normals && areas, "null surface array");                          \
        return mesh_metrics<T>(alpha_rad, nsurf, dims, verts_wing, colloc, normals, areas, to_cuda(stream));  \
    }
GB_BOTH(DEF_METRICS)

#define DEF_GWAKE(sfx, T)                                                                                     \
    int gbvlm_gamma_wake_from_coeffs_##sfx(T* gamma_wake, int64_t ns, int64_t ncols, const T* coeffs,        \
                                           int32_t harmonics, T tn, T omega, T dt, int64_t iteration,         \
                                           gbvlm_stream stream) {                                             \
        GB_REQUIRE(gamma_wake && coeffs && ns >= 1 && harmonics >= 0, "bad arguments");                      \
        GB_REQUIRE(iteration >= 0 && iteration <= ncols, "iteration=%lld outside [0, ncols]", (long long)iteration); \
        if (iteration == 0) return GBVLM_OK;                                                                  \
        k_gamma_wake<T><<<(unsigned)cdiv(ns * iteration, 256), 256, 0, to_cuda(stream)>>>(                   \
            gamma_wake, ns, ncols, coeffs, harmonics, tn, omega, dt, iteration);                             \
        GB_LAUNCH_CHECK();                                                                                   \
        return GBVLM_OK;                                                                                      \
    }
GB_BOTH(DEF_GWAKE)

#define DEF_DISPLACE(sfx, T)                                                                                  \
    int gbvlm_displace_wing_##sfx(int32_t nsurf, const gbvlm_dims* dims, const T* const* transforms,         \
                                  T* const* verts_wing, const T* const* verts_wing_init, gbvlm_stream stream) { \
        Surfs<T> s;                                                                                          \
        int rc = make_surfs(s, nsurf, dims);                                                                  \
        if (rc) return rc;                                                                                    \
        GB_REQUIRE(transforms && verts_wing && verts_wing_init, "null surface array");                       \
        int64_t total = 0;                                                                                    \
        for (int m = 0; m < nsurf; m++) {                                                                     \
            GB_REQUIRE(transforms[m] && verts_wing[m] && verts_wing_init[m], "null pointer surface %d", m);   \
            s.a[m] = transforms[m];                                                                           \
            s.b[m] = verts_wing_init[m];                                                                      \
            s.o0[m] = verts_wing[m];                                                                          \
            total += (dims[m].ns + 1) * (dims[m].nc + 1);                                                     \
        }                                                                                                     \
        k_displace<T><<<(unsigned)cdiv(total, 256), 256, 0, to_cuda(stream)>>>(s);                            \
        GB_LAUNCH_CHECK();                                                                                   \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_wake_shed_##sfx(int32_t nsurf, const gbvlm_dims* dims, const T* const* verts_wing,             \
                              T* const* verts_wake, int32_t iteration, gbvlm_stream stream) {                 \
        Surfs<T> s;                                                                                          \
        int rc = make_surfs(s, nsurf, dims);                                                                  \
        if (rc) return rc;                                                                                    \
        GB_REQUIRE(verts_wing && verts_wake, "null surface array");                                          \
        int64_t total = 0;                                                                                    \
        for (int m = 0; m < nsurf; m++) {                                                                     \
            GB_REQUIRE(verts_wing[m] && verts_wake[m], "null pointer surface %d", m);                        \
            GB_REQUIRE(iteration >= 0 && iteration < dims[m].nwv, "iteration %d outside wake of surface %d",   \
                       iteration, m);                                                                        \
            s.a[m] = verts_wing[m];                                                                           \
            s.o0[m] = verts_wake[m];                                                                          \
            total += 4 * (dims[m].ns + 1);                                                                    \
        }                                                                                                     \
        k_wake_shed<T><<<(unsigned)cdiv(total, 256), 256, 0, to_cuda(stream)>>>(s, iteration);                \
        GB_LAUNCH_CHECK();                                                                                   \
        return GBVLM_OK;                                                                                      \
    }
GB_BOTH(DEF_DISPLACE)

#define DEF_ROLLUP(sfx, T)                                                                                    \
    int gbvlm_wake_rollup_##sfx(int32_t nsurf, const gbvlm_dims* dims, T* const* verts_wake,                 \
                                const T* const* verts_wing, const T* const* gamma_wing,                      \
                                const T* const* gamma_wake, const int32_t* lifting, T sigma, T dt,           \
                                int32_t iteration, gbvlm_stream stream) {                                    \
        GB_REQUIRE(verts_wake && verts_wing && gamma_wing, "null surface array");                            \
        return wake_rollup<T>(nsurf, dims, verts_wake, verts_wing, gamma_wing, gamma_wake, lifting, sigma, dt, \
                              iteration, to_cuda(stream));                                                    \
    }
GB_BOTH(DEF_ROLLUP)

#define DEF_TREFFTZ(sfx, T)                                                                                   \
    int gbvlm_trefftz_cd_##sfx(int64_t ns, int64_t nwv, const T* verts_wake, const T* gamma_wake,            \
                               const T* freestream, T area, T sigma, T* out, gbvlm_stream stream) {          \
        return trefftz<T>(ns, nwv, verts_wake, gamma_wake, freestream, area, sigma, out, to_cuda(stream));    \
    }
GB_BOTH(DEF_TREFFTZ)

#define DEF_GUPDATE(sfx, T)                                                                                   \
    int gbvlm_gamma_update_##sfx(int64_t ns, int64_t nc, const T* x, T* gamma, T* gamma_delta, T* gamma_wake, \
                                 int64_t wake_col, const T* gamma_prev, T* dgamma_dt, T dt, gbvlm_stream stream) { \
        GB_REQUIRE(ns >= 1 && nc >= 1 && x && gamma && gamma_delta, "bad arguments");                        \
        GB_REQUIRE(!dgamma_dt || (gamma_prev && dt != (T)0), "dgamma_dt needs gamma_prev and dt != 0");      \
        k_gamma_update<T><<<(unsigned)cdiv(ns * nc, 256), 256, 0, to_cuda(stream)>>>(                         \
            ns, nc, x, gamma, gamma_delta, gamma_wake, wake_col, gamma_prev, dgamma_dt,                      \
            dgamma_dt ? (T)1 / dt : (T)0);                                                                   \
        GB_LAUNCH_CHECK();                                                                                   \
        return GBVLM_OK;                                                                                      \
    }
GB_BOTH(DEF_GUPDATE)

}  // extern "C"

// ===========================================================================
// Allocation-free variant of the float wake-influence entry point.
//
// Some callers cannot call cudaMalloc: a host application whose device
// memory is all owned by its own allocator or pool, a serving loop that
// admits work by a fixed device-memory budget and must not grow it behind
// the budget's back, and latency paths that must keep cudaMalloc's
// device-wide synchronisation out of every step.  For them the split-K
// partial sums of gbvlm_rhs_assemble_wake_influence_f32 live in the fixed
// array below instead of the library's grown-on-demand scratch buffer.
//
// The array is GBVLM_WAKE_SCRATCH_FLOATS floats (4 MiB) in this library's
// device image, so every GPU that loads the library holds it until the
// process exits.  Host code cannot hand the array's name to a kernel (on the
// host it is only a stand-in symbol), so the first call on each device looks
// up its device address with cudaGetSymbolAddress while that device is
// current and caches it with the context it belongs to; a later call from a
// different context (the primary context released and created again) looks
// it up again.
// All calls share the one array and every call overwrites the part it uses
// (each partial is written before it is read), so no contents carry over;
// calls whose kernels overlap on the GPU (different streams, no ordering
// between them) race on the array and must not be issued.
// ===========================================================================
#define GBVLM_WAKE_SCRATCH_FLOATS (1 << 20)

static __device__ __align__(256) float g_wake_scratch[GBVLM_WAKE_SCRATCH_FLOATS];

// cuCtxGetCurrent, resolved through the runtime so that loading the library
// needs no driver library (hosts without a GPU load it to check its exports)
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
static CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = []() -> CtxGetCurrentFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return (CtxGetCurrentFn)p;
    }();
    return fn;
}

static float* wake_scratch_address(int* rc) {
    static std::mutex mu;
    static float* addr[64] = {nullptr};
    static CUcontext owner[64] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *rc = cuda_fail(e, "cudaGetDevice", __FILE__, __LINE__);
        return nullptr;
    }
    if (dev < 0 || dev >= 64) {
        set_error("device index %d out of range", dev);
        *rc = GBVLM_ERR_ARG;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    CtxGetCurrentFn get_ctx = ctx_get_current();
    CUcontext cur = nullptr;
    if (addr[dev] && (!get_ctx || get_ctx(&cur) != CUDA_SUCCESS || cur != owner[dev])) addr[dev] = nullptr;
    if (!addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_wake_scratch);
        if (e != cudaSuccess) {
            *rc = cuda_fail(e, "cudaGetSymbolAddress(g_wake_scratch)", __FILE__, __LINE__);
            return nullptr;
        }
        if (!get_ctx || get_ctx(&cur) != CUDA_SUCCESS || cur == nullptr) {
            set_error("no current CUDA context after cudaGetSymbolAddress (cuCtxGetCurrent %s)",
                      get_ctx ? "failed" : "unavailable");
            *rc = GBVLM_ERR_CUDA;
            return nullptr;
        }
        addr[dev] = (float*)p;
        owner[dev] = cur;
    }
    *rc = GBVLM_OK;
    return addr[dev];
}

extern "C" int gbvlm_rhs_assemble_wake_influence_f32_noalloc(
    float* rhs, int32_t nsurf, const gbvlm_dims* dims, const float* const* gamma_wake, const float* const* colloc,
    const float* const* normals, const float* const* verts_wake, const int32_t* lifting, int32_t iteration,
    float sigma, gbvlm_stream stream) {
    GB_REQUIRE(colloc && normals && dims, "null surface array");
    GB_REQUIRE(nsurf >= 1 && nsurf <= GBVLM_MAX_SURFACES, "nsurf=%d outside [1, %d]", nsurf, GBVLM_MAX_SURFACES);
    int64_t ntg = 0;
    for (int m = 0; m < nsurf; m++) ntg += dims[m].ns * dims[m].nc;
    GB_REQUIRE(ntg <= GBVLM_WAKE_SCRATCH_FLOATS,
               "%lld collocation points exceed the %d-float fixed scratch of the allocation-free entry point",
               (long long)ntg, GBVLM_WAKE_SCRATCH_FLOATS);
    int rc = GBVLM_OK;
    float* scratch = wake_scratch_address(&rc);
    if (!scratch) return rc;
    // wake_influence() sizes its split-K slices from the problem and rejects a
    // partial-sum table larger than the scratch it is given
    return wake_influence<float>(rhs, nsurf, dims, gamma_wake, colloc, normals, verts_wake, lifting, iteration, sigma,
                                 5000, scratch, GBVLM_WAKE_SCRATCH_FLOATS, to_cuda(stream));
}
