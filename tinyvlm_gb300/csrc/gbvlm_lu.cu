// Dense LU with partial pivoting for one matrix or a ragged batch of
// matrices ("variable-size batched" right-looking LU), plus multi-RHS
// triangular solves and mixed-precision iterative refinement.
//
// Replaces vlm::LU (vlm/include/vlm_backend.hpp:99-119), i.e. LAPACKE
// ?getrf/?getrs on the CPU backend (vlm_backend_cpu_lapack.cpp:40-94) and
// cuSOLVER on the CUDA backend (vlm_backend_cuda_solvers.cu:39-102).
//
// Panel step k of every system with n > k runs in the same launches, so a
// batch of uneven systems fills the GPU with the trailing updates of all of
// them at once:
//   panel  : one CTA per active system factors columns [k, k+nb) (pivot
//            search = largest |a|, first row on ties, like LAPACK i?amax)
//   swap   : the panel's row interchanges applied to the other columns
//   trsm   : U12 = L11^-1 A12 (unit lower, L11 staged in shared memory)
//   update : A22 -= L21 U12, 64x64 register-tiled tiles enumerated over all
//            systems through a per-step prefix table
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <float.h>
#include <limits.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <vector>

#include "gbvlm_internal.h"
#include "gbvlm_lu.h"
#include "gbvlm_tc.cuh"

namespace gbvlm {

constexpr int PANEL_THREADS = 512;
constexpr int PR_THREADS_F64 = 256;  // register panel, double: 32 doubles of panel per thread
constexpr int PR_MAX_CLUSTER = 16;   // largest cluster of the register panel
constexpr int SW2_THREADS = 256;     // k_swap2: columns per CTA
constexpr int PACK_MIN_SLICE = 128;  // narrowest slice of a packed one-CTA panel (at most 8 systems per CTA)
constexpr int TRSM_COLS = 128;
constexpr int GT = 64;  // update tile edge
constexpr int GK = LU_NB;
constexpr int PERM_SMEM = 12 * 1024;  // systems up to this size build the permutation in shared memory
constexpr int TS_SMEM_BYTES = 200 * 1024;

template <class T>
__device__ __forceinline__ T tabs(T x) { return x < (T)0 ? -x : x; }

// Element-wise copy of `total` elements (ld_(e) -> st_(e, v)) by `nthreads`
// threads with U loads in flight per thread before the first store.  Written
// as load-then-store per element, the compiler may not move a global load
// above the previous store (it cannot prove they do not alias), which leaves
// one memory round trip per element.
template <int U, class LD, class ST>
__device__ __forceinline__ void staged_copy(int64_t total, int tid, int nthreads, LD ld_, ST st_) {
    using V = decltype(ld_((int64_t)0));
    for (int64_t e0 = tid; e0 < total; e0 += (int64_t)nthreads * U) {
        V v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int64_t e = e0 + (int64_t)u * nthreads;
            v[u] = e < total ? ld_(e) : V(0);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int64_t e = e0 + (int64_t)u * nthreads;
            if (e < total) st_(e, v[u]);
        }
    }
}

// ---------------------------------------------------------------------------
// panel: CTA b handles system act[b]
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(PANEL_THREADS) k_panel(LuBatch<T> B, int64_t k, const int32_t* act) {
    const int32_t sid = act[blockIdx.x];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    int32_t* ipiv = B.ipiv[sid];
    const int nb = (int)min((int64_t)GK, n - k);
    __shared__ T s_val[PANEL_THREADS / 32];
    __shared__ int64_t s_idx[PANEL_THREADS / 32];
    __shared__ int64_t s_piv;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int jj = 0; jj < nb; jj++) {
        const int64_t col = k + jj;
        T* c = A + col * ld;
        T best = (T)-1;
        int64_t bi = col;
        for (int64_t r = col + tid; r < n; r += PANEL_THREADS) {
            T v = tabs(c[r]);
            if (v > best) { best = v; bi = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            T ov = __shfl_down_sync(0xffffffffu, best, o);
            int64_t oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { s_val[wid] = best; s_idx[wid] = bi; }
        __syncthreads();
        if (tid == 0) {
            T bv = s_val[0];
            int64_t bix = s_idx[0];
            for (int w = 1; w < PANEL_THREADS / 32; w++) {
                if (s_val[w] > bv || (s_val[w] == bv && s_idx[w] < bix)) { bv = s_val[w]; bix = s_idx[w]; }
            }
            s_piv = bix;
            ipiv[col] = (int32_t)bix;
            if (c[bix] == (T)0 && B.info[sid] == 0) B.info[sid] = (int32_t)(col + 1);
        }
        __syncthreads();
        const int64_t p = s_piv;
        if (p != col) {
            for (int t = tid; t < nb; t += PANEL_THREADS) {
                T* a = A + (k + t) * ld;
                T tmp = a[col];
                a[col] = a[p];
                a[p] = tmp;
            }
        }
        __syncthreads();
        const T d = c[col];
        if (d != (T)0) {
            for (int64_t r = col + 1 + tid; r < n; r += PANEL_THREADS) c[r] = c[r] / d;
        }
        __syncthreads();
        for (int64_t r = col + 1 + tid; r < n; r += PANEL_THREADS) {
            const T l = c[r];
            for (int t = jj + 1; t < nb; t++) {
                T* a = A + (k + t) * ld;
                a[r] -= l * a[col];
            }
        }
        __syncthreads();
    }
}

// Panel factorisation with the panel held in registers.  The panel (rows
// k..n-1, nb <= GK columns) is split over `csize` CTAs of a thread-block
// cluster (csize = 1: one CTA), CTA q owning rows [q*slab, (q+1)*slab) with
// slab <= NT; thread t owns row q*slab + t and keeps its nb columns in
// registers.
//
// Rows are never moved during the factorisation.  Each row carries its
// logical position (LAPACK's row order after the interchanges so far); the
// interchange jj <-> p only swaps two logical positions, and every row is
// written to its final logical position at the end.  Rows whose logical
// position is below jj are finished (pivot rows = rows of U).
//
// Per column jj, one CTA barrier (plus one cluster barrier when csize > 1,
// before which every CTA has pushed its candidate into all the others):
//   1. each warp reduces its candidates (largest |a|, smallest logical
//      position on ties, like LAPACK i?amax) with redux.sync; the winning
//      lane publishes its whole row in shared memory;
//   2. barrier; every warp reduces the warp candidates of its CTA (and, in a
//      cluster, the CTA candidates read over DSMEM) and finds the pivot
//      row in shared memory;
//   3. each active row is scaled and updated with the pivot row read as
//      16-byte broadcasts (the same address in every lane); the candidate
//      for column jj+1 comes out of the same pass.
// Candidate slots and published rows are double-buffered on jj, so a slot is
// rewritten only after every reader has passed the next barrier.
template <class T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4_16a; };

// Pivot candidates as unsigned keys compared lexicographically, so a warp
// picks its winner with redux.sync max: first the magnitude (IEEE bits of |a|
// plus one, order-preserving for non-negative numbers; NaN -> 0 ranks below
// every number; 0 -> no candidate), then the inverted logical position
// (largest |a|, then smallest position, like LAPACK i?amax).
template <class T> struct PivKey;
template <> struct PivKey<float> {
    uint32_t m, l;
    __device__ __forceinline__ static PivKey make(float x, int lid) {
        const float a = fabsf(x);
        return {a == a ? __float_as_uint(a) + 1u : 0u, ~(uint32_t)lid};
    }
    __device__ __forceinline__ static PivKey none() { return {0u, 0u}; }
    // warp-wide maximum, every lane gets it
    __device__ __forceinline__ PivKey warp_max() const {
        const uint32_t mm = __reduce_max_sync(0xffffffffu, m);
        const uint32_t ll = __reduce_max_sync(0xffffffffu, m == mm ? l : 0u);
        return {mm, ll};
    }
    __device__ __forceinline__ bool operator==(const PivKey& o) const { return m == o.m && l == o.l; }
    __device__ __forceinline__ int pos() const { return (int)~l; }
    __device__ __forceinline__ static PivKey kmax(const PivKey& a, const PivKey& b) {
        return (a.m > b.m || (a.m == b.m && a.l > b.l)) ? a : b;
    }
};
template <> struct PivKey<double> {
    uint32_t m, m2, l;
    __device__ __forceinline__ static PivKey make(double x, int lid) {
        const double a = fabs(x);
        const unsigned long long b = (unsigned long long)__double_as_longlong(a);
        return a == a ? PivKey{(uint32_t)(b >> 32) + 1u, (uint32_t)b, ~(uint32_t)lid} : PivKey{0u, 0u, ~(uint32_t)lid};
    }
    __device__ __forceinline__ static PivKey none() { return {0u, 0u, 0u}; }
    __device__ __forceinline__ PivKey warp_max() const {
        const uint32_t mm = __reduce_max_sync(0xffffffffu, m);
        const uint32_t mm2 = __reduce_max_sync(0xffffffffu, m == mm ? m2 : 0u);
        const uint32_t ll = __reduce_max_sync(0xffffffffu, (m == mm && m2 == mm2) ? l : 0u);
        return {mm, mm2, ll};
    }
    __device__ __forceinline__ bool operator==(const PivKey& o) const { return m == o.m && m2 == o.m2 && l == o.l; }
    __device__ __forceinline__ int pos() const { return (int)~l; }
    __device__ __forceinline__ static PivKey kmax(const PivKey& a, const PivKey& b) {
        return (a.m > b.m || (a.m == b.m && (a.m2 > b.m2 || (a.m2 == b.m2 && a.l > b.l)))) ? a : b;
    }
};

// compile-time loop: f(integral_constant<int, I>) for I in [B, E)
template <int B, int E, class F>
__device__ __forceinline__ void static_for(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + 1, E>(f);
    }
}

// Shared state of the register panel (dynamic shared memory, so the
// out-of-line pivot exchange below addresses the same buffers).
template <class T, int NT, bool CLUSTER>
struct PanelSmem {
    static constexpr int NW = NT / 32;
    static constexpr int CM = CLUSTER ? PR_MAX_CLUSTER : 1;
    T s_row[2][NW][GK];  // each warp's candidate row
    T c_row[2][CM][GK];  // candidate rows pushed by the CTAs of the cluster
    PivKey<T> s_key[2][NW];
    PivKey<T> c_key[2][CM];
};

template <class T>
struct PivotOut {
    uint32_t row;  // shared-memory address of the pivot row (32 values, 16-byte aligned)
    int p;         // logical position of the pivot row
};

// pivot-row reads: the same address in every lane (a broadcast)
__device__ __forceinline__ void lds4(uint32_t a, float (&v)[4]) {
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]) : "r"(a));
}
__device__ __forceinline__ void lds4(uint32_t a, double (&v)[4]) {
    asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v[0]), "=d"(v[1]) : "r"(a));
    asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v[2]), "=d"(v[3]) : "r"(a + 16));
}
__device__ __forceinline__ float lds1(uint32_t a, float) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ double lds1(uint32_t a, double) {
    double v;
    asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(a));
    return v;
}
// reciprocal rounded to nearest, the value of 1 / d in IEEE arithmetic
__device__ __forceinline__ float rcp_rn(float d) { return __frcp_rn(d); }
__device__ __forceinline__ double rcp_rn(double d) { return __drcp_rn(d); }

// Steps 2 of a column: barrier, CTA-wide (and cluster-wide) winner, the
// pivot row's shared-memory address.  Kept out of line: called once per column from the
// unrolled column loop, it is the same code for all 32 columns.
template <class T, int NT, bool CLUSTER>
__device__ __noinline__ PivotOut<T> panel_exchange(int buf, int csize, int rank, int nwa, int wbase, int bar) {
    namespace cg = cooperative_groups;
    using Key = PivKey<T>;
    using SM = PanelSmem<T, NT, CLUSTER>;
    extern __shared__ __align__(16) unsigned char pr_smem[];
    SM& sm = *reinterpret_cast<SM*>(pr_smem);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if constexpr (CLUSTER) {
        __syncthreads();
    } else {
        // the slice's first nwa warps (warps wbase ..); the others left at
        // entry.  Barrier 1 + slice, as an immediate: the kernel then holds
        // only the barriers its slices can use
        constexpr int MS = NT >= 2 * PACK_MIN_SLICE ? NT / PACK_MIN_SLICE : 1;
        static_for<1, MS + 1>([&](auto BI) {
            constexpr int id = decltype(BI)::value;
            if (bar == id) asm volatile("bar.sync %0, %1;" ::"n"(id), "r"(nwa * 32) : "memory");
        });
    }
    const Key mine = lane < nwa ? sm.s_key[buf][wbase + lane] : Key::none();
    const Key best = mine.warp_max();
    const int w = wbase + __ffs(__ballot_sync(0xffffffffu, lane < nwa && mine == best)) - 1;
    PivotOut<T> o;
    if constexpr (CLUSTER) {
        // warp 0 pushes this CTA's candidate (key and row) into every CTA of the
        // cluster; after the cluster barrier all reads are local
        cg::cluster_group cl = cg::this_cluster();
        if (wid == 0) {
            const T v = sm.s_row[buf][w][lane];
            for (int q = 0; q < csize; q++) {
                *cl.map_shared_rank(&sm.c_row[buf][rank][lane], q) = v;
                if (lane == 0) *cl.map_shared_rank(&sm.c_key[buf][rank], q) = best;
            }
        }
        cl.sync();
        const Key ck = lane < csize ? sm.c_key[buf][lane] : Key::none();
        const Key cbest = ck.warp_max();
        const int q = __ffs(__ballot_sync(0xffffffffu, lane < csize && ck == cbest)) - 1;
        o.p = cbest.pos();
        o.row = (uint32_t)__cvta_generic_to_shared(&sm.c_row[buf][q][0]);
    } else {
        o.p = best.pos();
        o.row = (uint32_t)__cvta_generic_to_shared(&sm.s_row[buf][w][0]);
    }
    return o;
}

template <class T, int NT, bool CLUSTER, int RPT>
__global__ void __launch_bounds__(NT) k_panel_reg(LuBatch<T> B, int64_t k, const int32_t* act, int slab, int trim,
                                                   const int32_t* pack, int count) {
    namespace cg = cooperative_groups;
    using Key = PivKey<T>;
    using SM = PanelSmem<T, NT, CLUSTER>;
    extern __shared__ __align__(16) unsigned char pr_smem[];
    SM& sm = *reinterpret_cast<SM*>(pr_smem);
    int csize = 1, rank = 0;
    if constexpr (CLUSTER) {
        csize = (int)cg::this_cluster().num_blocks();
        rank = (int)cg::this_cluster().block_rank();
    }
    // one CTA: one system, or (pack) P systems side by side in slices of
    // NT / P threads, each with its own barrier; the launch is sized for the
    // group's tallest system, and a warp without rows of its system leaves
    // at once (the per-column barrier counts the remaining warps)
    int sidx = blockIdx.x / csize, snt = NT, slice = 0;
    if constexpr (!CLUSTER) {
        if (pack) {
            const int P = pack[2 * blockIdx.x + 1];
            snt = NT / P;
            slice = (int)threadIdx.x / snt;
            sidx = pack[2 * blockIdx.x] + slice;
            if (sidx >= count) return;  // a slice of the last CTA without a system
        }
    }
    const int32_t sid = act[sidx];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    int32_t* ipiv = B.ipiv[sid];
    int zero_col = -1;  // first exactly zero pivot of this panel (thread 0 of rank 0)
    const int nb = (int)min((int64_t)GK, n - k);
    const int rows = (int)(n - k);
    const int tid = (int)threadIdx.x - slice * snt, lane = tid & 31;  // tid: within the slice
    const int wbase = slice * (snt >> 5), wid = wbase + (tid >> 5);    // wid: the CTA's warp
    const int bar = 1 + slice;
    int nwa = snt >> 5;
    if constexpr (!CLUSTER) {
        if (trim) {
            nwa = (min(rows, snt) + 31) >> 5;
            if (wid - wbase >= nwa) return;
        }
    }

    // own rows: slab-relative tid, tid + NT, ...; lid = logical position, -1: no row
    int lid[RPT];
    T x[RPT][GK];
#pragma unroll
    for (int i = 0; i < RPT; i++) {
        const int rr = tid + i * snt, r = rank * slab + rr;
        lid[i] = ((CLUSTER ? rr < slab : rr < snt) && r < rows) ? r : -1;
        const T* src = A + (k + r) + k * ld;
#pragma unroll
        for (int t = 0; t < GK; t++) x[i][t] = (lid[i] >= 0 && t < nb) ? src[t * ld] : (T)0;
    }
    Key cand = Key::none();  // best candidate of the own rows for the current column
#pragma unroll
    for (int i = 0; i < RPT; i++)
        if (lid[i] >= 0) cand = Key::kmax(cand, Key::make(x[i][0], lid[i]));

    static_for<0, GK>([&](auto JJ) {
        constexpr int jj = decltype(JJ)::value;
        if (jj < nb) {
            const int buf = jj & 1;
            // 1. warp candidate; its owner publishes the row
            {
                const Key w = cand.warp_max();
                if (cand == w) {
#pragma unroll
                    for (int i = 0; i < RPT; i++)
                        if (lid[i] >= 0 && lid[i] == w.pos()) {
                            using V2 = typename Vec4<T>::type;
#pragma unroll
                            for (int t = 0; t < GK; t += 4) {
                                V2 v;
                                v.x = x[i][t];
                                v.y = x[i][t + 1];
                                v.z = x[i][t + 2];
                                v.w = x[i][t + 3];
                                *reinterpret_cast<V2*>(&sm.s_row[buf][wid][t]) = v;
                            }
                        }
                }
                if (lane == 0) sm.s_key[buf][wid] = w;
            }
            // 2. pivot: (p, row) known to every warp
            const PivotOut<T> po = panel_exchange<T, NT, CLUSTER>(buf, csize, rank, nwa, wbase, bar);
            const int p = po.p;
            const T d = lds1(po.row + jj * (uint32_t)sizeof(T), T(0));
            if (tid == 0 && rank == 0) {
                ipiv[k + jj] = (int32_t)(k + p);  // a store: nothing waits on it
                if (d == (T)0 && zero_col < 0) zero_col = jj;
            }
            // 3. interchange of logical positions jj <-> p, then scale and update;
            // scaling by the reciprocal of the pivot (LAPACK ?getf2), dividing when it is subnormal
            const bool big = tabs(d) >= (sizeof(T) == 4 ? (T)FLT_MIN : (T)DBL_MIN);
            const T rd = big ? rcp_rn(d) : (T)0;
            T lm[RPT];
            bool active[RPT];
#pragma unroll
            for (int i = 0; i < RPT; i++) {
                if (lid[i] == p) lid[i] = jj;
                else if (lid[i] == jj) lid[i] = p;
                active[i] = lid[i] > jj;
                lm[i] = x[i][jj];
                if (active[i]) {
                    if (big) lm[i] = lm[i] * rd;
                    else if (d != (T)0) lm[i] = lm[i] / d;
                    x[i][jj] = lm[i];
                }
            }
            // the pivot row's columns jj+1.. as 16-byte broadcasts from shared memory
#pragma unroll
            for (int tg = (jj + 1) & ~3; tg < GK; tg += 4) {
                T u[4];
                lds4(po.row + tg * (uint32_t)sizeof(T), u);
#pragma unroll
                for (int e = 0; e < 4; e++)
                    if (tg + e > jj) {
#pragma unroll
                        for (int i = 0; i < RPT; i++)
                            if (active[i]) x[i][tg + e] -= lm[i] * u[e];
                    }
            }
            if constexpr (jj + 1 < GK) {
                cand = Key::none();
#pragma unroll
                for (int i = 0; i < RPT; i++)
                    if (active[i]) cand = Key::kmax(cand, Key::make(x[i][jj + 1], lid[i]));
            }
        }
    });
    if constexpr (CLUSTER) cg::this_cluster().sync();  // no CTA leaves while its rows may still be read
    // panels of a system run in order, so the first zero pivot recorded is the first of the factorisation
    if (zero_col >= 0) atomicCAS(&B.info[sid], 0, (int32_t)(k + zero_col + 1));
    if (B.mv) {  // the panel's row moves, for the other columns of the outer block
        int32_t* mv = B.mv + (int64_t)sid * 64;
#pragma unroll
        for (int i = 0; i < RPT; i++)
            if (lid[i] >= 0) {
                const int r = rank * slab + tid + i * snt;
                if (lid[i] < GK) mv[lid[i]] = r;
                if (r < GK) mv[GK + r] = lid[i];
            }
    }
#pragma unroll
    for (int i = 0; i < RPT; i++)
        if (lid[i] >= 0) {
            T* dst = A + (k + lid[i]) + k * ld;
#pragma unroll
            for (int t = 0; t < GK; t++)
                if (t < nb) dst[t * ld] = x[i][t];
        }
}

// ---------------------------------------------------------------------------
// swap: one thread per column outside the panel, per system.  col table:
// blocks enumerated through prefix pfx (over act).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_block(const int64_t* pfx, int cnt, int64_t b) {
    int lo = 0, hi = cnt - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pfx[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <class T>
__global__ void k_swap(LuBatch<T> B, int64_t k, const int32_t* act, const int64_t* pfx, int cnt) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t tot = pfx[cnt];
    if (g >= tot) return;
    const int a = find_block(pfx, cnt, g);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    const int nb = (int)min((int64_t)GK, n - k);
    int64_t j = g - pfx[a];  // 0 .. n-nb-1
    if (j >= k) j += nb;     // skip the panel columns
    T* col = B.A[sid] + j * ld;
    const int32_t* ip = B.ipiv[sid];
    for (int t = 0; t < nb; t++) {
        const int64_t r = k + t, p = ip[r];
        if (p != r) {
            T tmp = col[r];
            col[r] = col[p];
            col[p] = tmp;
        }
    }
}

// Interchanges of rows [r_lo, min(n, r_hi)) applied to the columns
// [a_lo, min(n, a_hi)) and [min(n, b_lo), min(n, b_hi)) of every system, one
// thread per column (two-level blocking: inner swaps stay inside the outer
// panel, the outer block's swaps reach the other columns in one pass).
template <class T>
__global__ void __launch_bounds__(SW2_THREADS) k_swap2(LuBatch<T> B, const int32_t* act, const int64_t* pfx, int cnt,
                                                      int64_t r_lo, int64_t r_hi, int64_t a_lo, int64_t a_hi,
                                                      int64_t b_lo, int64_t b_hi) {
    // a CTA owns SW2_THREADS columns of one system (pfx: CTAs per system);
    // it stages the block's pivots once, and leaves when none moved a row
    // (a diagonally dominant AIC keeps every row in place)
    __shared__ int32_t s_ip[LU_OUTER];
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    const int32_t* ip = B.ipiv[sid];
    const int nr = (int)(min(n, r_hi) - r_lo);
    int moved = 0;
    for (int t = threadIdx.x; t < nr; t += SW2_THREADS) {
        const int32_t p = ip[r_lo + t];
        s_ip[t] = p;
        moved |= p != (int32_t)(r_lo + t);
    }
    if (!__syncthreads_or(moved)) return;
    const int64_t na = max((int64_t)0, min(n, a_hi) - a_lo);
    const int64_t ncols = na + (n - min(n, b_lo));
    int64_t j = (int64_t)(blockIdx.x - pfx[a]) * SW2_THREADS + threadIdx.x;
    if (j >= ncols) return;
    j = j < na ? a_lo + j : min(n, b_lo) + (j - na);
    T* col = B.A[sid] + j * ld;
    for (int t = 0; t < nr; t++) {
        const int64_t r = r_lo + t, p = s_ip[t];
        if (p != r) {
            const T tmp = col[r];
            col[r] = col[p];
            col[p] = tmp;
        }
    }
}

// ---------------------------------------------------------------------------
// trsm: U12 = L11^-1 A12, one thread per column, TRSM_COLS columns per block
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(TRSM_COLS) k_trsm(LuBatch<T> B, int64_t k, const int32_t* act, const int64_t* pfx,
                                                   int cnt, int64_t c_hi) {
    __shared__ T L[GK][GK + 1];
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    const int nb = (int)min((int64_t)GK, n - k);
    staged_copy<8>(
        nb * nb, threadIdx.x, blockDim.x, [&](int64_t t) { return A[(k + t % nb) + (k + t / nb) * ld]; },
        [&](int64_t t, T v) { L[t % nb][t / nb] = v; });
    __syncthreads();
    const int64_t j = k + nb + (int64_t)(blockIdx.x - pfx[a]) * TRSM_COLS + threadIdx.x;
    if (j >= min(n, c_hi)) return;
    T x[GK];
    T* col = A + j * ld + k;
#pragma unroll
    for (int r = 0; r < GK; r++) x[r] = r < nb ? col[r] : (T)0;
#pragma unroll
    for (int r = 1; r < GK; r++) {
        if (r < nb) {
            T s = x[r];
#pragma unroll
            for (int l = 0; l < r; l++) s -= L[r][l] * x[l];
            x[r] = s;
        }
    }
#pragma unroll
    for (int r = 0; r < GK; r++)
        if (r < nb) col[r] = x[r];
}

// ---------------------------------------------------------------------------
// two-level blocking, end of an outer block [k0, k0 + WW): U12 = L11^-1 A12
// for the columns right of the block, L11 the WW x WW unit lower triangle.
// One CTA per COLS (64, or 32 on the identity) columns: L11 and the columns
// in shared memory, solved in 32-row blocks:
//   * diagonal block: a lane per row holding its row of the 32 x 32 block
//     in registers, COLS / 8 columns in flight per warp;
//   * rows below: thread (column j, row group g) keeps the 32 solved values
//     of column j in registers and sweeps rows g, g+4, ... with the L rows
//     read as float4 broadcasts.
// ---------------------------------------------------------------------------
constexpr int TW_COLS = 64;
constexpr int TW_LS = LU_OUTER + 4;  // L row stride (float4-aligned rows)

template <int WW, int COLS = TW_COLS>
constexpr size_t trsm_wide_smem() { return sizeof(float) * ((size_t)WW * TW_LS + (size_t)WW * (COLS + 1)); }

// U12 through the explicit inverse for every system (GBVLM_TC_TRSM=0: the
// triangular solve).  It stages each L11 once instead of once per 64 columns,
// which saves SM time in a batch (config D: 249,600 -> 256,300 solves/s);
// for one large system its two dependent launches add latency to the
// critical path (config C: 88.8 -> 90.3 ms).  The choice does not depend on
// what else is in the batch, so a system's factors are the same alone and in
// any batch.
constexpr int TC_TRSM_MIN_SYSTEMS = 1;

// INV: the same solve on the identity, two CTAs per system (64 columns
// each): writes M = I - L11^-1 (strictly lower, column-major, ld WW) to
// minv + (sid - base) * WW * WW, for U12 = A12 - M A12 on the tensor cores
template <int WW, bool INV = false, int COLS = TW_COLS>
__global__ void __launch_bounds__(256, 2) k_trsm_wide(LuBatch<float> B, int64_t k0, const int32_t* act,
                                                     const int64_t* pfx, int cnt, float* minv, int32_t base) {
    static_assert(WW == LU_OUTER, "row stride sized for the outer block");
    static_assert(COLS == 64 || COLS == 32, "eight warps of COLS / 8 columns");
    constexpr int TW_XS = COLS + 1;      // X row stride (odd: conflict-free columns)
    constexpr int CPW = COLS / 8;        // columns per warp on the diagonal block
    constexpr int CTAS = WW / COLS;      // CTAs per system on the identity
    extern __shared__ __align__(16) float tw_smem[];
    float* L = tw_smem;            // L[r * TW_LS + c]
    float* X = L + WW * TW_LS;     // X[r * TW_XS + j]
    const int a = INV ? (int)(blockIdx.x / CTAS) : find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    float* A = B.A[sid];
    // columns of A12 (systems here have n > k0 + WW), or of the identity
    const int64_t c0 = INV ? (int64_t)(blockIdx.x % CTAS) * COLS : k0 + WW + (int64_t)(blockIdx.x - pfx[a]) * COLS;
    const int ncols = INV ? COLS : (int)min((int64_t)COLS, n - c0);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const float* Ab = A + k0 + k0 * ld;
    // on the identity the CTA reads L11 only from its first column block on
    const int cs = INV ? (int)c0 : 0;
    staged_copy<16>(
        WW * WW, tid, 256,
        [&](int64_t e) {
            const int r = (int)(e & (WW - 1)), c = (int)(e >> 7);
            return (r >= cs && c >= cs) ? Ab[r + c * ld] : 0.f;
        },
        [&](int64_t e, float v) { L[(int)(e & (WW - 1)) * TW_LS + (int)(e >> 7)] = v; });
    if constexpr (INV) {
        for (int e = tid; e < WW * COLS; e += 256) {
            const int r = e & (WW - 1), j = e >> 7;
            X[r * TW_XS + j] = (r == (int)c0 + j) ? 1.f : 0.f;
        }
    } else {
        const float* Xb = A + k0 + c0 * ld;
        staged_copy<16>(
            WW * COLS, tid, 256,
            [&](int64_t e) { return (int)(e >> 7) < ncols ? Xb[(int)(e & (WW - 1)) + (e >> 7) * ld] : 0.f; },
            [&](int64_t e, float v) { X[(int)(e & (WW - 1)) * TW_XS + (int)(e >> 7)] = v; });
    }
    __syncthreads();
    // on the identity, rows above the CTA's first column stay zero: start there
#pragma unroll 1
    for (int b = INV ? (int)(c0 / 32) : 0; b < WW / 32; b++) {
        const int rb = 32 * b;
        // diagonal block
        {
            float lrow[32];
#pragma unroll
            for (int l = 0; l < 32; l++) lrow[l] = L[(rb + lane) * TW_LS + rb + l];
            // warp w: columns CPW w .. CPW w + CPW - 1, all in flight
            const int j0 = CPW * wid;
            float x[CPW];
#pragma unroll
            for (int c = 0; c < CPW; c++) x[c] = X[(rb + lane) * TW_XS + j0 + c];
#pragma unroll
            for (int l = 0; l < 32; l++) {
#pragma unroll
                for (int c = 0; c < CPW; c++) {
                    const float xl = __shfl_sync(0xffffffffu, x[c], l);
                    if (lane > l) x[c] -= lrow[l] * xl;
                }
            }
#pragma unroll
            for (int c = 0; c < CPW; c++) X[(rb + lane) * TW_XS + j0 + c] = x[c];
        }
        __syncthreads();
        // rows below the block
        if (rb + 32 < WW) {
            constexpr int RG = 256 / COLS;  // row groups
            const int j = tid & (COLS - 1), g = tid / COLS;
            float xb[32];
#pragma unroll
            for (int l = 0; l < 32; l++) xb[l] = X[(rb + l) * TW_XS + j];
#pragma unroll 1
            for (int r = rb + 32 + g; r < WW; r += RG) {
                const float4* lr = reinterpret_cast<const float4*>(L + r * TW_LS + rb);
                float acc = 0.f;
#pragma unroll
                for (int m = 0; m < 8; m++) {
                    const float4 v = lr[m];
                    acc += v.x * xb[4 * m] + v.y * xb[4 * m + 1] + v.z * xb[4 * m + 2] + v.w * xb[4 * m + 3];
                }
                X[r * TW_XS + j] -= acc;
            }
        }
        __syncthreads();
    }
    if constexpr (INV) {
        float* Mo = minv + (int64_t)(sid - base) * WW * WW + c0 * WW;
        for (int e = tid; e < WW * COLS; e += 256) {
            const int r = e & (WW - 1), j = e >> 7;
            Mo[r + j * WW] = r > (int)c0 + j ? -X[r * TW_XS + j] : 0.f;
        }
    } else {
        float* Xo = A + k0 + c0 * ld;
        for (int e = tid; e < WW * COLS; e += 256) {
            const int r = e & (WW - 1), j = e >> 7;
            if (j < ncols) Xo[r + (int64_t)j * ld] = X[r * TW_XS + j];
        }
    }
}

// The inner update of the two-level factorisation on the tensor cores: after
// the 32-column panel [k, k + 32) of the outer block [.., kend), rows and
// columns [k + 32, min(n, kend)) -= L21 U12 with K = 32, one 128-row tile of
// at most 96 columns per CTA (the CUDA-core k_update in mode 1 does the same
// in 64 x 64 tiles)
template <int PASSES>
__global__ void __launch_bounds__(tc::THREADS, 2) k_inner_tc(LuBatch<float> B, int64_t k, int64_t kend,
                                                             const int32_t* act, const int64_t* pfx, int cnt,
                                                             int* err) {
    extern __shared__ __align__(16) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tslot;
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    float* A = B.A[sid];
    const int64_t lo = k + GK, ke = min(n, kend);
    const int64_t r0 = lo + (int64_t)(blockIdx.x - pfx[a]) * tc::BM;
    tc::update_tile<PASSES, false, tc::BN>(A + r0 + k * ld, ld, A + k + lo * ld, ld, A + r0 + lo * ld, ld,
                                           (int)min((int64_t)tc::BM, n - r0), (int)(ke - lo), GK, tc_smem, bar,
                                           &tslot, err);
}

// U12 = L11^-1 A12 = A12 - M A12 (M = I - L11^-1 from k_trsm_wide<.., true>)
// in place, on the tensor cores: one 128-row tile of TBN columns of A12 per
// CTA.  The tile's operand chunks are all read before its epilogue writes,
// and tiles own disjoint columns.
template <int PASSES, int TBN>
__global__ void __launch_bounds__(tc::THREADS, 2) k_trsm_tc12(LuBatch<float> B, int64_t k0, const int32_t* act,
                                                              const int64_t* pfx, int cnt, const float* minv,
                                                              int32_t base, int* err) {
    extern __shared__ __align__(16) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tslot;
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    float* A = B.A[sid];
    const int64_t c0 = k0 + LU_OUTER + (int64_t)(blockIdx.x - pfx[a]) * TBN;
    const float* M = minv + (int64_t)(sid - base) * LU_OUTER * LU_OUTER;
    float* X = A + k0 + c0 * ld;
    tc::update_tile<PASSES, false, TBN>(M, LU_OUTER, X, ld, X, ld, LU_OUTER, (int)min((int64_t)TBN, n - c0), LU_OUTER,
                                        tc_smem, bar, &tslot, err);
}

// ---------------------------------------------------------------------------
// inner step of the two-level float factorisation, after the panel of
// columns [k, k + nb) inside the outer block [k0, kend): for the outer
// block's other columns, the panel's row moves (from the move lists the
// panel wrote: LAPACK's sequential interchanges composed) and the U rows
// U12 = L11^-1 A12 right of the panel; the update of the rows below follows
// in 64 x 64 tiles (k_update).  A CTA owns IN_COLS columns of one system:
// warp c, lane t holds column c, row t of the 32 moved rows; all moved values
// are read before any is written (a pivot row's old place receives a
// displaced top row), and the U rows are solved by shuffles down the warp.
// (Updating the rows below here as well, a thread per row, measured slower:
// it costs more SM time than the tiles.)
// ---------------------------------------------------------------------------
constexpr int IN_COLS = 16;
constexpr int IN_THREADS = 512;  // IN_COLS warps of 32 rows

__global__ void __launch_bounds__(IN_THREADS) k_inner(LuBatch<float> B, int64_t k, int64_t k0, int64_t kend,
                                                     const int32_t* act, const int64_t* pfx, int cnt) {
    __shared__ float L11[GK][GK + 1];
    __shared__ int32_t msrc[GK], mdst[GK];
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    float* A = B.A[sid];
    const int nb = (int)min((int64_t)GK, n - k);  // rows k .. k + nb - 1 and their pivots move
    // chunks: the columns left of the panel [k0, k), then right of it [k + nb, min(n, kend))
    const int64_t nleft = k - k0;
    const int64_t cidx = (int64_t)(blockIdx.x - pfx[a]) * IN_COLS;
    const bool right = cidx >= nleft;
    const int64_t c0 = right ? k + nb + (cidx - nleft) : k0 + cidx;
    const int cw = (int)min((int64_t)IN_COLS, (right ? min(n, kend) : k) - c0);
    const int tid = threadIdx.x, t = tid & 31, c = tid >> 5;
    int moved = 0;
    if (tid < GK) {
        const int32_t* mv = B.mv + (int64_t)sid * 64;
        msrc[tid] = tid < nb ? mv[tid] : tid;
        mdst[tid] = tid < nb ? mv[GK + tid] : tid;
        moved = msrc[tid] != tid || mdst[tid] != tid;
    }
    if (right)
        for (int e = tid; e < GK * GK; e += IN_THREADS) {
            const int rr = e & (GK - 1), cc = e >> 5;
            L11[rr][cc] = rr < nb && cc < nb ? A[(k + rr) + (k + cc) * ld] : 0.f;
        }
    // a chunk left of the panel only takes the row moves: none, nothing to do
    if (!__syncthreads_or(moved) && !right) return;
    const bool live = c < cw && t < nb;
    float* col = A + (c0 + c) * ld;
    float top = 0.f, out = 0.f;
    if (live) {
        top = col[k + msrc[t]];  // the row that ends at k + t
        out = col[k + t];        // the row that starts at k + t
    }
    __syncthreads();  // every moved value read before any is written
    if (live && mdst[t] >= GK) col[k + mdst[t]] = out;
    if (right) {
#pragma unroll
        for (int r = 0; r < GK; r++) {
            const float xr = __shfl_sync(0xffffffffu, top, r);
            if (t > r) top -= L11[t][r] * xr;
        }
    }
    if (live) col[k + t] = top;
}

// ---------------------------------------------------------------------------
// update: A22 -= L21 * U12 on 64x64 tiles, 256 threads, each a 4x4 block of
// consecutive rows/columns read from shared memory as vectors
// ---------------------------------------------------------------------------

// mode 0: the whole trailing matrix, rows and columns [k+GK, n).
// mode 1 (two-level blocking, outer block ending at column kend): only the
// outer panel's columns [k+GK, min(n, kend)) over rows [k+GK, n); the columns
// right of the block wait for the block's swaps, U12 solve and tensor-core
// update.
template <class T>
__global__ void __launch_bounds__(256) k_update(LuBatch<T> B, int64_t k, const int32_t* act, const int64_t* pfx,
                                               int cnt, int64_t kend, int mode) {
    constexpr int SW = GT + 4;  // row stride keeps 16-byte alignment of every 4-run
    __shared__ __align__(16) T sA[GK][SW];  // L21 tile: [kk][row]
    __shared__ __align__(16) T sB[GK][SW];  // U12 tile: [kk][col]
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    const int64_t lo = k + GK;  // systems here have n > k + GK
    const int64_t t = blockIdx.x - pfx[a];
    int64_t r0, c0, row_hi = n, col_hi = n;
    if (mode == 0) {
        const int64_t tiles = (n - lo + GT - 1) / GT;
        r0 = lo + (t % tiles) * GT;
        c0 = lo + (t / tiles) * GT;
    } else {
        const int64_t ke = min(n, kend);
        const int64_t tr = (n - lo + GT - 1) / GT;
        r0 = lo + (t % tr) * GT;
        c0 = lo + (t / tr) * GT;
        col_hi = ke;
    }
    const int tid = threadIdx.x;
    {
        constexpr int PER = GK * GT / 256;  // elements of each tile per thread
        T va[PER], vb[PER];
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int e = tid + u * 256;
            const int64_t r = r0 + e % GT, c = c0 + e / GK;
            va[u] = r < row_hi ? A[r + (k + e / GT) * ld] : (T)0;
            vb[u] = c < col_hi ? A[(k + e % GK) + c * ld] : (T)0;
        }
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int e = tid + u * 256;
            sA[e / GT][e % GT] = va[u];
            sB[e % GK][e / GK] = vb[u];
        }
    }
    __syncthreads();
    const int tx = tid & 15, ty = tid >> 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0;
    using V = typename Vec4<T>::type;
#pragma unroll 8
    for (int kk = 0; kk < GK; kk++) {
        const V av = *reinterpret_cast<const V*>(&sA[kk][4 * tx]);
        const V bv = *reinterpret_cast<const V*>(&sB[kk][4 * ty]);
        const T a4[4] = {av.x, av.y, av.z, av.w}, b4[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] += a4[i] * b4[j];
    }
    // all 16 loads of the output block before its stores
    T cur[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int64_t c = c0 + 4 * ty + j;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int64_t r = r0 + 4 * tx + i;
            cur[i][j] = (c < col_hi && r < row_hi) ? A[r + c * ld] : (T)0;
        }
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int64_t c = c0 + 4 * ty + j;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int64_t r = r0 + 4 * tx + i;
            if (c < col_hi && r < row_hi) A[r + c * ld] = cur[i][j] - acc[i][j];
        }
    }
}

// ---------------------------------------------------------------------------
// update on the tensor cores: the same A22 -= L21 U12 on 128 x 128 tiles
// (gbvlm_tc.cuh), tiles enumerated over all systems through a prefix table
// ---------------------------------------------------------------------------
template <int PASSES, int TBN>
__global__ void __launch_bounds__(tc::THREADS, 2) k_update_tc(LuBatch<float> B, int64_t k0, int w, const int32_t* act,
                                                             const int64_t* pfx, int cnt, int* err, int part) {
    // outer update of the block [k0, k0 + w): rows and columns [k0 + w, n), K = w.
    // part 0: all tiles; part 1: the first column of tiles (the next outer
    // panel, w = 128 columns, TBN = 128); part 2: the columns right of it.
    // Tiles are 128 rows x TBN columns, row tiles fastest.
    extern __shared__ __align__(16) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tslot;
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    float* A = B.A[sid];
    const int64_t lo = k0 + w;  // systems here have n > k0 + w
    const int64_t tiles = (n - lo + tc::BM - 1) / tc::BM;
    const int64_t t = blockIdx.x - pfx[a];
    const int64_t cbase = lo + (part == 2 ? (int64_t)tc::BN : 0);
    const int64_t r0 = lo + (t % tiles) * tc::BM, c0 = cbase + (t / tiles) * TBN;
    tc::update_tile<PASSES, false, TBN>(A + r0 + k0 * ld, ld, A + k0 + c0 * ld, ld, A + r0 + c0 * ld, ld,
                                        (int)min((int64_t)tc::BM, n - r0), (int)min((int64_t)TBN, n - c0), w, tc_smem,
                                        bar, &tslot, err);
}

// persistent warp-specialised form of k_update_tc (gbvlm_tc.cuh): one CTA per
// SM over the same tile list; tile blk of the launch is prefix block blk
template <int PASSES>
__global__ void __launch_bounds__(tc::P_THREADS, 1) k_update_tcp(LuBatch<float> B, int64_t k0, int w, const int32_t* act,
                                                                const int64_t* pfx, int cnt, int* err, int part,
                                                                int64_t ntiles) {
    extern __shared__ __align__(16) unsigned char tc_smem[];
    auto job = [&](int64_t blk) {
        const int a = find_block(pfx, cnt, blk);
        const int32_t sid = act[a];
        const int64_t n = B.n[sid], ld = B.ld[sid];
        float* A = B.A[sid];
        const int64_t lo = k0 + w;
        const int64_t tiles = (n - lo + tc::BM - 1) / tc::BM;
        const int64_t t = blk - pfx[a] + (part == 2 ? tiles : 0);
        const int64_t r0 = lo + (t % tiles) * tc::BM, c0 = lo + (t / tiles) * tc::BN;
        tc::TileJob J;
        J.Lp = A + r0 + k0 * ld;
        J.ldl = ld;
        J.Up = A + k0 + c0 * ld;
        J.ldu = ld;
        J.Cp = A + r0 + c0 * ld;
        J.ldc = ld;
        J.m_rows = (int)min((int64_t)tc::BM, n - r0);
        J.n_cols = (int)min((int64_t)tc::BN, n - c0);
        J.K = w;
        return J;
    };
    tc::update_persistent<PASSES>(ntiles, job, tc_smem, err);
}

// ---------------------------------------------------------------------------
// row permutation of a finished factorisation: perm[r] = original row that
// ends up in position r (the ipiv interchanges composed in order)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_perm(LuBatch<T> B, int32_t base) {
    extern __shared__ int32_t sp[];
    const int32_t sid = base + blockIdx.x;
    const int64_t n = B.n[sid];
    const int32_t* ip = B.ipiv[sid];
    int32_t* pm = B.perm[sid];
    if (n <= PERM_SMEM) {
        for (int64_t r = threadIdx.x; r < n; r += blockDim.x) sp[r] = (int32_t)r;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int64_t r = 0; r < n; r++) {
                const int32_t p = ip[r];
                const int32_t t = sp[r];
                sp[r] = sp[p];
                sp[p] = t;
            }
        }
        __syncthreads();
        for (int64_t r = threadIdx.x; r < n; r += blockDim.x) pm[r] = sp[r];
    } else {
        for (int64_t r = threadIdx.x; r < n; r += blockDim.x) pm[r] = (int32_t)r;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int64_t r = 0; r < n; r++) {
                const int32_t p = ip[r];
                const int32_t t = pm[r];
                pm[r] = pm[p];
                pm[p] = t;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// triangular solves, one CTA per system and block of up to TS_MAXRHS
// right-hand sides held in shared memory (n * nrhs values).  The diagonal
// blocks are solved one warp per right-hand side, a lane per row: after
// row r is final, lanes below subtract L[l][r] x_r in parallel.
// ---------------------------------------------------------------------------
constexpr int TS_THREADS = 512;
constexpr int TS_MAXRHS = 8;

// acc[q] = sum_l a[l * ld] * xs[l][q] over the nb <= GK columns of a block row;
// a full block issues all GK loads before the first use
template <class T>
__device__ __forceinline__ void trs_row_dot(const T* a, int64_t ld, int nb, const T (*xs)[TS_MAXRHS],
                                            T (&acc)[TS_MAXRHS]) {
#pragma unroll
    for (int q = 0; q < TS_MAXRHS; q++) acc[q] = 0;
    if (nb == GK) {
        T v[GK];
#pragma unroll
        for (int l = 0; l < GK; l++) v[l] = a[l * ld];
#pragma unroll
        for (int l = 0; l < GK; l++)
#pragma unroll
            for (int q = 0; q < TS_MAXRHS; q++) acc[q] += v[l] * xs[l][q];
    } else {
        for (int l = 0; l < nb; l++) {
            const T v = a[l * ld];
#pragma unroll
            for (int q = 0; q < TS_MAXRHS; q++) acc[q] += v * xs[l][q];
        }
    }
}

template <class T>
__global__ void __launch_bounds__(TS_THREADS) k_trsolve(LuBatch<T> B, int32_t rhs0, int32_t nrhs_blk, int use_smem) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int32_t sid = blockIdx.x;
    rhs0 += (int32_t)blockIdx.y * nrhs_blk;  // right-hand-side block of this CTA
    const int64_t n = B.n[sid], ld = B.ld[sid];
    const T* A = B.A[sid];
    const int32_t nr = (int32_t)min((int64_t)nrhs_blk, (int64_t)B.nrhs[sid] - rhs0);
    if (nr <= 0) return;
    T* X = B.X[sid] + (int64_t)rhs0 * B.ldx[sid];
    const int64_t ldx = B.ldx[sid];
    const int32_t* pm = B.perm[sid];
    __shared__ T dg[GK][GK + 1];
    __shared__ T xs[GK][TS_MAXRHS];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // working copy of X: shared memory (n x TS_MAXRHS, row-major) or X itself after an in-place gather
    T* W = reinterpret_cast<T*>(smem_raw);
    const int64_t wld = use_smem ? 1 : ldx;     // stride between rows
    const int64_t wcs = use_smem ? TS_MAXRHS : 1;  // unused when not smem
    (void)wcs;
    auto WX = [&](int64_t r, int q) -> T& { return use_smem ? W[r * TS_MAXRHS + q] : X[r + q * ldx]; };
    if (use_smem) {
        staged_copy<8>(
            n * nr, tid, TS_THREADS, [&](int64_t e) { return X[pm[e % n] + (e / n) * ldx]; },
            [&](int64_t e, T v) { W[(e % n) * TS_MAXRHS + e / n] = v; });
    } else {
        // gather through the double-buffer-free route: rows are permuted one
        // right-hand side at a time with the CTA's shared scratch as staging
        T* stage = W;  // n entries (caller sized the shared memory for one column)
        for (int q = 0; q < nr; q++) {
            for (int64_t r = tid; r < n; r += TS_THREADS) stage[r] = X[pm[r] + q * ldx];
            __syncthreads();
            for (int64_t r = tid; r < n; r += TS_THREADS) X[r + q * ldx] = stage[r];
            __syncthreads();
        }
    }
    (void)wld;
    __syncthreads();
    // forward: L (unit lower)
    for (int64_t k = 0; k < n; k += GK) {
        const int nb = (int)min((int64_t)GK, n - k);
        staged_copy<4>(
            nb * nb, tid, TS_THREADS, [&](int64_t e) { return A[(k + e % nb) + (k + e / nb) * ld]; },
            [&](int64_t e, T v) { dg[e % nb][e / nb] = v; });
        __syncthreads();
        if (wid < nr) {
            T x = lane < nb ? WX(k + lane, wid) : (T)0;
            for (int r = 0; r < nb; r++) {
                const T xr = __shfl_sync(0xffffffffu, x, r);
                if (lane > r && lane < nb) x -= dg[lane][r] * xr;
            }
            if (lane < nb) {
                xs[lane][wid] = x;
                WX(k + lane, wid) = x;
            }
        }
        __syncthreads();
        for (int64_t r = k + nb + tid; r < n; r += TS_THREADS) {
            T acc[TS_MAXRHS];
            trs_row_dot(A + r + k * ld, ld, nb, xs, acc);
#pragma unroll
            for (int q = 0; q < TS_MAXRHS; q++)
                if (q < nr) WX(r, q) -= acc[q];
        }
        __syncthreads();
    }
    // backward: U
    const int64_t nblk = (n + GK - 1) / GK;
    for (int64_t bk = nblk - 1; bk >= 0; bk--) {
        const int64_t k = bk * GK;
        const int nb = (int)min((int64_t)GK, n - k);
        staged_copy<4>(
            nb * nb, tid, TS_THREADS, [&](int64_t e) { return A[(k + e % nb) + (k + e / nb) * ld]; },
            [&](int64_t e, T v) { dg[e % nb][e / nb] = v; });
        __syncthreads();
        if (wid < nr) {
            T x = lane < nb ? WX(k + lane, wid) : (T)0;
            for (int r = nb - 1; r >= 0; r--) {
                T xr = __shfl_sync(0xffffffffu, x, r);
                xr = xr / dg[r][r];
                if (lane == r) x = xr;
                if (lane < r) x -= dg[lane][r] * xr;
            }
            if (lane < nb) {
                xs[lane][wid] = x;
                WX(k + lane, wid) = x;
            }
        }
        __syncthreads();
        for (int64_t r = tid; r < k; r += TS_THREADS) {
            T acc[TS_MAXRHS];
            trs_row_dot(A + r + k * ld, ld, nb, xs, acc);
#pragma unroll
            for (int q = 0; q < TS_MAXRHS; q++)
                if (q < nr) WX(r, q) -= acc[q];
        }
        __syncthreads();
    }
    if (use_smem) {
        for (int64_t e = tid; e < n * nr; e += TS_THREADS) {
            const int64_t r = e % n;
            const int q = (int)(e / n);
            X[r + q * ldx] = W[r * TS_MAXRHS + q];
        }
    }
}

// ---------------------------------------------------------------------------
// dataflow triangular solves of a float batch: one persistent launch runs
// the forward (L, unit lower) and backward (U) sweeps of every system in
// blocks of FL_B rows.  Work items are (system, block) pairs handed out in a
// fixed order by an atomic counter: all forward items by block level, then
// all backward items by distance from the last block.  Item (s, i) of the
// forward sweep accumulates b_i - sum_{j<i} L_ij y_j as y_j become final,
// then solves its diagonal block; the backward sweep likewise with U and
// x_j, j > i.  A system's finished blocks are counted (forward and backward
// separately, each finishing in order), and an item waits only on items
// handed out before it, which are held by running CTAs, so the launch cannot
// deadlock whatever the number of resident CTAs.  Every wait is bounded
// (tc::WAIT_NS) and ends early once any CTA has recorded an error.
//
// One item: 256 threads; thread t holds rows t%64 and t%64+64 of the block
// and columns 32*(t/64) .. +31 of each off-diagonal FL_B x FL_B block (64
// loads issued before waiting for that block's x); the four column quarters
// are summed in shared memory at the end.  The diagonal block (the triangle
// the sweep needs) is copied to shared memory with cp.async while the
// off-diagonal blocks stream; it is solved one warp per right-hand side in
// 32-row steps.
// ---------------------------------------------------------------------------
constexpr int FL_B = 128;
constexpr int FL_SYS_BITS = 20, FL_SYS_MASK = (1 << FL_SYS_BITS) - 1;  // item: system | group << 20
constexpr int FL_THREADS = 256;
constexpr int FL_R = 8;  // right-hand sides per launch
constexpr int FL_LD = FL_B + 4;  // rows 16-byte aligned: a lane reads its row as float4, conflict-free
constexpr int FL_SMEM = (FL_B * FL_LD + 5 * FL_B * FL_R) * 4;  // diagonal block + quarter sums (x staging aliased) + the block's values

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// 4-byte cp.async; src_bytes 0 fills the destination with zero and reads nothing
__device__ __forceinline__ void cp_async4_zfill(uint32_t dst, const float* src, bool load) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(load ? 4 : 0) : "memory");
}

// all threads: true once *cnt > need; false if the launch has failed or the
// wait ran out (which records the failure)
__device__ __forceinline__ bool flow_wait(const int* cnt, int need, int* err, int* s_ok) {
    if (threadIdx.x == 0) {
        bool ok = ld_acquire_gpu(cnt) > need;
        if (!ok) {
            const uint64_t t0 = tc::global_ns();
            while (true) {
                __nanosleep(100);
                if (ld_acquire_gpu(cnt) > need) {
                    ok = true;
                    break;
                }
                if (*(volatile int*)err) break;
                if (tc::global_ns() - t0 > tc::WAIT_NS) {
                    atomicCAS(err, 0, 1);
                    break;
                }
            }
        }
        *s_ok = ok;
    }
    __syncthreads();
    const bool ok = *(volatile int*)s_ok != 0;
    __syncthreads();  // every thread has read the flag before thread 0 can write the next one
    return ok;
}

// One warp inverts the 32-row triangle sb of the diagonal block in place,
// lane j computing column j by substitution on the unit vector e_j: the
// strict lower part of L^-1 (unit lower, forward sweep) or the upper part
// with the diagonal of U^-1 (backward sweep).  Rows at or past nb are left
// zero.
__device__ __noinline__ void flow_invert_lower(float* T, int lane) {
    float t[32];
#pragma unroll
    for (int r = 0; r < 32; r++) {
        float d0 = 0.f, d1 = 0.f;
#pragma unroll
        for (int c = 0; c < 32; c++)
            if (c < r) {
                if (c & 1) d1 += T[r * FL_LD + c] * t[c];
                else d0 += T[r * FL_LD + c] * t[c];
            }
        t[r] = r < lane ? 0.f : (r == lane ? 1.f : -(d0 + d1));
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 32; r++)
        if (r > lane) T[r * FL_LD + lane] = t[r];
}

__device__ __noinline__ void flow_invert_upper(float* T, int cmax, int lane) {
    float t[32];
#pragma unroll
    for (int r = 31; r >= 0; r--) {
        float d0 = 0.f, d1 = 0.f;
#pragma unroll
        for (int c = 0; c < 32; c++)
            if (c > r) {
                if (c & 1) d1 += T[r * FL_LD + c] * t[c];
                else d0 += T[r * FL_LD + c] * t[c];
            }
        const float rd = r < cmax ? __frcp_rn(T[r * FL_LD + r]) : 0.f;
        t[r] = r > lane ? 0.f : (r == lane ? rd : -(d0 + d1) * rd);
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 32; r++)
        if (r <= lane) T[r * FL_LD + lane] = lane < cmax ? t[r] : 0.f;
}

// One warp inverts the 32-row triangle sb of the diagonal block in place,
// lane j computing column j by substitution on the unit vector e_j: the
// strict lower part of L^-1 (unit lower, forward sweep) or the upper part
// with the diagonal of U^-1 (backward sweep).  Rows at or past nb are left
// zero.
__device__ __forceinline__ void flow_invert_tri(float* Ld, int sb, int nb, bool fwd, int lane) {
    float* T = Ld + sb * 32 * FL_LD + sb * 32;  // T[r * FL_LD + c]
    if (fwd) flow_invert_lower(T, lane);
    else flow_invert_upper(T, min(32, nb - sb * 32), lane);
}

// ctl: [0] dispatch counter, [1] error word, then per group g of FL_R
// right-hand sides: [2 + 2 g nsys, + nsys) forward blocks finished per
// system, [2 + (2 g + 1) nsys, + nsys) backward blocks finished.  An item's
// x holds its system in the low 20 bits and its group above them.
__global__ void __launch_bounds__(FL_THREADS, 2) k_trs_flow(LuBatch<float> B, const int2* items, int nfwd, int nitems,
                                                            int nsys, int* ctl, float* const* Yp, int32_t rhs0) {
    extern __shared__ __align__(16) float fsm[];
    float* Ld = fsm;                  // [FL_B][FL_LD] diagonal block
    float* xs = fsm + FL_B * FL_LD;   // [2][FL_B][FL_R] x of an off-diagonal block (two buffers)
    float* red = xs;                  // [4][FL_B][FL_R] column-quarter sums
    float* xT = red + 4 * FL_B * FL_R;  // [FL_R][FL_B] the block's values, a right-hand side per row
    __shared__ int s_item, s_ok;
    int* err = ctl + 1;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int r = tid & 63, cq = tid >> 6;
    while (true) {
        __syncthreads();  // the previous item is done with shared memory
        if (tid == 0) s_item = *(volatile int*)err ? nitems : atomicAdd(ctl, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= nitems) return;
        const bool fwd = it < nfwd;
        const int2 w = items[it];
        const int s = w.x & FL_SYS_MASK, grp = w.x >> FL_SYS_BITS, bi = w.y;
        const int32_t r0 = rhs0 + grp * FL_R;
        int* gctl = ctl + 2 * (int64_t)grp * nsys;  // this group's progress words at gctl + 2
        const int nr = min(FL_R, B.nrhs[s] - r0);
        if (nr <= 0) continue;  // no right-hand side of this launch: no item of the system waits
        const int64_t n = B.n[s], ld = B.ld[s], ldx = B.ldx[s];
        const int nblk = (int)((n + FL_B - 1) / FL_B);
        const int64_t R0 = (int64_t)bi * FL_B;
        const int nb = (int)min((int64_t)FL_B, n - R0);
        const float* A = B.A[s];
        float* Y = Yp[(int64_t)grp * nsys + s];  // n x FL_R, row-major: y (forward), then x (backward)
        float* X = B.X[s] + (int64_t)r0 * ldx;
        int* done = gctl + 2 + (fwd ? 0 : nsys) + s;
        // diagonal block: the strict lower triangle (forward) or the upper one
        // with the diagonal (backward), zero elsewhere
        for (int e = tid; e < FL_B * FL_B; e += FL_THREADS) {
            const int rr = e & (FL_B - 1), cc = e >> 7;
            const bool need = rr < nb && cc < nb && (fwd ? cc < rr : cc >= rr);
            cp_async4_zfill(tc::smem_u32(Ld + rr * FL_LD + cc), need ? A + (R0 + rr) + (R0 + cc) * ld : A, need);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        float acc[2][FL_R];
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int q = 0; q < FL_R; q++) acc[h][q] = 0.f;
        if (fwd) {
            if (cq == 0) {  // b = P x: rows of X through the factorisation's permutation
                const int32_t* pm = B.perm[s];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int row = r + 64 * h;
                    if (row < nb) {
                        const int64_t p = pm[R0 + row];
#pragma unroll
                        for (int q = 0; q < FL_R; q++)
                            if (q < nr) acc[h][q] = X[p + q * ldx];
                    }
                }
            }
        } else {
            if (!flow_wait(gctl + 2 + s, bi, err, &s_ok)) {  // y_i
                asm volatile("cp.async.wait_group 0;" ::: "memory");  // no copy into shared memory outlives the CTA
                break;
            }
            if (cq == 0) {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int row = r + 64 * h;
                    if (row < nb) {
                        const float4* y4 = reinterpret_cast<const float4*>(Y + (R0 + row) * FL_R);
                        const float4 a = __ldcg(y4), b = __ldcg(y4 + 1);
                        acc[h][0] = a.x, acc[h][1] = a.y, acc[h][2] = a.z, acc[h][3] = a.w;
                        acc[h][4] = b.x, acc[h][5] = b.y, acc[h][6] = b.z, acc[h][7] = b.w;
                    }
                }
            }
        }
        // the diagonal block's 32-row triangles inverted in place (warp sb:
        // triangle sb) while the item may still wait for other blocks
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();
        if (wid < 4 && wid * 32 < nb) flow_invert_tri(Ld, wid, nb, fwd, lane);
        __syncthreads();
        // off-diagonal blocks, in the order their x become final
        const int nj = fwd ? bi : nblk - 1 - bi;
        bool ok = true;
        for (int t = 0; t < nj; t++) {
            const int bj = fwd ? t : nblk - 1 - t;
            const int64_t C0 = (int64_t)bj * FL_B;
            const int ncol = (int)min((int64_t)FL_B, n - C0);
            const float* a0 = A + (R0 + r) + (C0 + cq * 32) * ld;
            float v[2][32];
#pragma unroll
            for (int c = 0; c < 32; c++) {
                const bool cok = cq * 32 + c < ncol;
                v[0][c] = (cok && r < nb) ? a0[c * ld] : 0.f;
                v[1][c] = (cok && r + 64 < nb) ? a0[64 + c * ld] : 0.f;
            }
            if (!flow_wait(done, fwd ? bj : nblk - 1 - bj, err, &s_ok)) {
                ok = false;
                break;
            }
            float* xb = xs + (t & 1) * FL_B * FL_R;
            reinterpret_cast<float4*>(xb)[tid] =
                tid < 2 * ncol ? __ldcg(reinterpret_cast<const float4*>(Y + C0 * FL_R) + tid) : make_float4(0, 0, 0, 0);
            __syncthreads();
            const float4* x4 = reinterpret_cast<const float4*>(xb) + cq * 64;
#pragma unroll
            for (int c = 0; c < 32; c++) {
                const float4 xa = x4[2 * c], xb4 = x4[2 * c + 1];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    acc[h][0] -= v[h][c] * xa.x;
                    acc[h][1] -= v[h][c] * xa.y;
                    acc[h][2] -= v[h][c] * xa.z;
                    acc[h][3] -= v[h][c] * xa.w;
                    acc[h][4] -= v[h][c] * xb4.x;
                    acc[h][5] -= v[h][c] * xb4.y;
                    acc[h][6] -= v[h][c] * xb4.z;
                    acc[h][7] -= v[h][c] * xb4.w;
                }
            }
        }
        if (!ok) break;
        __syncthreads();  // x staging (aliased by the sums) no longer read
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float4* d = reinterpret_cast<float4*>(red + (cq * FL_B + r + 64 * h) * FL_R);
            d[0] = make_float4(acc[h][0], acc[h][1], acc[h][2], acc[h][3]);
            d[1] = make_float4(acc[h][4], acc[h][5], acc[h][6], acc[h][7]);
        }
        __syncthreads();
        for (int e = tid; e < FL_B * FL_R; e += FL_THREADS)  // e = row * FL_R + q
            xT[(e & (FL_R - 1)) * FL_B + (e >> 3)] =
                red[e] + red[e + FL_B * FL_R] + red[e + 2 * FL_B * FL_R] + red[e + 3 * FL_B * FL_R];
        __syncthreads();
        // diagonal block: warp q solves right-hand side q, 32 rows at a time
        // (a lane per row): the 32 values times the lane's row of the
        // inverted triangle, then the block's remaining rows updated with the
        // 32 results.  Rows of the tile and the 32 values are read as float4
        // (the values as broadcasts); rows past nb hold zeros throughout.
        if (wid < nr) {
            float* xq = xT + wid * FL_B;
            const int nsb = (nb + 31) >> 5;
            auto dot32 = [&](const float* arow, const float* vals) {
                const float4* a4 = reinterpret_cast<const float4*>(arow);
                const float4* v4 = reinterpret_cast<const float4*>(vals);
                float e0 = 0.f, e1 = 0.f, e2 = 0.f, e3 = 0.f;
#pragma unroll
                for (int m = 0; m < 8; m++) {
                    const float4 av = a4[m], vv = v4[m];
                    e0 += av.x * vv.x;
                    e1 += av.y * vv.y;
                    e2 += av.z * vv.z;
                    e3 += av.w * vv.w;
                }
                return (e0 + e1) + (e2 + e3);
            };
            if (fwd) {
                for (int sb = 0; sb < nsb; sb++) {
                    const int row = sb * 32 + lane;
                    // row of L^-1: zero on and above the diagonal (its unit diagonal implied)
                    const float x = xq[row] + dot32(Ld + row * FL_LD + sb * 32, xq + sb * 32);
                    __syncwarp();
                    xq[row] = x;
                    __syncwarp();
                    for (int g = sb + 1; g < nsb; g++)
                        xq[g * 32 + lane] -= dot32(Ld + (g * 32 + lane) * FL_LD + sb * 32, xq + sb * 32);
                    __syncwarp();  // the next step reads rows other lanes updated
                }
            } else {
                for (int sb = nsb - 1; sb >= 0; sb--) {
                    const int row = sb * 32 + lane;
                    // row of U^-1: zero below the diagonal
                    float x = dot32(Ld + row * FL_LD + sb * 32, xq + sb * 32);
                    if (lane >= min(32, nb - sb * 32)) x = 0.f;
                    __syncwarp();
                    xq[row] = x;
                    __syncwarp();
                    for (int g = 0; g < sb; g++)
                        xq[g * 32 + lane] -= dot32(Ld + (g * 32 + lane) * FL_LD + sb * 32, xq + sb * 32);
                    __syncwarp();  // the next step reads rows other lanes updated
                }
            }
        }
        __syncthreads();
        if (tid < 2 * nb) {
            const int row = tid >> 1, q0 = (tid & 1) * 4;
            __stcg(reinterpret_cast<float4*>(Y + R0 * FL_R) + tid,
                   make_float4(xT[q0 * FL_B + row], xT[(q0 + 1) * FL_B + row], xT[(q0 + 2) * FL_B + row],
                               xT[(q0 + 3) * FL_B + row]));
        }
        if (!fwd)
            for (int e = tid; e < FL_B * FL_R; e += FL_THREADS) {
                const int row = e & (FL_B - 1), q = e >> 7;
                if (row < nb && q < nr) X[R0 + row + q * ldx] = xT[q * FL_B + row];
            }
        __syncthreads();
        if (tid == 0) st_release_gpu(done, fwd ? bi + 1 : nblk - bi);  // after the barrier: publishes the CTA's writes
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");  // leaving early: no copy into shared memory in flight
}

// ---------------------------------------------------------------------------
// triangular solves of one large system (n too big for the per-CTA solve):
// block-row sweeps, each block step = one CTA solving the 32 x 32 diagonal
// block for every right-hand side + a grid updating all rows below (above)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_perm_apply(LuBatch<T> B) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* stage = reinterpret_cast<T*>(smem_raw);
    const int64_t n = B.n[0], ldx = B.ldx[0];
    T* x = B.X[0] + (int64_t)blockIdx.x * ldx;
    const int32_t* pm = B.perm[0];
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) stage[r] = x[pm[r]];
    __syncthreads();
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) x[r] = stage[r];
}

// one warp per right-hand side, a lane per row of the diagonal block
template <class T>
__global__ void __launch_bounds__(256) k_trs_diag(LuBatch<T> B, int64_t k, int upper) {
    __shared__ T dg[GK][GK + 1];
    const int64_t n = B.n[0], ld = B.ld[0], ldx = B.ldx[0];
    const T* A = B.A[0];
    const int nb = (int)min((int64_t)GK, n - k);
    staged_copy<4>(
        nb * nb, threadIdx.x, blockDim.x, [&](int64_t e) { return A[(k + e % nb) + (k + e / nb) * ld]; },
        [&](int64_t e, T v) { dg[e % nb][e / nb] = v; });
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int nw = blockDim.x >> 5;
    for (int q = threadIdx.x >> 5; q < B.nrhs[0]; q += nw) {
        T* x = B.X[0] + (int64_t)q * ldx + k;
        T v = lane < nb ? x[lane] : (T)0;
        if (!upper) {
            for (int r = 0; r < nb; r++) {
                const T xr = __shfl_sync(0xffffffffu, v, r);
                if (lane > r && lane < nb) v -= dg[lane][r] * xr;
            }
        } else {
            for (int r = nb - 1; r >= 0; r--) {
                T xr = __shfl_sync(0xffffffffu, v, r);
                xr = xr / dg[r][r];
                if (lane == r) v = xr;
                if (lane < r) v -= dg[lane][r] * xr;
            }
        }
        if (lane < nb) x[lane] = v;
    }
}

// rows [lo, hi) -= A[rows, k:k+nb] x[k:k+nb, :]; grid (row blocks, rhs blocks of 8)
template <class T>
__global__ void __launch_bounds__(256) k_trs_update(LuBatch<T> B, int64_t k, int64_t lo, int64_t hi) {
    __shared__ T xs[GK][8];
    const int64_t n = B.n[0], ld = B.ld[0], ldx = B.ldx[0];
    const T* A = B.A[0];
    const int nb = (int)min((int64_t)GK, n - k);
    const int q0 = blockIdx.y * 8;
    const int nq = min(8, B.nrhs[0] - q0);
    for (int e = threadIdx.x; e < nb * 8; e += blockDim.x) {
        const int l = e % nb, q = e / nb;
        xs[l][q] = q < nq ? B.X[0][(k + l) + (int64_t)(q0 + q) * ldx] : (T)0;
    }
    __syncthreads();
    const int64_t r = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= hi) return;
    T acc[8];
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q] = 0;
    for (int l = 0; l < nb; l++) {
        const T a = A[r + (k + l) * ld];
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] += a * xs[l][q];
    }
    for (int q = 0; q < nq; q++) B.X[0][r + (int64_t)(q0 + q) * ldx] -= acc[q];
}

// ---------------------------------------------------------------------------
// single large float system on the tensor cores: triangular solves in
// 128-row blocks.  Per block: the diagonal triangle (unit lower forward,
// upper with its diagonal backward) solved in shared memory for up to 64
// right-hand sides per CTA, then the rows below (forward) or above (backward)
// updated with the block's solution by the 3xTF32 tcgen05 tile routine.
// ---------------------------------------------------------------------------
constexpr int TB = LU_OUTER;
constexpr int TB_COLS = 64;
constexpr int TB_LS = TB + 4, TB_XS = TB_COLS + 1;
constexpr size_t trs_block_smem() { return sizeof(float) * ((size_t)TB * TB_LS + (size_t)TB * TB_XS); }

template <bool UPPER>
__global__ void __launch_bounds__(256, 2) k_trs_block(LuBatch<float> B, int64_t k) {
    extern __shared__ __align__(16) float tb_smem[];
    float* L = tb_smem;          // triangle, L[r * TB_LS + c], padded to 128 with the identity
    float* X = L + TB * TB_LS;   // X[r * TB_XS + j]
    const int64_t n = B.n[0], ld = B.ld[0], ldx = B.ldx[0];
    const float* A = B.A[0] + k + k * ld;
    const int j0 = blockIdx.x * TB_COLS;
    const int ncols = min(TB_COLS, B.nrhs[0] - j0);
    const int bw = (int)min((int64_t)TB, n - k);
    float* Xg = B.X[0] + k + (int64_t)j0 * ldx;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    staged_copy<16>(
        TB * TB, tid, 256,
        [&](int64_t e) {
            const int r = (int)(e & (TB - 1)), c = (int)(e >> 7);
            return (r < bw && c < bw) ? A[r + (int64_t)c * ld] : (r == c ? 1.f : 0.f);
        },
        [&](int64_t e, float v) { L[(int)(e & (TB - 1)) * TB_LS + (int)(e >> 7)] = v; });
    staged_copy<16>(
        TB * TB_COLS, tid, 256,
        [&](int64_t e) {
            const int r = (int)(e & (TB - 1)), j = (int)(e >> 7);
            return (r < bw && j < ncols) ? Xg[r + (int64_t)j * ldx] : 0.f;
        },
        [&](int64_t e, float v) { X[(int)(e & (TB - 1)) * TB_XS + (int)(e >> 7)] = v; });
    __syncthreads();
#pragma unroll 1
    for (int bi = 0; bi < TB / 32; bi++) {
        const int rb = 32 * (UPPER ? TB / 32 - 1 - bi : bi);
        // diagonal 32 x 32: a warp per column, a lane per row, four columns in flight
        {
            float lrow[32];
#pragma unroll
            for (int l = 0; l < 32; l++) lrow[l] = L[(rb + lane) * TB_LS + rb + l];
#pragma unroll 1
            for (int jc = 4 * wid; jc < TB_COLS; jc += 32) {
                float x[4];
#pragma unroll
                for (int c = 0; c < 4; c++) x[c] = X[(rb + lane) * TB_XS + jc + c];
                if (!UPPER) {
#pragma unroll
                    for (int l = 0; l < 32; l++)
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const float xl = __shfl_sync(0xffffffffu, x[c], l);
                            if (lane > l) x[c] -= lrow[l] * xl;
                        }
                } else {
                    // each lane's reciprocal of its own diagonal entry, computed once
                    float dinv = 0.f;
#pragma unroll
                    for (int l = 0; l < 32; l++)
                        if (lane == l) dinv = 1.f / lrow[l];
#pragma unroll
                    for (int l = 31; l >= 0; l--) {
                        const float rl = __shfl_sync(0xffffffffu, dinv, l);
#pragma unroll
                        for (int c = 0; c < 4; c++) {
                            const float xl = __shfl_sync(0xffffffffu, x[c], l) * rl;
                            if (lane == l) x[c] = xl;
                            else if (lane < l) x[c] -= lrow[l] * xl;
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 4; c++) X[(rb + lane) * TB_XS + jc + c] = x[c];
            }
        }
        __syncthreads();
        // the other rows of the block: below (forward) or above (backward)
        const int r_lo = UPPER ? 0 : rb + 32, r_hi = UPPER ? rb : TB;
        if (r_hi > r_lo) {
            const int j = tid & (TB_COLS - 1), g = tid >> 6;
            float xb[32];
#pragma unroll
            for (int l = 0; l < 32; l++) xb[l] = X[(rb + l) * TB_XS + j];
#pragma unroll 1
            for (int r = r_lo + g; r < r_hi; r += 4) {
                const float4* lr = reinterpret_cast<const float4*>(L + r * TB_LS + rb);
                float acc = 0.f;
#pragma unroll
                for (int m = 0; m < 8; m++) {
                    const float4 v = lr[m];
                    acc += v.x * xb[4 * m] + v.y * xb[4 * m + 1] + v.z * xb[4 * m + 2] + v.w * xb[4 * m + 3];
                }
                X[r * TB_XS + j] -= acc;
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < TB * TB_COLS; e += 256) {
        const int r = e & (TB - 1), j = e >> 7;
        if (r < bw && j < ncols) Xg[r + (int64_t)j * ldx] = X[r * TB_XS + j];
    }
}

// rows [k + bw, n) (forward) or [0, k) (backward) of X -= A[rows, k:k+bw] X[k:k+bw, :]
template <bool UPPER>
__global__ void __launch_bounds__(tc::THREADS, 2) k_trs_tc(LuBatch<float> B, int64_t k, int* err) {
    extern __shared__ __align__(16) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tslot;
    const int64_t n = B.n[0], ld = B.ld[0], ldx = B.ldx[0];
    const int nrhs = B.nrhs[0];
    const int bw = (int)min((int64_t)TB, n - k);
    const int64_t lo = UPPER ? 0 : k + bw, hi = UPPER ? k : n;
    const int64_t r0 = lo + (int64_t)blockIdx.x * tc::BM, c0 = (int64_t)blockIdx.y * tc::BN;
    const float* A = B.A[0];
    float* X = B.X[0];
    tc::update_tile<3>(A + r0 + k * ld, ld, X + k + c0 * ldx, ldx, X + r0 + c0 * ldx, ldx,
                       (int)min((int64_t)tc::BM, hi - r0), (int)min((int64_t)tc::BN, (int64_t)nrhs - c0), bw, tc_smem,
                       bar, &tslot, err);
}

// persistent form of k_trs_tc: tile blk = (row tile blk % nrt, right-hand-side tile blk / nrt)
template <bool UPPER>
__global__ void __launch_bounds__(tc::P_THREADS, 1) k_trs_tcp(LuBatch<float> B, int64_t k, int* err, int64_t nrt,
                                                             int64_t ntiles) {
    extern __shared__ __align__(16) unsigned char tc_smem[];
    const int64_t n = B.n[0], ld = B.ld[0], ldx = B.ldx[0];
    const int nrhs = B.nrhs[0];
    const int bw = (int)min((int64_t)TB, n - k);
    const int64_t lo = UPPER ? 0 : k + bw, hi = UPPER ? k : n;
    const float* A = B.A[0];
    float* X = B.X[0];
    auto job = [&](int64_t blk) {
        const int64_t r0 = lo + (blk % nrt) * tc::BM, c0 = (blk / nrt) * tc::BN;
        tc::TileJob J;
        J.Lp = A + r0 + k * ld;
        J.ldl = ld;
        J.Up = X + k + c0 * ldx;
        J.ldu = ldx;
        J.Cp = X + r0 + c0 * ldx;
        J.ldc = ldx;
        J.m_rows = (int)min((int64_t)tc::BM, hi - r0);
        J.n_cols = (int)min((int64_t)tc::BN, (int64_t)nrhs - c0);
        J.K = bw;
        return J;
    };
    tc::update_persistent<3>(ntiles, job, tc_smem, err);
}

static int tc_num_sms() {
    static int sms[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && sms[dev]) return sms[dev];
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (v <= 0) v = 1;
    if (dev < 64) sms[dev] = v;
    return v;
}

// GBVLM_TC_PERSISTENT=1 selects the persistent warp-specialised update
static bool tc_persistent() {
    static int mode = -1;
    if (mode < 0) {
        const char* e = getenv("GBVLM_TC_PERSISTENT");
        mode = (e && atoi(e) == 1) ? 1 : 0;
    }
    return mode == 1;
}

template <class T>
int lu_large_solve(const LuBatch<T>& B, int64_t n, int32_t nrhs, cudaStream_t st, int* err) {
    GB_REQUIRE(sizeof(T) * (size_t)n <= (size_t)TS_SMEM_BYTES, "triangular solve: n=%lld too large", (long long)n);
    k_perm_apply<T><<<nrhs, 256, sizeof(T) * n, st>>>(B);
    GB_LAUNCH_CHECK();
    if constexpr (sizeof(T) == 4) {
        if (err) {  // tensor cores available: 128-row blocks
            const unsigned cb = (unsigned)cdiv(nrhs, TB_COLS), ct = (unsigned)cdiv(nrhs, tc::BN);
            for (int64_t k = 0; k < n; k += TB) {
                k_trs_block<false><<<cb, 256, trs_block_smem(), st>>>(B, k);
                GB_LAUNCH_CHECK();
                if (k + TB < n) {
                    const int64_t nrt = cdiv(n - k - TB, tc::BM);
                    if (tc_persistent()) {
                        const int64_t nt = nrt * ct;
                        k_trs_tcp<false><<<(unsigned)std::min<int64_t>(nt, tc_num_sms()), tc::P_THREADS, tc::P_SMEM_BYTES,
                                           st>>>(B, k, err, nrt, nt);
                    } else {
                        k_trs_tc<false><<<dim3((unsigned)nrt, ct), tc::THREADS, tc::SMEM_BYTES, st>>>(B, k, err);
                    }
                    GB_LAUNCH_CHECK();
                }
            }
            for (int64_t k = ((n - 1) / TB) * TB; k >= 0; k -= TB) {
                k_trs_block<true><<<cb, 256, trs_block_smem(), st>>>(B, k);
                GB_LAUNCH_CHECK();
                if (k > 0) {
                    const int64_t nrt = cdiv(k, tc::BM);
                    if (tc_persistent()) {
                        const int64_t nt = nrt * ct;
                        k_trs_tcp<true><<<(unsigned)std::min<int64_t>(nt, tc_num_sms()), tc::P_THREADS, tc::P_SMEM_BYTES,
                                          st>>>(B, k, err, nrt, nt);
                    } else {
                        k_trs_tc<true><<<dim3((unsigned)nrt, ct), tc::THREADS, tc::SMEM_BYTES, st>>>(B, k, err);
                    }
                    GB_LAUNCH_CHECK();
                }
            }
            return GBVLM_OK;
        }
    }
    const unsigned qb = (unsigned)cdiv(nrhs, 8);
    for (int64_t k = 0; k < n; k += GK) {
        k_trs_diag<T><<<1, 256, 0, st>>>(B, k, 0);
        GB_LAUNCH_CHECK();
        const int64_t lo = k + GK;
        if (lo < n) {
            k_trs_update<T><<<dim3((unsigned)cdiv(n - lo, 256), qb), 256, 0, st>>>(B, k, lo, n);
            GB_LAUNCH_CHECK();
        }
    }
    for (int64_t k = ((n - 1) / GK) * GK; k >= 0; k -= GK) {
        k_trs_diag<T><<<1, 256, 0, st>>>(B, k, 1);
        GB_LAUNCH_CHECK();
        if (k > 0) {
            k_trs_update<T><<<dim3((unsigned)cdiv(k, 256), qb), 256, 0, st>>>(B, k, 0, k);
            GB_LAUNCH_CHECK();
        }
    }
    return GBVLM_OK;
}

// ---------------------------------------------------------------------------
// panel launch: register panel with the thread count of the group
// ---------------------------------------------------------------------------
// GBVLM_INV_COLS=32 or 64 fixes the CTA width of L11^-1 (by default chosen per step)
static int inv_cols() {
    static int mode = -1;
    if (mode < 0) {
        const char* e = getenv("GBVLM_INV_COLS");
        mode = (e && (atoi(e) == 32 || atoi(e) == 64)) ? atoi(e) : 0;
    }
    return mode;
}

// GBVLM_PANEL_PACK=0 keeps one system per one-CTA panel
static bool panel_pack() {
    static int mode = -1;
    if (mode < 0) {
        const char* e = getenv("GBVLM_PANEL_PACK");
        mode = (e && atoi(e) == 0) ? 0 : 1;
    }
    return mode == 1;
}

// GBVLM_PANEL_TRIM=0 keeps every warp of a one-CTA panel in the column loop
static bool panel_trim() {
    static int mode = -1;
    if (mode < 0) {
        const char* e = getenv("GBVLM_PANEL_TRIM");
        mode = (e && atoi(e) == 0) ? 0 : 1;
    }
    return mode == 1;
}

template <class T, int NT, int RPT>
static int launch_panel_nt(const LuBatch<T>& B, int64_t k, const int32_t* act, const PanelGroup& g,
                           const int32_t* d_pack, cudaStream_t st) {
    if (g.csize == 1) {
        const bool packed = g.ctas > 0 && d_pack;
        k_panel_reg<T, NT, false, RPT><<<packed ? g.ctas : g.count, NT, sizeof(PanelSmem<T, NT, false>), st>>>(
            B, k, act, g.slab, panel_trim() ? 1 : 0, packed ? d_pack + 2 * g.pack_off : nullptr, g.count);
        GB_LAUNCH_CHECK();
        return GBVLM_OK;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(g.count * g.csize));
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = sizeof(PanelSmem<T, NT, true>);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = g.csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    GB_CUDA(cudaLaunchKernelEx(&cfg, k_panel_reg<T, NT, true, RPT>, B, k, act, g.slab, 0, (const int32_t*)nullptr,
                               g.count));
    return GBVLM_OK;
}

template <class T>
static int launch_panel(const LuBatch<T>& B, int64_t k, const int32_t* act, const PanelGroup& g,
                        const int32_t* d_pack, cudaStream_t st) {
    if (g.csize == 0) {
        k_panel<T><<<g.count, PANEL_THREADS, 0, st>>>(B, k, act);
        GB_LAUNCH_CHECK();
        return GBVLM_OK;
    }
    if constexpr (sizeof(T) == 4) {  // one row per thread (two per thread, half the warps, measured
                                     // slower with both shuffled and shared-memory pivot rows, for
                                     // the cluster panels alone, and with two batches in flight)
        switch (g.nt) {
            case 128: return launch_panel_nt<T, 128, 1>(B, k, act, g, d_pack, st);
            case 256: return launch_panel_nt<T, 256, 1>(B, k, act, g, d_pack, st);
            case 512: return launch_panel_nt<T, 512, 1>(B, k, act, g, d_pack, st);
            default: return launch_panel_nt<T, 1024, 1>(B, k, act, g, d_pack, st);
        }
    } else {
        return launch_panel_nt<T, PR_THREADS_F64, 1>(B, k, act, g, nullptr, st);
    }
}

// ---------------------------------------------------------------------------
// host plan
// ---------------------------------------------------------------------------
template <class T>
int lu_batch_factor(const LuBatch<T>& B, const LuPlan& plan, cudaStream_t st, bool lookahead) {
    lookahead = lookahead && plan.la_stream != nullptr && plan.tc_events == nullptr;
    bool pending = false;  // a lookahead update in flight on plan.la_stream
    for (size_t s = 0; s < plan.steps.size(); s++) {
        const LuStep& S = plan.steps[s];
        if (S.n_panel == 0) continue;
        for (const PanelGroup& g : S.panels[sizeof(T) == 4 ? 0 : 1]) {
            const int rc = launch_panel<T>(B, S.k, plan.d_act + S.act_off + g.first, g, plan.d_pack, st);
            if (rc) return rc;
        }
        const bool two_level = sizeof(T) == 4 && plan.W > GK;
        const int32_t* act = plan.d_act + S.act_off;
        if (!two_level) {
            if (S.swap_total > 0) {
                k_swap<T><<<(unsigned)cdiv(S.swap_total, 256), 256, 0, st>>>(B, S.k, act, plan.d_pfx + S.swap_pfx,
                                                                           S.n_panel);
                GB_LAUNCH_CHECK();
            }
            if (S.trsm_blocks > 0) {
                k_trsm<T><<<(unsigned)S.trsm_blocks, TRSM_COLS, 0, st>>>(B, S.k, act, plan.d_pfx + S.trsm_pfx, S.n_panel,
                                                                       INT64_MAX);
                GB_LAUNCH_CHECK();
            }
            if (S.upd_blocks > 0) {
                k_update<T><<<(unsigned)S.upd_blocks, 256, 0, st>>>(B, S.k, act, plan.d_pfx + S.upd_pfx, S.n_upd, 0, 0);
                GB_LAUNCH_CHECK();
            }
            continue;
        }
        // two-level blocking, outer block [k0, kend)
        const int64_t k0 = S.kend - plan.W;
        // the panel's row moves and U rows in one launch, then the inner update in tiles
        if constexpr (sizeof(T) == 4) {
            if (S.ik_blocks > 0) {
                k_inner<<<(unsigned)S.ik_blocks, IN_THREADS, 0, st>>>(B, S.k, k0, S.kend, act, plan.d_pfx + S.ik_pfx,
                                                                      S.n_panel);
                GB_LAUNCH_CHECK();
            }
            if (S.in_blocks > 0 && plan.tc_inner) {
                if (plan.tc_passes == 1)
                    k_inner_tc<1><<<(unsigned)S.inc_blocks, tc::THREADS, tc::SMEM_BYTES, st>>>(
                        B, S.k, S.kend, act, plan.d_pfx + S.inc_pfx, S.n_in, plan.d_err);
                else
                    k_inner_tc<3><<<(unsigned)S.inc_blocks, tc::THREADS, tc::SMEM_BYTES, st>>>(
                        B, S.k, S.kend, act, plan.d_pfx + S.inc_pfx, S.n_in, plan.d_err);
                GB_LAUNCH_CHECK();
            } else if (S.in_blocks > 0) {
                k_update<T><<<(unsigned)S.in_blocks, 256, 0, st>>>(B, S.k, act, plan.d_pfx + S.in_pfx, S.n_in, S.kend, 1);
                GB_LAUNCH_CHECK();
            }
        }
        if (pending && ((S.bswap_first == 0 && S.bswap_total > 0) || S.tc_blocks > 0)) {
            // at the block's last step its swaps (and U12 solve) reach the columns the
            // lookahead update is still working on; systems that end the block earlier
            // have n <= kend of the previous block + W and no lookahead tiles
            GB_CUDA(cudaStreamWaitEvent(st, plan.la_join, 0));
            pending = false;
        }
        if (S.bswap_total > 0) {
            k_swap2<T><<<(unsigned)S.bswap_total, SW2_THREADS, 0, st>>>(
                B, act + S.bswap_first, plan.d_pfx + S.bswap_pfx, S.n_panel - S.bswap_first, k0, S.kend, 0, k0, S.kend,
                INT64_MAX);
            GB_LAUNCH_CHECK();
        }
        if constexpr (sizeof(T) == 4) {
            if (S.tc_blocks > 0) {
                if (plan.tc_trsm && S.n_tc >= plan.tc_trsm_min) {
                    // four CTAs of 32 columns per system when the step's systems fill
                    // less than a wave (the chain of few large systems is shorter), two
                    // of 64 otherwise (fewer CTAs when the SMs are busy); the same arithmetic
                    const int ic = inv_cols();
                    if (ic == 32 || (ic == 0 && 4 * (int64_t)S.n_tc <= tc_num_sms()))
                        k_trsm_wide<LU_OUTER, true, 32><<<(unsigned)(4 * S.n_tc), 256, trsm_wide_smem<LU_OUTER, 32>(),
                                                          st>>>(B, k0, act, nullptr, S.n_tc, plan.d_minv, plan.base);
                    else
                        k_trsm_wide<LU_OUTER, true><<<(unsigned)(2 * S.n_tc), 256, trsm_wide_smem<LU_OUTER>(), st>>>(
                            B, k0, act, nullptr, S.n_tc, plan.d_minv, plan.base);
                    GB_LAUNCH_CHECK();
                    const int64_t* tp = plan.d_pfx + S.tcs_pfx;
                    if (plan.tc_wide) {
                        constexpr int SM_ = tc::smem_bytes<tc::BN_WIDE>();
                        if (plan.tc_passes == 1)
                            k_trsm_tc12<1, tc::BN_WIDE><<<(unsigned)S.tcs_blocks, tc::THREADS, SM_, st>>>(
                                B, k0, act, tp, S.n_tc, plan.d_minv, plan.base, plan.d_err);
                        else
                            k_trsm_tc12<3, tc::BN_WIDE><<<(unsigned)S.tcs_blocks, tc::THREADS, SM_, st>>>(
                                B, k0, act, tp, S.n_tc, plan.d_minv, plan.base, plan.d_err);
                    } else {
                        if (plan.tc_passes == 1)
                            k_trsm_tc12<1, tc::BN><<<(unsigned)S.tcs_blocks, tc::THREADS, tc::SMEM_BYTES, st>>>(
                                B, k0, act, tp, S.n_tc, plan.d_minv, plan.base, plan.d_err);
                        else
                            k_trsm_tc12<3, tc::BN><<<(unsigned)S.tcs_blocks, tc::THREADS, tc::SMEM_BYTES, st>>>(
                                B, k0, act, tp, S.n_tc, plan.d_minv, plan.base, plan.d_err);
                    }
                    GB_LAUNCH_CHECK();
                } else {
                    k_trsm_wide<LU_OUTER><<<(unsigned)S.btrsm_blocks, 256, trsm_wide_smem<LU_OUTER>(), st>>>(
                        B, k0, act, plan.d_pfx + S.btrsm_pfx, S.n_tc, nullptr, 0);
                    GB_LAUNCH_CHECK();
                }
                if (plan.tc_events) {
                    cudaEvent_t e0, e1;
                    GB_CUDA(cudaEventCreate(&e0));
                    GB_CUDA(cudaEventCreate(&e1));
                    plan.tc_events->push_back(e0);
                    plan.tc_events->push_back(e1);
                    GB_CUDA(cudaEventRecord(e0, st));
                }
                auto tc_launch = [&](int64_t blocks, int64_t pfx_off, int part, cudaStream_t s_) {
                    const int64_t* pfx = plan.d_pfx + pfx_off;
                    if (tc_persistent()) {
                        const unsigned grid = (unsigned)std::min<int64_t>(blocks, tc_num_sms());
                        if (plan.tc_passes == 1)
                            k_update_tcp<1><<<grid, tc::P_THREADS, tc::P_SMEM_BYTES, s_>>>(B, k0, plan.W, act, pfx, S.n_tc,
                                                                                        plan.d_err, part, blocks);
                        else
                            k_update_tcp<3><<<grid, tc::P_THREADS, tc::P_SMEM_BYTES, s_>>>(B, k0, plan.W, act, pfx, S.n_tc,
                                                                                        plan.d_err, part, blocks);
                        return;
                    }
                    // the next outer panel (part 1) in 128-column tiles, the rest in the plan's width
                    if (part != 1 && plan.tc_wide) {
                        constexpr int SM_ = tc::smem_bytes<tc::BN_WIDE>();
                        if (plan.tc_passes == 1)
                            k_update_tc<1, tc::BN_WIDE><<<(unsigned)blocks, tc::THREADS, SM_, s_>>>(
                                B, k0, plan.W, act, pfx, S.n_tc, plan.d_err, part);
                        else
                            k_update_tc<3, tc::BN_WIDE><<<(unsigned)blocks, tc::THREADS, SM_, s_>>>(
                                B, k0, plan.W, act, pfx, S.n_tc, plan.d_err, part);
                        return;
                    }
                    if (plan.tc_passes == 1)
                        k_update_tc<1, tc::BN><<<(unsigned)blocks, tc::THREADS, tc::SMEM_BYTES, s_>>>(
                            B, k0, plan.W, act, pfx, S.n_tc, plan.d_err, part);
                    else
                        k_update_tc<3, tc::BN><<<(unsigned)blocks, tc::THREADS, tc::SMEM_BYTES, s_>>>(
                            B, k0, plan.W, act, pfx, S.n_tc, plan.d_err, part);
                };
                if (!lookahead) {
                    tc_launch(S.tc_blocks, S.tc_pfx, 0, st);
                    GB_LAUNCH_CHECK();
                } else {
                    // lookahead: the next outer panel's columns first; the rest of the
                    // trailing matrix on the side stream while the next block's inner
                    // steps (confined to that panel) run here
                    tc_launch(S.tcn_blocks, S.tcn_pfx, 1, st);
                    GB_LAUNCH_CHECK();
                    if (S.tcr_blocks > 0) {
                        GB_CUDA(cudaEventRecord(plan.la_fork, st));
                        GB_CUDA(cudaStreamWaitEvent(plan.la_stream, plan.la_fork, 0));
                        tc_launch(S.tcr_blocks, S.tcr_pfx, 2, plan.la_stream);
                        GB_LAUNCH_CHECK();
                        GB_CUDA(cudaEventRecord(plan.la_join, plan.la_stream));
                        pending = true;
                    }
                }
                if (plan.tc_events) GB_CUDA(cudaEventRecord(plan.tc_events->back(), st));
            }
        }
    }
    if (pending) GB_CUDA(cudaStreamWaitEvent(st, plan.la_join, 0));
    if (plan.nsys > 0) {
        k_perm<T><<<plan.nsys, 256, sizeof(int32_t) * std::min<int64_t>(plan.maxn, PERM_SMEM), st>>>(B, plan.base);
        GB_LAUNCH_CHECK();
    }
    return GBVLM_OK;
}

template <class T>
int lu_batch_solve(const LuBatch<T>& B, int32_t nsys, int32_t max_nrhs, int64_t maxn, cudaStream_t st, int* err) {
    // X of the largest system in shared memory when it fits, else staged per column
    const size_t full = sizeof(T) * (size_t)maxn * TS_MAXRHS;
    const int use_smem = full <= (size_t)TS_SMEM_BYTES ? 1 : 0;
    if (!use_smem && nsys == 1) return lu_large_solve<T>(B, maxn, max_nrhs, st, err);
    const size_t smem = use_smem ? full : sizeof(T) * (size_t)maxn;
    GB_REQUIRE(smem <= (size_t)TS_SMEM_BYTES, "triangular solve: n=%lld needs %zu bytes of shared memory",
               (long long)maxn, smem);
    // one CTA per system and block of TS_MAXRHS right-hand sides, all in one launch
    const int64_t blocks = cdiv(max_nrhs, TS_MAXRHS);
    GB_REQUIRE(blocks <= 65535, "triangular solve: %d right-hand sides exceed one launch", max_nrhs);
    k_trsolve<T><<<dim3((unsigned)nsys, (unsigned)blocks), TS_THREADS, smem, st>>>(B, 0, TS_MAXRHS, use_smem);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

template int lu_batch_factor<float>(const LuBatch<float>&, const LuPlan&, cudaStream_t, bool);
template int lu_batch_factor<double>(const LuBatch<double>&, const LuPlan&, cudaStream_t, bool);
template int lu_batch_solve<float>(const LuBatch<float>&, int32_t, int32_t, int64_t, cudaStream_t, int*);
template int lu_batch_solve<double>(const LuBatch<double>&, int32_t, int32_t, int64_t, cudaStream_t, int*);

// Build the per-step tables.  Systems must be sorted by n descending so the
// active systems of every step form a prefix of the order.
int lu_plan_build(LuPlan& plan, const std::vector<int64_t>& n_sorted, cudaStream_t st, int32_t base) {
    plan.release();
    plan.base = base;
    GB_CUDA(cudaFuncSetAttribute(k_trsolve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_trsolve<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_perm<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, PERM_SMEM * 4));
    GB_CUDA(cudaFuncSetAttribute(k_perm_apply<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_perm_apply<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_perm<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, PERM_SMEM * 4));
    plan.nsys = (int32_t)n_sorted.size();
    plan.maxn = n_sorted.empty() ? 0 : n_sorted[0];
    plan.tc_flops = plan.tc_bytes = 0;
    plan.tc_launches = 0;
    // trailing update of the float factorisation: tensor cores (3xTF32) on
    // devices with tcgen05, or as GBVLM_LU_TC asks (0: CUDA cores, 1: TF32, 3: 3xTF32)
    {
        int dev = 0, major = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
        plan.tc_passes = major >= 10 ? 3 : 0;
        if (const char* e = getenv("GBVLM_LU_TC")) {
            const int v = atoi(e);
            plan.tc_passes = (v == 1 || v == 3) && major >= 10 ? v : 0;
        }
        plan.W = plan.tc_passes ? LU_OUTER : GK;
        {
            const char* e = getenv("GBVLM_TC_WIDE");
            plan.tc_wide = plan.tc_passes && !tc_persistent() && !(e && e[0] == '0');
            const char* ti = getenv("GBVLM_TC_INNER");
            plan.tc_inner = plan.tc_passes && !(ti && ti[0] == '0');
            const char* t = getenv("GBVLM_TC_TRSM");
            plan.tc_trsm = plan.tc_passes && !(t && t[0] == '0');
            plan.tc_trsm_min = TC_TRSM_MIN_SYSTEMS;
        }
        if (plan.tc_passes) {
            GB_CUDA(cudaFuncSetAttribute(k_update_tc<1, tc::BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_update_tc<3, tc::BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_update_tc<1, tc::BN_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::smem_bytes<tc::BN_WIDE>()));
            GB_CUDA(cudaFuncSetAttribute(k_update_tc<3, tc::BN_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::smem_bytes<tc::BN_WIDE>()));
            GB_CUDA(cudaFuncSetAttribute(k_inner_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_inner_tc<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_trsm_wide<LU_OUTER, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)trsm_wide_smem<LU_OUTER>()));
            GB_CUDA(cudaFuncSetAttribute(k_trsm_wide<LU_OUTER, true, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)trsm_wide_smem<LU_OUTER, 32>()));
            GB_CUDA(cudaFuncSetAttribute(k_trsm_tc12<1, tc::BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_trsm_tc12<3, tc::BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_trsm_tc12<1, tc::BN_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::smem_bytes<tc::BN_WIDE>()));
            GB_CUDA(cudaFuncSetAttribute(k_trsm_tc12<3, tc::BN_WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::smem_bytes<tc::BN_WIDE>()));
            GB_CUDA(cudaFuncSetAttribute(k_trsm_wide<LU_OUTER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)trsm_wide_smem<LU_OUTER>()));
            GB_CUDA(cudaFuncSetAttribute(k_trs_block<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)trs_block_smem()));
            GB_CUDA(cudaFuncSetAttribute(k_trs_block<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)trs_block_smem()));
            GB_CUDA(cudaFuncSetAttribute(k_trs_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_trs_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_update_tcp<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::P_SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_update_tcp<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::P_SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_trs_tcp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::P_SMEM_BYTES));
            GB_CUDA(cudaFuncSetAttribute(k_trs_tcp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::P_SMEM_BYTES));
        }
        GB_CUDA(dev_alloc((void**)&plan.d_err, sizeof(int), plan.mem));
        GB_CUDA(cudaMemsetAsync(plan.d_err, 0, sizeof(int), st));
        if (plan.tc_passes) {  // lookahead stream (lowest priority) and its events
            int least = 0, greatest = 0;
            GB_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
            GB_CUDA(cudaStreamCreateWithPriority(&plan.la_stream, cudaStreamNonBlocking, least));
            GB_CUDA(cudaEventCreateWithFlags(&plan.la_fork, cudaEventDisableTiming));
            GB_CUDA(cudaEventCreateWithFlags(&plan.la_join, cudaEventDisableTiming));
        }
    }
    // largest cluster the device schedules for the register panel (16 needs the
    // non-portable opt-in), probed once per device
    static std::mutex probe_mu;
    static int probed[64];
    int dev_id = 0;
    GB_CUDA(cudaGetDevice(&dev_id));
    std::lock_guard<std::mutex> probe_lock(probe_mu);
    plan.cluster = dev_id < 64 && probed[dev_id] ? probed[dev_id] : 1;
    if (dev_id >= 64 || !probed[dev_id]) {
        cudaFuncSetAttribute(k_panel_reg<float, 1024, true, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(k_panel_reg<float, 512, true, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(k_panel_reg<float, 256, true, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(k_panel_reg<float, 128, true, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(k_panel_reg<double, PR_THREADS_F64, true, 1>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        for (int c : {16, 8, 4, 2}) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(1024);
            cfg.dynamicSmemBytes = sizeof(PanelSmem<float, 1024, true>);
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int n2 = 0, n1 = 0;
            const bool ok2 = cudaOccupancyMaxActiveClusters(&n2, k_panel_reg<float, 1024, true, 1>, &cfg) == cudaSuccess;
            cfg.blockDim = dim3(PR_THREADS_F64);
            cfg.dynamicSmemBytes = sizeof(PanelSmem<double, PR_THREADS_F64, true>);
            const bool ok1 =
                cudaOccupancyMaxActiveClusters(&n1, k_panel_reg<double, PR_THREADS_F64, true, 1>, &cfg) == cudaSuccess;
            if (ok2 && ok1 && n2 > 0 && n1 > 0) {
                plan.cluster = c;
                break;
            }
            cudaGetLastError();
        }
        if (dev_id < 64) probed[dev_id] = plan.cluster;
    }
    const int nsys = (int)n_sorted.size();
    for (int i = 1; i < nsys; i++) GB_REQUIRE(n_sorted[i] <= n_sorted[i - 1], "lu plan: sizes not sorted");
    std::vector<int32_t> act, pack;
    std::vector<int64_t> pfx;
    const int64_t maxn = nsys ? n_sorted[0] : 0;
    for (int64_t k = 0; k < maxn; k += GK) {
        LuStep S;
        S.k = k;
        S.act_off = (int64_t)act.size();
        int cnt = 0;
        while (cnt < nsys && n_sorted[cnt] > k) cnt++;
        for (int i = 0; i < cnt; i++) act.push_back(base + i);
        S.n_panel = cnt;
        for (int e = 0; e < 2; e++) {
            // rows per CTA = threads (one row per thread in registers): float up to 1024, double 256
            const int64_t slab_max = e == 0 ? 1024 : PR_THREADS_F64;
            S.panels[e].clear();
            int i = 0;
            while (i < cnt) {
                const int64_t rows = n_sorted[i] - k;
                int cs = 1;
                while ((int64_t)cs * slab_max < rows) cs *= 2;
                PanelGroup g;
                g.first = i;
                int j = i;
                if (cs > plan.cluster) {
                    g.csize = 0;  // too tall for the largest cluster
                    while (j < cnt && n_sorted[j] - k > (int64_t)plan.cluster * slab_max) j++;
                } else {
                    g.csize = cs;
                    g.slab = (int)cdiv(rows, cs);
                    g.nt = e == 0 ? 128 : PR_THREADS_F64;
                    while (g.nt < g.slab) g.nt *= 2;
                    while (j < cnt && n_sorted[j] - k > (int64_t)(cs / 2) * slab_max) j++;
                }
                g.count = j - i;
                if (e == 0 && g.csize == 1 && g.nt >= 2 * PACK_MIN_SLICE && panel_pack() && panel_trim()) {
                    // systems sorted by size: a CTA takes the next system and
                    // as many after it as slices of that one's width fit
                    g.pack_off = (int64_t)pack.size() / 2;
                    for (int q = i; q < j;) {
                        int w = PACK_MIN_SLICE;
                        while (w < n_sorted[q] - k) w *= 2;
                        const int P = std::min(g.nt / w, j - q);
                        pack.push_back(q - i);
                        pack.push_back(g.nt / w);
                        g.ctas++;
                        q += P;
                    }
                }
                S.panels[e].push_back(g);
                i = j;
            }
        }
        // swap: columns outside the panel, n - nb each
        S.swap_pfx = (int64_t)pfx.size();
        int64_t acc = 0;
        for (int i = 0; i < cnt; i++) {
            pfx.push_back(acc);
            acc += n_sorted[i] - std::min<int64_t>(GK, n_sorted[i] - k);
        }
        pfx.push_back(acc);
        S.swap_total = acc;
        // trsm: blocks of TRSM_COLS over columns k+nb .. n
        S.trsm_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < cnt; i++) {
            pfx.push_back(acc);
            int64_t m = n_sorted[i] - k - std::min<int64_t>(GK, n_sorted[i] - k);
            acc += m > 0 ? cdiv(m, TRSM_COLS) : 0;
        }
        pfx.push_back(acc);
        S.trsm_blocks = acc;
        // update: systems with n > k + GK (a prefix), tiles GT x GT
        int cu = 0;
        while (cu < cnt && n_sorted[cu] > k + GK) cu++;
        S.n_upd = cu;
        S.upd_act_skip = 0;
        S.upd_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < cu; i++) {
            pfx.push_back(acc);
            int64_t t = cdiv(n_sorted[i] - k - GK, GT);
            acc += t * t;
        }
        pfx.push_back(acc);
        S.upd_blocks = acc;
        // two-level blocking (float, tensor cores): outer block [k0, kend) of W columns
        S.kend = (k / plan.W + 1) * plan.W;
        const int64_t k0 = S.kend - plan.W;
        // inner update: rows [k + GK, n) x columns [k + GK, min(n, kend))
        S.in_pfx = (int64_t)pfx.size();
        acc = 0;
        int ci = 0;
        for (int i = 0; i < cu; i++) {
            const int64_t ke = std::min<int64_t>(n_sorted[i], S.kend);
            if (ke <= k + GK) break;  // a suffix of the sorted systems
            pfx.push_back(acc);
            acc += cdiv(n_sorted[i] - k - GK, GT) * cdiv(ke - k - GK, GT);
            ci++;
        }
        pfx.push_back(acc);
        S.n_in = ci;
        S.in_blocks = acc;
        S.inc_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < ci; i++) {
            pfx.push_back(acc);
            acc += cdiv(n_sorted[i] - k - GK, tc::BM);
        }
        pfx.push_back(acc);
        S.inc_blocks = acc;
        // k_inner: IN_COLS-column chunks of [k0, k) and [k + nb, min(n, kend))
        S.ik_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < cnt; i++) {
            pfx.push_back(acc);
            const int64_t n = n_sorted[i], nbk = std::min<int64_t>(GK, n - k);
            acc += (k - k0) / IN_COLS + cdiv(std::max<int64_t>(0, std::min(n, S.kend) - (k + nbk)), IN_COLS);
        }
        pfx.push_back(acc);
        S.ik_blocks = acc;
        // end of the outer block for the systems whose last step in it is this one:
        // all active systems at the block's last step, else those with n <= k + GK
        const bool block_end = k + GK == S.kend;
        S.bswap_first = block_end ? 0 : cu;
        S.bswap_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = S.bswap_first; i < cnt; i++) {
            pfx.push_back(acc);
            const int64_t n = n_sorted[i];
            acc += cdiv(k0 + (n - std::min(n, S.kend)), (int64_t)SW2_THREADS);  // CTAs of the system
        }
        pfx.push_back(acc);
        S.bswap_total = acc;
        // U12 solve and tensor-core update: systems with n > kend, at the block's last step
        ci = 0;
        if (block_end)
            while (ci < nsys && n_sorted[ci] > S.kend) ci++;
        S.n_tc = ci;
        S.btrsm_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < ci; i++) {
            pfx.push_back(acc);
            acc += cdiv(n_sorted[i] - S.kend, TW_COLS);
        }
        pfx.push_back(acc);
        S.btrsm_blocks = acc;
        S.tc_pfx = (int64_t)pfx.size();
        acc = 0;
        const int64_t cw = plan.tc_wide ? tc::BN_WIDE : tc::BN;  // tile columns of parts 0 and 2
        for (int i = 0; i < ci; i++) {
            pfx.push_back(acc);
            const int64_t m = n_sorted[i] - S.kend;
            const int64_t t = cdiv(m, tc::BM);
            acc += t * cdiv(m, cw);
            plan.tc_flops += 2.0 * (double)m * (double)m * plan.W;
            plan.tc_bytes += 8.0 * (double)m * (double)m + 8.0 * (double)m * plan.W;
        }
        pfx.push_back(acc);
        S.tc_blocks = acc;
        plan.tc_launches += acc > 0;
        // the same update split for lookahead: first column of tiles / the rest
        S.tcn_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < ci; i++) {
            pfx.push_back(acc);
            acc += cdiv(n_sorted[i] - S.kend, tc::BM);
        }
        pfx.push_back(acc);
        S.tcn_blocks = acc;
        S.tcr_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < ci; i++) {
            pfx.push_back(acc);
            const int64_t m = n_sorted[i] - S.kend;
            acc += cdiv(m, tc::BM) * (m > tc::BN ? cdiv(m - tc::BN, cw) : 0);
        }
        pfx.push_back(acc);
        S.tcr_blocks = acc;
        S.tcs_pfx = (int64_t)pfx.size();
        acc = 0;
        for (int i = 0; i < ci; i++) {
            pfx.push_back(acc);
            acc += cdiv(n_sorted[i] - S.kend, cw);
        }
        pfx.push_back(acc);
        S.tcs_blocks = acc;
        plan.steps.push_back(S);
    }
    if (plan.tc_trsm && plan.nsys > 0)
        GB_CUDA(dev_alloc((void**)&plan.d_minv, sizeof(float) * LU_OUTER * LU_OUTER * (size_t)plan.nsys, plan.mem));
    if (!act.empty()) {
        GB_CUDA(dev_alloc((void**)&plan.d_act, act.size() * sizeof(int32_t), plan.mem));
        GB_CUDA(cudaMemcpyAsync(plan.d_act, act.data(), act.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    if (!pack.empty()) {
        GB_CUDA(dev_alloc((void**)&plan.d_pack, pack.size() * sizeof(int32_t), plan.mem));
        GB_CUDA(cudaMemcpyAsync(plan.d_pack, pack.data(), pack.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    if (!pfx.empty()) {
        GB_CUDA(dev_alloc((void**)&plan.d_pfx, pfx.size() * sizeof(int64_t), plan.mem));
        GB_CUDA(cudaMemcpyAsync(plan.d_pfx, pfx.data(), pfx.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    }
    GB_CUDA(cudaStreamSynchronize(st));
    return GBVLM_OK;
}

int lu_plan_check(const LuPlan& plan, cudaStream_t st) {
    if (!plan.d_err) return GBVLM_OK;
    int* h = (int*)host_scratch(sizeof(int));
    GB_CUDA(cudaMemcpyAsync(h, plan.d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (*h != 0) {
        set_error("LU: a tensor-core update tile timed out waiting for its MMAs");
        return GBVLM_ERR_CUDA;
    }
    return GBVLM_OK;
}

int64_t lu_plan_launches(const LuPlan& plan, int es) {
    const int e = es == 4 ? 0 : 1;
    const bool two_level = es == 4 && plan.W > GK;
    int64_t n = 0;
    for (const LuStep& S : plan.steps) {
        if (S.n_panel == 0) continue;
        n += (int64_t)S.panels[e].size();
        if (!two_level) {
            n += (S.swap_total > 0) + (S.trsm_blocks > 0) + (S.upd_blocks > 0);
        } else {
            n += (S.ik_blocks > 0) + (S.in_blocks > 0) + (S.bswap_total > 0) +
                 (2 + (plan.tc_trsm && S.n_tc >= plan.tc_trsm_min)) * (S.tc_blocks > 0) +
                 (S.tc_blocks > 0 && plan.la_stream && S.tcr_blocks > 0);
        }
    }
    return n + (plan.nsys > 0);  // + the permutation kernel
}

int trs_flow_build(TrsFlow& f, const std::vector<int64_t>& n_sorted, cudaStream_t st, int32_t groups) {
    f.release();
    f.nsys = (int32_t)n_sorted.size();
    f.groups = std::max(1, groups);
    if (f.nsys == 0) return GBVLM_OK;
    GB_REQUIRE(f.nsys <= FL_SYS_MASK + 1 && f.groups <= 1024, "dataflow solve: %d systems, %d groups", f.nsys,
               f.groups);
    std::vector<int32_t> nblk(f.nsys);
    int32_t maxblk = 0;
    int64_t rows = 0;
    for (int32_t s = 0; s < f.nsys; s++) {
        GB_REQUIRE(s == 0 || n_sorted[s] <= n_sorted[s - 1], "dataflow solve: systems must be sorted by size");
        nblk[s] = (int32_t)((n_sorted[s] + FL_B - 1) / FL_B);
        maxblk = std::max(maxblk, nblk[s]);
        rows += n_sorted[s];
    }
    // forward items by block level, backward items by distance from the last
    // block; within a level the groups of right-hand sides, then the largest
    // systems (longest chains) first
    std::vector<int2> items;
    for (int32_t i = 0; i < maxblk; i++)
        for (int32_t g = 0; g < f.groups; g++)
            for (int32_t s = 0; s < f.nsys && nblk[s] > i; s++) items.push_back(make_int2(s | (g << FL_SYS_BITS), i));
    f.nfwd = (int32_t)items.size();
    for (int32_t d = 0; d < maxblk; d++)
        for (int32_t g = 0; g < f.groups; g++)
            for (int32_t s = 0; s < f.nsys && nblk[s] > d; s++)
                items.push_back(make_int2(s | (g << FL_SYS_BITS), nblk[s] - 1 - d));
    f.nitems = (int32_t)items.size();
    GB_CUDA(cudaFuncSetAttribute(k_trs_flow, cudaFuncAttributeMaxDynamicSharedMemorySize, FL_SMEM));
    int dev = 0, sms = 0, per_sm = 0;
    GB_CUDA(cudaGetDevice(&dev));
    GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trs_flow, FL_THREADS, FL_SMEM));
    GB_REQUIRE(per_sm > 0, "dataflow solve: kernel does not fit on an SM");
    f.grid = (int32_t)std::min<int64_t>((int64_t)sms * per_sm, f.nitems);
    const size_t G = (size_t)f.groups;
    std::vector<float*> yp(G * f.nsys);
    GB_CUDA(dev_alloc((void**)&f.d_items, sizeof(int2) * items.size(), f.mem));
    GB_CUDA(dev_alloc((void**)&f.d_ctl, sizeof(int32_t) * (2 + 2 * G * f.nsys), f.mem));
    GB_CUDA(dev_alloc((void**)&f.d_y, sizeof(float) * FL_R * G * (size_t)rows, f.mem));
    GB_CUDA(dev_alloc((void**)&f.d_yp, sizeof(float*) * G * f.nsys, f.mem));
    int64_t off = 0;
    for (size_t g = 0; g < G; g++)
        for (int32_t s = 0; s < f.nsys; s++) {
            yp[g * f.nsys + s] = f.d_y + off;
            off += FL_R * n_sorted[s];
        }
    GB_CUDA(cudaMemcpyAsync(f.d_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemcpyAsync(f.d_yp, yp.data(), sizeof(float*) * yp.size(), cudaMemcpyHostToDevice, st));
    GB_CUDA(cudaMemsetAsync(f.d_ctl, 0, sizeof(int32_t) * (2 + 2 * G * f.nsys), st));
    GB_CUDA(cudaStreamSynchronize(st));  // the host tables above are about to go out of scope
    return GBVLM_OK;
}

int64_t trs_flow_launches(int32_t max_nrhs, int32_t groups) {
    const int32_t per = FL_R * std::max(1, groups);  // right-hand sides one launch covers
    return (max_nrhs + per - 1) / per;
}

int trs_flow_solve(const LuBatch<float>& B, const TrsFlow& f, int32_t max_nrhs, cudaStream_t st) {
    if (f.nitems == 0) return GBVLM_OK;
    const int32_t per = FL_R * f.groups;
    for (int32_t r0 = 0; r0 < max_nrhs; r0 += per) {
        // the counter and progress words restart; the error word is kept
        GB_CUDA(cudaMemsetAsync(f.d_ctl, 0, sizeof(int32_t), st));
        GB_CUDA(cudaMemsetAsync(f.d_ctl + 2, 0, sizeof(int32_t) * 2 * (size_t)f.groups * f.nsys, st));
        k_trs_flow<<<f.grid, FL_THREADS, FL_SMEM, st>>>(B, f.d_items, f.nfwd, f.nitems, f.nsys, f.d_ctl, f.d_yp, r0);
        GB_LAUNCH_CHECK();
    }
    return GBVLM_OK;
}

int trs_flow_check(const TrsFlow& f, cudaStream_t st) {
    if (!f.d_ctl) return GBVLM_OK;
    int* h = (int*)host_scratch(sizeof(int));
    GB_CUDA(cudaMemcpyAsync(h, f.d_ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (*h != 0) {
        set_error("triangular solve: a block timed out waiting for the blocks it depends on");
        return GBVLM_ERR_CUDA;
    }
    return GBVLM_OK;
}

void TrsFlow::release() {
    dev_free(d_items, mem);
    dev_free(d_ctl, mem);
    dev_free(d_y, mem);
    dev_free(d_yp, mem);
    d_items = nullptr;
    d_ctl = nullptr;
    d_y = nullptr;
    d_yp = nullptr;
    nsys = nfwd = nitems = grid = 0;
}

void LuPlan::release() {
    dev_free(d_minv, mem);
    d_minv = nullptr;
    dev_free(d_act, mem);
    dev_free(d_pack, mem);
    dev_free(d_pfx, mem);
    dev_free(d_err, mem);
    if (la_stream) cudaStreamDestroy(la_stream);
    if (la_fork) cudaEventDestroy(la_fork);
    if (la_join) cudaEventDestroy(la_join);
    d_act = nullptr;
    d_pack = nullptr;
    d_pfx = nullptr;
    d_err = nullptr;
    la_stream = nullptr;
    la_fork = la_join = nullptr;
    steps.clear();
}

// ---------------------------------------------------------------------------
// mixed-precision refinement helpers
// ---------------------------------------------------------------------------
// R = B - A X   (A float n x n col-major, X/B/R double), grid (row blocks, rhs)
__global__ void k_residual(const float* A, int64_t n, int64_t ld, const double* X, int64_t ldx, const double* Bm,
                           int64_t ldb, double* R, int64_t ldr) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int q = blockIdx.y;
    if (r >= n) return;
    const double* x = X + q * ldx;
    double s = 0, c = 0;
    for (int64_t j = 0; j < n; j++) {
        double p = (double)A[r + j * ld] * x[j];
        double t = s + p;
        c += (fabs(s) >= fabs(p)) ? ((s - t) + p) : ((p - t) + s);
        s = t;
    }
    R[r + q * ldr] = Bm[r + q * ldb] - (s + c);
}

__global__ void k_d2f(const double* in, int64_t n, int64_t ldi, float* out, int64_t ldo) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) out[r + blockIdx.y * ldo] = (float)in[r + blockIdx.y * ldi];
}

__global__ void k_axpy_f2d(const float* d, int64_t n, int64_t ldd, double* x, int64_t ldx, double* maxupd) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const double v = (double)d[r + blockIdx.y * ldd];
    x[r + blockIdx.y * ldx] += v;
    if (maxupd) {
        unsigned long long* p = (unsigned long long*)maxupd;
        double a = fabs(v);
        atomicMax(p, __double_as_longlong(a));  // non-negative doubles order like their bit patterns
    }
}


template <class T>
int make_single_batch(LuBatch<T>& B, int64_t n, int64_t ld, T* A, int32_t* ipiv, int32_t* perm, int32_t* info, T* X,
                      int64_t ldx, int32_t nrhs, void** work, size_t* work_bytes, cudaStream_t st) {
    struct Tab {
        int64_t n, ld, ldx;
        T* A;
        int32_t* ipiv;
        T* X;
        int32_t nrhs;
        int32_t* perm;
    } tab{n, ld, ldx, A, ipiv, X, nrhs, perm};
    constexpr size_t MV_OFF = 256;  // the panel's move lists after the table
    static_assert(sizeof(Tab) <= MV_OFF, "table larger than its slot");
    if (*work_bytes < MV_OFF + 64 * sizeof(int32_t)) {
        if (*work) cudaFree(*work);
        *work = nullptr;
        GB_CUDA(cudaMalloc(work, MV_OFF + 64 * sizeof(int32_t)));
        *work_bytes = MV_OFF + 64 * sizeof(int32_t);
    }
    // pageable source: the call returns once the table is staged, so the
    // stack copy may go out of scope
    GB_CUDA(cudaMemcpyAsync(*work, &tab, sizeof(Tab), cudaMemcpyHostToDevice, st));
    Tab* d = (Tab*)*work;
    B.n = &d->n;
    B.ld = &d->ld;
    B.ldx = &d->ldx;
    B.A = &d->A;
    B.ipiv = &d->ipiv;
    B.X = &d->X;
    B.nrhs = &d->nrhs;
    B.perm = &d->perm;
    B.info = info;
    B.mv = (int32_t*)((char*)*work + MV_OFF);
    return GBVLM_OK;
}
template int make_single_batch<float>(LuBatch<float>&, int64_t, int64_t, float*, int32_t*, int32_t*, int32_t*, float*,
                                      int64_t, int32_t, void**, size_t*, cudaStream_t);
template int make_single_batch<double>(LuBatch<double>&, int64_t, int64_t, double*, int32_t*, int32_t*, int32_t*,
                                       double*, int64_t, int32_t, void**, size_t*, cudaStream_t);

}  // namespace gbvlm

using namespace gbvlm;

struct gbvlm_lu_s {
    int64_t n = 0;
    int32_t* d_perm = nullptr;
    int32_t* d_ipiv = nullptr;
    int32_t* d_info = nullptr;
    LuPlan plan;
    int64_t plan_n = -1;
    void* work = nullptr;
    size_t work_bytes = 0;
    // float solves: the dataflow solve of the one system, built for flow_n
    // unknowns and flow_groups blocks of 8 right-hand sides
    TrsFlow flow;
    int64_t flow_n = -1;
    int32_t flow_groups = 0;
};

// the dataflow solve for nrhs right-hand sides of the handle's system, built
// on first use; false for systems of up to two 128-row blocks (one CTA's
// k_trsolve has no chain to overlap there: measured faster in the coupled
// 2 x 2 + 2 x 2 panel time step) or when GBVLM_TRS_FLOW=0 selects the
// per-system solves
static int lu_flow_ready(gbvlm_lu h, int64_t n, int64_t nrhs, cudaStream_t st, bool* use) {
    const char* fe = getenv("GBVLM_TRS_FLOW");
    const int64_t groups64 = (nrhs + 7) / 8;
    *use = !(fe && fe[0] == '0') && n > 2 * FL_B && trs_flow_fits(1, groups64);
    if (!*use) return GBVLM_OK;
    const int32_t groups = (int32_t)groups64;
    if (h->flow_n == n && h->flow_groups >= groups) return GBVLM_OK;
    h->flow_n = -1;
    int rc = trs_flow_build(h->flow, std::vector<int64_t>{n}, st, groups);
    if (rc) return rc;
    h->flow_n = n;
    h->flow_groups = groups;
    return GBVLM_OK;
}

static int lu_ensure(gbvlm_lu h, int64_t n, cudaStream_t st) {
    if (h->plan_n == n && h->d_ipiv) return GBVLM_OK;
    if (h->d_ipiv) cudaFree(h->d_ipiv);
    if (h->d_info) cudaFree(h->d_info);
    if (h->d_perm) cudaFree(h->d_perm);
    h->d_ipiv = nullptr;
    h->d_info = nullptr;
    h->d_perm = nullptr;
    GB_CUDA(cudaMalloc(&h->d_ipiv, sizeof(int32_t) * (n > 0 ? n : 1)));
    GB_CUDA(cudaMalloc(&h->d_perm, sizeof(int32_t) * (n > 0 ? n : 1)));
    GB_CUDA(cudaMalloc(&h->d_info, sizeof(int32_t)));
    std::vector<int64_t> ns(1, n);
    int rc = lu_plan_build(h->plan, ns, st);
    if (rc) return rc;
    h->plan_n = n;
    h->n = n;
    return GBVLM_OK;
}

template <class T>
static int lu_factor_one(gbvlm_lu h, T* A, int64_t n, int64_t ld, cudaStream_t st) {
    GB_REQUIRE(h && A && n >= 1 && ld >= n, "bad LU arguments");
    int rc = lu_ensure(h, n, st);
    if (rc) return rc;
    GB_CUDA(cudaMemsetAsync(h->d_info, 0, sizeof(int32_t), st));
    LuBatch<T> B;
    rc = make_single_batch<T>(B, n, ld, A, h->d_ipiv, h->d_perm, h->d_info, nullptr, 0, 0, &h->work, &h->work_bytes, st);
    if (rc) return rc;
    rc = lu_batch_factor<T>(B, h->plan, st, true);
    if (rc) return rc;
    int32_t* hi = (int32_t*)host_scratch(sizeof(int32_t));
    GB_CUDA(cudaMemcpyAsync(hi, h->d_info, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (*hi != 0) {
        set_error("LU: exactly zero pivot at column %d", *hi);
        return GBVLM_ERR_SINGULAR;
    }
    if (h->flow_n >= 0 && (rc = trs_flow_check(h->flow, st))) return rc;  // a solve since the last factorisation
    return lu_plan_check(h->plan, st);
}

template <class T>
static int lu_solve_one(gbvlm_lu h, const T* A, int64_t n, int64_t ld, T* X, int64_t ldx, int64_t nrhs,
                        cudaStream_t st) {
    GB_REQUIRE(h && A && X && n >= 1 && ld >= n && ldx >= n && nrhs >= 1, "bad LU solve arguments");
    GB_REQUIRE(h->plan_n == n, "LU solve before factorize for this size");
    LuBatch<T> B;
    int rc = make_single_batch<T>(B, n, ld, (T*)A, h->d_ipiv, h->d_perm, h->d_info, X, ldx, (int32_t)nrhs,
                                  &h->work, &h->work_bytes, st);
    if (rc) return rc;
    if constexpr (std::is_same<T, float>::value) {
        bool flow = false;
        if ((rc = lu_flow_ready(h, n, nrhs, st, &flow))) return rc;
        if (flow) return trs_flow_solve(B, h->flow, (int32_t)nrhs, st);
    }
    return lu_batch_solve<T>(B, 1, (int32_t)nrhs, n, st, h->plan.tc_passes ? h->plan.d_err : nullptr);
}

namespace gbvlm {

struct LuSolveTables {
    LuBatch<float> B;
    void* work = nullptr;
    size_t work_bytes = 0;
    bool flow = false;  // the handle's dataflow solve (built at prepare) serves the solves
};

int lu_solve_prepare_f32(gbvlm_lu h, const float* A, int64_t n, float* X, void** tables, cudaStream_t st) {
    GB_REQUIRE(h && A && X && tables && n >= 1, "null argument");
    GB_REQUIRE(h->plan_n == n, "LU solve before factorize for this size");
    auto* t = new LuSolveTables();
    int rc = make_single_batch<float>(t->B, n, n, (float*)A, h->d_ipiv, h->d_perm, h->d_info, X, n, 1, &t->work,
                                      &t->work_bytes, st);
    if (!rc) rc = lu_flow_ready(h, n, 1, st, &t->flow);
    if (rc) {
        lu_solve_tables_free(t);
        return rc;
    }
    *tables = t;
    return GBVLM_OK;
}

int lu_solve_prepared_f32(gbvlm_lu h, void* tables, int64_t n, cudaStream_t st) {
    GB_REQUIRE(h && tables, "null argument");
    const LuSolveTables* t = (const LuSolveTables*)tables;
    if (t->flow && h->flow_n == n) return trs_flow_solve(t->B, h->flow, 1, st);
    return lu_batch_solve<float>(t->B, 1, 1, n, st, h->plan.tc_passes ? h->plan.d_err : nullptr);
}

int lu_solve_check(gbvlm_lu h, cudaStream_t st) {
    GB_REQUIRE(h, "null argument");
    return h->flow_n >= 0 ? trs_flow_check(h->flow, st) : GBVLM_OK;
}

void lu_solve_tables_free(void* tables) {
    auto* t = (LuSolveTables*)tables;
    if (!t) return;
    if (t->work) cudaFree(t->work);
    delete t;
}

// test hook kernel: one tensor-core tile whose MMA thread withholds its
// MMAs and commit (update_tile<1, true>), over a 128 x 128 matrix, K = 32
__global__ void __launch_bounds__(tc::THREADS) k_test_tc_withhold(float* A, int* err) {
    extern __shared__ __align__(16) unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tslot;
    tc::update_tile<1, true>(A, 128, A, 128, A, 128, 128, 128, tc::BK, tc_smem, bar, &tslot, err);
}

}  // namespace gbvlm

extern "C" {

int gbvlm_test_tc_wait_timeout(gbvlm_stream stream) {
    cudaStream_t st = to_cuda(stream);
    float* A = nullptr;
    int* err = nullptr;
    auto run = [&]() -> int {
        GB_CUDA(cudaMalloc(&A, sizeof(float) * 128 * 128));
        GB_CUDA(cudaMalloc(&err, sizeof(int)));
        GB_CUDA(cudaMemsetAsync(A, 0, sizeof(float) * 128 * 128, st));
        GB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        GB_CUDA(cudaFuncSetAttribute(k_test_tc_withhold, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES));
        k_test_tc_withhold<<<1, tc::THREADS, tc::SMEM_BYTES, st>>>(A, err);
        GB_LAUNCH_CHECK();
        int h = 0;
        GB_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        if (h != 0) {
            set_error("tensor-core update tile: the wait for its MMAs timed out");
            return GBVLM_ERR_CUDA;
        }
        set_error("tensor-core update tile: the withheld MMAs were not detected");
        return GBVLM_ERR_STATE;
    };
    const int rc = run();
    cudaStreamSynchronize(st);
    if (A) cudaFree(A);
    if (err) cudaFree(err);
    return rc;
}

int gbvlm_test_flow_wait_timeout(int32_t n, gbvlm_stream stream) {
    GB_REQUIRE(n > FL_B && n <= 4 * FL_B, "n must span 2 to 4 blocks of %d rows", FL_B);
    cudaStream_t st = to_cuda(stream);
    // an identity system of n unknowns; only the forward item of its second
    // block is handed out, so that item's wait for the first block never ends
    float *A = nullptr, *X = nullptr;
    int32_t *ipiv = nullptr, *perm = nullptr, *info = nullptr;
    void* work = nullptr;
    size_t work_bytes = 0;
    TrsFlow f;
    auto run = [&]() -> int {
        GB_CUDA(cudaMalloc(&A, sizeof(float) * n * n));
        GB_CUDA(cudaMalloc(&X, sizeof(float) * n));
        GB_CUDA(cudaMalloc(&ipiv, sizeof(int32_t) * n));
        GB_CUDA(cudaMalloc(&perm, sizeof(int32_t) * n));
        GB_CUDA(cudaMalloc(&info, sizeof(int32_t)));
        std::vector<float> a((size_t)n * n, 0.f);
        std::vector<int32_t> id(n);
        for (int32_t i = 0; i < n; i++) {
            a[(size_t)i * n + i] = 1.f;
            id[i] = i;
        }
        GB_CUDA(cudaMemcpy(A, a.data(), sizeof(float) * a.size(), cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemcpy(perm, id.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice));
        GB_CUDA(cudaMemset(X, 0, sizeof(float) * n));
        LuBatch<float> B;
        if (int rc = make_single_batch<float>(B, n, n, A, ipiv, perm, info, X, n, 1, &work, &work_bytes, st)) return rc;
        if (int rc = trs_flow_build(f, std::vector<int64_t>{n}, st)) return rc;
        GB_CUDA(cudaMemsetAsync(f.d_ctl, 0, sizeof(int32_t) * 4, st));
        k_trs_flow<<<1, FL_THREADS, FL_SMEM, st>>>(B, f.d_items + 1, 1, 1, 1, f.d_ctl, f.d_yp, 0);
        GB_LAUNCH_CHECK();
        return trs_flow_check(f, st);
    };
    const int rc = run();
    cudaStreamSynchronize(st);
    for (void* p : {(void*)A, (void*)X, (void*)ipiv, (void*)perm, (void*)info, work})
        if (p) cudaFree(p);
    return rc;
}

int gbvlm_lu_create(gbvlm_lu* out) {
    GB_REQUIRE(out != nullptr, "out is null");
    *out = new gbvlm_lu_s();
    return GBVLM_OK;
}

int gbvlm_lu_destroy(gbvlm_lu h) {
    if (!h) return GBVLM_OK;
    if (h->d_ipiv) cudaFree(h->d_ipiv);
    if (h->d_info) cudaFree(h->d_info);
    if (h->d_perm) cudaFree(h->d_perm);
    if (h->work) cudaFree(h->work);
    h->plan.release();
    delete h;
    return GBVLM_OK;
}

int gbvlm_lu_init(gbvlm_lu h, int64_t n) {
    GB_REQUIRE(h && n >= 1, "bad LU init arguments");
    return lu_ensure(h, n, 0);
}

int gbvlm_lu_factor_f32(gbvlm_lu h, float* A, int64_t n, int64_t ld, gbvlm_stream s) {
    return lu_factor_one<float>(h, A, n, ld, to_cuda(s));
}
int gbvlm_lu_factor_f64(gbvlm_lu h, double* A, int64_t n, int64_t ld, gbvlm_stream s) {
    return lu_factor_one<double>(h, A, n, ld, to_cuda(s));
}
int gbvlm_lu_solve_f32(gbvlm_lu h, const float* A, int64_t n, int64_t ld, float* X, int64_t ldx, int64_t nrhs,
                       gbvlm_stream s) {
    return lu_solve_one<float>(h, A, n, ld, X, ldx, nrhs, to_cuda(s));
}
int gbvlm_lu_solve_f64(gbvlm_lu h, const double* A, int64_t n, int64_t ld, double* X, int64_t ldx, int64_t nrhs,
                       gbvlm_stream s) {
    return lu_solve_one<double>(h, A, n, ld, X, ldx, nrhs, to_cuda(s));
}

int gbvlm_lu_solve_refined(gbvlm_lu h, const float* LU, const float* A, int64_t n, int64_t ld, const double* Bm,
                           double* X, int64_t nrhs, int32_t iters, double* last_update, gbvlm_stream s) {
    GB_REQUIRE(h && LU && A && Bm && X && n >= 1 && ld >= n && nrhs >= 1 && nrhs <= 65535 && iters >= 0,
               "bad refined-solve arguments");
    GB_REQUIRE(h->plan_n == n, "refined solve before factorize for this size");
    cudaStream_t st = to_cuda(s);
    // workspace: float n*nrhs + double n*nrhs + 1 double
    size_t need = sizeof(float) * n * nrhs + sizeof(double) * (n * nrhs + 1);
    void* ws = nullptr;
    int rc = device_scratch(need, &ws, st);
    if (rc) return rc;
    float* xf = (float*)ws;
    double* R = (double*)((char*)ws + ((sizeof(float) * n * nrhs + 7) / 8) * 8);
    double* dmax = R + n * nrhs;
    dim3 g((unsigned)cdiv(n, 256), (unsigned)nrhs);
    // x0 = LU^-1 b in float
    k_d2f<<<g, 256, 0, st>>>(Bm, n, n, xf, n);
    GB_LAUNCH_CHECK();
    rc = gbvlm_lu_solve_f32(h, LU, n, ld, xf, n, nrhs, s);
    if (rc) return rc;
    GB_CUDA(cudaMemsetAsync(X, 0, sizeof(double) * n * nrhs, st));
    k_axpy_f2d<<<g, 256, 0, st>>>(xf, n, n, X, n, nullptr);
    GB_LAUNCH_CHECK();
    for (int it = 0; it < iters; it++) {
        k_residual<<<g, 256, 0, st>>>(A, n, ld, X, n, Bm, n, R, n);
        GB_LAUNCH_CHECK();
        k_d2f<<<g, 256, 0, st>>>(R, n, n, xf, n);
        GB_LAUNCH_CHECK();
        rc = gbvlm_lu_solve_f32(h, LU, n, ld, xf, n, nrhs, s);
        if (rc) return rc;
        if (it == iters - 1 && last_update) GB_CUDA(cudaMemsetAsync(dmax, 0, sizeof(double), st));
        k_axpy_f2d<<<g, 256, 0, st>>>(xf, n, n, X, n, (it == iters - 1 && last_update) ? dmax : nullptr);
        GB_LAUNCH_CHECK();
    }
    if (last_update) {
        if (iters == 0) {
            *last_update = 0;
        } else {
            GB_CUDA(cudaMemcpyAsync(last_update, dmax, sizeof(double), cudaMemcpyDeviceToHost, st));
            GB_CUDA(cudaStreamSynchronize(st));
        }
    }
    return GBVLM_OK;
}

}  // extern "C"
