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
#include <string.h>

#include <algorithm>
#include <vector>

#include "gbvlm_internal.h"
#include "gbvlm_lu.h"

namespace gbvlm {

constexpr int PANEL_THREADS = 512;
constexpr int TRSM_COLS = 128;
constexpr int GT = 64;  // update tile edge
constexpr int GK = LU_NB;
constexpr int PERM_SMEM = 12 * 1024;  // systems up to this size build the permutation in shared memory
constexpr int TS_SMEM_BYTES = 200 * 1024;

template <class T>
__device__ __forceinline__ T tabs(T x) { return x < (T)0 ? -x : x; }

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

// Same panel factorisation with the panel (rows k..n-1, nb columns) staged in
// shared memory, column-major with leading dimension `rows`.  Used when the
// panel fits (PANEL_SMEM_ROWS rows); the panel is read once and written once.
constexpr int PANEL_SMEM_BYTES = 220 * 1024;

template <class T>
__global__ void __launch_bounds__(PANEL_THREADS) k_panel_smem(LuBatch<T> B, int64_t k, const int32_t* act) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* P = reinterpret_cast<T*>(smem_raw);
    const int32_t sid = act[blockIdx.x];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    int32_t* ipiv = B.ipiv[sid];
    const int nb = (int)min((int64_t)GK, n - k);
    const int rows = (int)(n - k);
    __shared__ T s_val[PANEL_THREADS / 32];
    __shared__ int s_idx[PANEL_THREADS / 32];
    __shared__ int s_piv;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int t = 0; t < nb; t++)
        for (int r = tid; r < rows; r += PANEL_THREADS) P[t * rows + r] = A[(k + r) + (k + t) * ld];
    __syncthreads();
    for (int jj = 0; jj < nb; jj++) {
        T* c = P + jj * rows;
        T best = (T)-1;
        int bi = jj;
        for (int r = jj + tid; r < rows; r += PANEL_THREADS) {
            T v = tabs(c[r]);
            if (v > best) { best = v; bi = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            T ov = __shfl_down_sync(0xffffffffu, best, o);
            int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { s_val[wid] = best; s_idx[wid] = bi; }
        __syncthreads();
        if (tid == 0) {
            T bv = s_val[0];
            int bix = s_idx[0];
            for (int w = 1; w < PANEL_THREADS / 32; w++) {
                if (s_val[w] > bv || (s_val[w] == bv && s_idx[w] < bix)) { bv = s_val[w]; bix = s_idx[w]; }
            }
            s_piv = bix;
            ipiv[k + jj] = (int32_t)(k + bix);
            if (c[bix] == (T)0 && B.info[sid] == 0) B.info[sid] = (int32_t)(k + jj + 1);
        }
        __syncthreads();
        const int p = s_piv;
        if (p != jj) {
            for (int t = tid; t < nb; t += PANEL_THREADS) {
                T tmp = P[t * rows + jj];
                P[t * rows + jj] = P[t * rows + p];
                P[t * rows + p] = tmp;
            }
        }
        __syncthreads();
        const T d = c[jj];
        const T inv = (d != (T)0) ? (T)1 / d : (T)0;
        for (int r = jj + 1 + tid; r < rows; r += PANEL_THREADS) {
            const T l = (d != (T)0) ? c[r] / d : c[r];
            c[r] = l;
            for (int t = jj + 1; t < nb; t++) P[t * rows + r] -= l * P[t * rows + jj];
        }
        (void)inv;
        __syncthreads();
    }
    for (int t = 0; t < nb; t++)
        for (int r = tid; r < rows; r += PANEL_THREADS) A[(k + r) + (k + t) * ld] = P[t * rows + r];
}

// Tall panels: a thread-block cluster of `csize` CTAs holds the panel in its
// distributed shared memory, CTA q owning rows [q*slab, (q+1)*slab) of it.
// Per column: local arg-max, cluster barrier, every CTA reads the csize
// candidates over DSMEM and picks the same pivot (largest |a|, first row on
// ties); the CTA owning the diagonal row swaps it with the pivot row across
// the panel over DSMEM; after a second barrier every CTA copies the pivot row
// and updates its own rows.  All remote accesses finish before the final
// barrier, so no CTA exits while another still reads its shared memory.
constexpr int PC_THREADS = 512;

template <class T>
__global__ void __launch_bounds__(PC_THREADS) k_panel_cluster(LuBatch<T> B, int64_t k, const int32_t* act, int slab) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int csize = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* P = reinterpret_cast<T*>(smem_raw);  // [nb][slab]
    __shared__ T cand_v;
    __shared__ int cand_i;
    __shared__ T prow[GK];
    __shared__ T s_val[PC_THREADS / 32];
    __shared__ int s_idx[PC_THREADS / 32];
    __shared__ int s_piv;
    const int32_t sid = act[blockIdx.x / csize];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    int32_t* ipiv = B.ipiv[sid];
    const int nb = (int)min((int64_t)GK, n - k);
    const int rows = (int)(n - k);
    const int r0 = rank * slab, r1 = min(rows, r0 + slab);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int t = 0; t < nb; t++)
        for (int r = r0 + tid; r < r1; r += PC_THREADS) P[t * slab + (r - r0)] = A[(k + r) + (k + t) * ld];
    cl.sync();
    for (int jj = 0; jj < nb; jj++) {
        T best = (T)-1;
        int bi = rows;
        for (int r = max(r0, jj) + tid; r < r1; r += PC_THREADS) {
            const T v = tabs(P[jj * slab + (r - r0)]);
            if (v > best) { best = v; bi = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const T ov = __shfl_down_sync(0xffffffffu, best, o);
            const int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { s_val[wid] = best; s_idx[wid] = bi; }
        __syncthreads();
        if (tid == 0) {
            T bv = s_val[0];
            int bix = s_idx[0];
            for (int w = 1; w < PC_THREADS / 32; w++)
                if (s_val[w] > bv || (s_val[w] == bv && s_idx[w] < bix)) { bv = s_val[w]; bix = s_idx[w]; }
            cand_v = bv;
            cand_i = bix;
        }
        cl.sync();
        if (tid == 0) {
            T bv = (T)-1;
            int bix = rows;
            for (int q = 0; q < csize; q++) {
                const T v = *cl.map_shared_rank(&cand_v, q);
                const int i = *cl.map_shared_rank(&cand_i, q);
                if (v > bv || (v == bv && i < bix)) { bv = v; bix = i; }
            }
            s_piv = bix;
            if (rank == 0) {
                ipiv[k + jj] = (int32_t)(k + bix);
                if (bv == (T)0 && B.info[sid] == 0) B.info[sid] = (int32_t)(k + jj + 1);
            }
        }
        __syncthreads();
        const int p = s_piv;
        const int owner_j = jj / slab, owner_p = p / slab;
        if (p != jj && rank == owner_j) {
            T* Pp = cl.map_shared_rank(P, owner_p);
            for (int t = tid; t < nb; t += PC_THREADS) {
                const T a = P[t * slab + (jj - r0)];
                const T b = Pp[t * slab + (p - owner_p * slab)];
                P[t * slab + (jj - r0)] = b;
                Pp[t * slab + (p - owner_p * slab)] = a;
            }
        }
        cl.sync();
        const T* Pj = cl.map_shared_rank(P, owner_j);
        for (int t = tid; t < nb; t += PC_THREADS) prow[t] = Pj[t * slab + (jj - owner_j * slab)];
        __syncthreads();
        const T d = prow[jj];
        for (int r = max(r0, jj + 1) + tid; r < r1; r += PC_THREADS) {
            T l = P[jj * slab + (r - r0)];
            if (d != (T)0) l = l / d;
            P[jj * slab + (r - r0)] = l;
            for (int t = jj + 1; t < nb; t++) P[t * slab + (r - r0)] -= l * prow[t];
        }
    }
    cl.sync();
    for (int t = 0; t < nb; t++)
        for (int r = r0 + tid; r < r1; r += PC_THREADS) A[(k + r) + (k + t) * ld] = P[t * slab + (r - r0)];
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

// ---------------------------------------------------------------------------
// trsm: U12 = L11^-1 A12, one thread per column, TRSM_COLS columns per block
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(TRSM_COLS) k_trsm(LuBatch<T> B, int64_t k, const int32_t* act, const int64_t* pfx,
                                                   int cnt) {
    __shared__ T L[GK][GK + 1];
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    const int nb = (int)min((int64_t)GK, n - k);
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
        int r = t % nb, c = t / nb;
        L[r][c] = A[(k + r) + (k + c) * ld];
    }
    __syncthreads();
    const int64_t j = k + nb + (int64_t)(blockIdx.x - pfx[a]) * TRSM_COLS + threadIdx.x;
    if (j >= n) return;
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
// update: A22 -= L21 * U12 on 64x64 tiles, 256 threads, each a 4x4 block of
// consecutive rows/columns read from shared memory as vectors
// ---------------------------------------------------------------------------
template <class T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4; };

template <class T>
__global__ void __launch_bounds__(256) k_update(LuBatch<T> B, int64_t k, const int32_t* act, const int64_t* pfx,
                                               int cnt) {
    constexpr int SW = GT + 4;  // row stride keeps 16-byte alignment of every 4-run
    __shared__ __align__(16) T sA[GK][SW];  // L21 tile: [kk][row]
    __shared__ __align__(16) T sB[GK][SW];  // U12 tile: [kk][col]
    const int a = find_block(pfx, cnt, blockIdx.x);
    const int32_t sid = act[a];
    const int64_t n = B.n[sid], ld = B.ld[sid];
    T* A = B.A[sid];
    const int64_t m = n - k - GK;  // trailing size (systems here have n > k + GK)
    const int64_t tiles = (m + GT - 1) / GT;
    const int64_t t = blockIdx.x - pfx[a];
    const int64_t r0 = k + GK + (t % tiles) * GT, c0 = k + GK + (t / tiles) * GT;
    const int tid = threadIdx.x;
    for (int e = tid; e < GK * GT; e += 256) {
        const int kk = e / GT, rr = e % GT;
        const int64_t r = r0 + rr;
        sA[kk][rr] = r < n ? A[r + (k + kk) * ld] : (T)0;
        const int cc = e / GK, k2 = e % GK;
        const int64_t c = c0 + cc;
        sB[k2][cc] = c < n ? A[(k + k2) + c * ld] : (T)0;
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
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int64_t c = c0 + 4 * ty + j;
        if (c >= n) continue;
        T* col = A + c * ld;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int64_t r = r0 + 4 * tx + i;
            if (r < n) col[r] -= acc[i][j];
        }
    }
}

// ---------------------------------------------------------------------------
// row permutation of a finished factorisation: perm[r] = original row that
// ends up in position r (the ipiv interchanges composed in order)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_perm(LuBatch<T> B) {
    extern __shared__ int32_t sp[];
    const int32_t sid = blockIdx.x;
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
constexpr int TS_THREADS = 256;
constexpr int TS_MAXRHS = 8;

template <class T>
__global__ void __launch_bounds__(TS_THREADS) k_trsolve(LuBatch<T> B, int32_t rhs0, int32_t nrhs_blk, int use_smem) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int32_t sid = blockIdx.x;
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
        for (int64_t e = tid; e < n * nr; e += TS_THREADS) {
            const int64_t r = e % n;
            const int q = (int)(e / n);
            W[r * TS_MAXRHS + q] = X[pm[r] + q * ldx];
        }
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
        for (int e = tid; e < nb * nb; e += TS_THREADS) {
            const int r = e % nb, c = e / nb;
            dg[r][c] = A[(k + r) + (k + c) * ld];
        }
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
#pragma unroll
            for (int q = 0; q < TS_MAXRHS; q++) acc[q] = 0;
            for (int l = 0; l < nb; l++) {
                const T a = A[r + (k + l) * ld];
#pragma unroll
                for (int q = 0; q < TS_MAXRHS; q++) acc[q] += a * xs[l][q];
            }
            for (int q = 0; q < nr; q++) WX(r, q) -= acc[q];
        }
        __syncthreads();
    }
    // backward: U
    const int64_t nblk = (n + GK - 1) / GK;
    for (int64_t bk = nblk - 1; bk >= 0; bk--) {
        const int64_t k = bk * GK;
        const int nb = (int)min((int64_t)GK, n - k);
        for (int e = tid; e < nb * nb; e += TS_THREADS) {
            const int r = e % nb, c = e / nb;
            dg[r][c] = A[(k + r) + (k + c) * ld];
        }
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
#pragma unroll
            for (int q = 0; q < TS_MAXRHS; q++) acc[q] = 0;
            for (int l = 0; l < nb; l++) {
                const T a = A[r + (k + l) * ld];
#pragma unroll
                for (int q = 0; q < TS_MAXRHS; q++) acc[q] += a * xs[l][q];
            }
            for (int q = 0; q < nr; q++) WX(r, q) -= acc[q];
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
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) dg[e % nb][e / nb] = A[(k + e % nb) + (k + e / nb) * ld];
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

template <class T>
int lu_large_solve(const LuBatch<T>& B, int64_t n, int32_t nrhs, cudaStream_t st) {
    GB_REQUIRE(sizeof(T) * (size_t)n <= (size_t)TS_SMEM_BYTES, "triangular solve: n=%lld too large", (long long)n);
    k_perm_apply<T><<<nrhs, 256, sizeof(T) * n, st>>>(B);
    GB_LAUNCH_CHECK();
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
// host plan
// ---------------------------------------------------------------------------
template <class T>
int lu_batch_factor(const LuBatch<T>& B, const LuPlan& plan, cudaStream_t st) {
    for (size_t s = 0; s < plan.steps.size(); s++) {
        const LuStep& S = plan.steps[s];
        if (S.n_panel == 0) continue;
        // systems are sorted by n descending: the ones whose panel is too tall
        // for shared memory form a prefix of the active list
        const int64_t max_rows = (PANEL_SMEM_BYTES / (int64_t)(GK * sizeof(T)));
        const int n_glob = S.n_tall_by_elem[sizeof(T) == 4 ? 0 : 1];
        (void)max_rows;
        if (n_glob > 0) {
            // rows of the tallest panel spread over a cluster of CTAs
            const int64_t rows_max = S.n_tall_rows[sizeof(T) == 4 ? 0 : 1];
            const int csize = plan.cluster;
            const int slab = (int)cdiv(rows_max, csize);
            const size_t smem = (size_t)slab * GK * sizeof(T);
            if (csize >= 2 && smem <= (size_t)PANEL_SMEM_BYTES) {
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3((unsigned)(n_glob * csize));
                cfg.blockDim = dim3(PC_THREADS);
                cfg.dynamicSmemBytes = smem;
                cfg.stream = st;
                cudaLaunchAttribute at[1];
                at[0].id = cudaLaunchAttributeClusterDimension;
                at[0].val.clusterDim.x = csize;
                at[0].val.clusterDim.y = 1;
                at[0].val.clusterDim.z = 1;
                cfg.attrs = at;
                cfg.numAttrs = 1;
                GB_CUDA(cudaLaunchKernelEx(&cfg, k_panel_cluster<T>, B, S.k, plan.d_act + S.act_off, slab));
            } else {
                k_panel<T><<<n_glob, PANEL_THREADS, 0, st>>>(B, S.k, plan.d_act + S.act_off);
                GB_LAUNCH_CHECK();
            }
        }
        if (S.n_panel > n_glob) {
            const int64_t rows = S.smem_rows[sizeof(T) == 4 ? 0 : 1];
            const size_t smem = (size_t)rows * GK * sizeof(T);
            k_panel_smem<T><<<S.n_panel - n_glob, PANEL_THREADS, smem, st>>>(B, S.k, plan.d_act + S.act_off + n_glob);
            GB_LAUNCH_CHECK();
        }
        if (S.swap_total > 0) {
            k_swap<T><<<(unsigned)cdiv(S.swap_total, 256), 256, 0, st>>>(B, S.k, plan.d_act + S.act_off,
                                                                       plan.d_pfx + S.swap_pfx, S.n_panel);
            GB_LAUNCH_CHECK();
        }
        if (S.trsm_blocks > 0) {
            k_trsm<T><<<(unsigned)S.trsm_blocks, TRSM_COLS, 0, st>>>(B, S.k, plan.d_act + S.act_off,
                                                                   plan.d_pfx + S.trsm_pfx, S.n_panel);
            GB_LAUNCH_CHECK();
        }
        if (S.upd_blocks > 0) {
            k_update<T><<<(unsigned)S.upd_blocks, 256, 0, st>>>(B, S.k, plan.d_act + S.act_off + S.upd_act_skip,
                                                              plan.d_pfx + S.upd_pfx, S.n_upd);
            GB_LAUNCH_CHECK();
        }
    }
    if (plan.nsys > 0) {
        k_perm<T><<<plan.nsys, 256, sizeof(int32_t) * std::min<int64_t>(plan.maxn, PERM_SMEM), st>>>(B);
        GB_LAUNCH_CHECK();
    }
    return GBVLM_OK;
}

template <class T>
int lu_batch_solve(const LuBatch<T>& B, int32_t nsys, int32_t max_nrhs, int64_t maxn, cudaStream_t st) {
    // X of the largest system in shared memory when it fits, else staged per column
    const size_t full = sizeof(T) * (size_t)maxn * TS_MAXRHS;
    const int use_smem = full <= (size_t)TS_SMEM_BYTES ? 1 : 0;
    if (!use_smem && nsys == 1) return lu_large_solve<T>(B, maxn, max_nrhs, st);
    const size_t smem = use_smem ? full : sizeof(T) * (size_t)maxn;
    GB_REQUIRE(smem <= (size_t)TS_SMEM_BYTES, "triangular solve: n=%lld needs %zu bytes of shared memory",
               (long long)maxn, smem);
    for (int32_t r0 = 0; r0 < max_nrhs; r0 += TS_MAXRHS) {
        k_trsolve<T><<<nsys, TS_THREADS, smem, st>>>(B, r0, TS_MAXRHS, use_smem);
        GB_LAUNCH_CHECK();
    }
    return GBVLM_OK;
}

template int lu_batch_factor<float>(const LuBatch<float>&, const LuPlan&, cudaStream_t);
template int lu_batch_factor<double>(const LuBatch<double>&, const LuPlan&, cudaStream_t);
template int lu_batch_solve<float>(const LuBatch<float>&, int32_t, int32_t, int64_t, cudaStream_t);
template int lu_batch_solve<double>(const LuBatch<double>&, int32_t, int32_t, int64_t, cudaStream_t);

// Build the per-step tables.  Systems must be sorted by n descending so the
// active systems of every step form a prefix of the order.
int lu_plan_build(LuPlan& plan, const std::vector<int64_t>& n_sorted, cudaStream_t st) {
    plan.release();
    GB_CUDA(cudaFuncSetAttribute(k_panel_smem<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, PANEL_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_panel_smem<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, PANEL_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_trsolve<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_trsolve<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_perm<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, PERM_SMEM * 4));
    GB_CUDA(cudaFuncSetAttribute(k_perm_apply<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_perm_apply<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, TS_SMEM_BYTES));
    GB_CUDA(cudaFuncSetAttribute(k_perm<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, PERM_SMEM * 4));
    plan.nsys = (int32_t)n_sorted.size();
    plan.maxn = n_sorted.empty() ? 0 : n_sorted[0];
    // largest cluster the device schedules for the tall-panel kernel (16 needs the non-portable opt-in)
    plan.cluster = 0;
    {
        cudaFuncSetAttribute(k_panel_cluster<float>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        cudaFuncSetAttribute(k_panel_cluster<double>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        GB_CUDA(cudaFuncSetAttribute(k_panel_cluster<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, PANEL_SMEM_BYTES));
        GB_CUDA(cudaFuncSetAttribute(k_panel_cluster<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, PANEL_SMEM_BYTES));
        for (int c : {16, 8, 4}) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(c);
            cfg.blockDim = dim3(PC_THREADS);
            cfg.dynamicSmemBytes = PANEL_SMEM_BYTES;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = c;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, k_panel_cluster<float>, &cfg) == cudaSuccess && nclusters > 0) {
                plan.cluster = c;
                break;
            }
            cudaGetLastError();
        }
    }
    const int nsys = (int)n_sorted.size();
    for (int i = 1; i < nsys; i++) GB_REQUIRE(n_sorted[i] <= n_sorted[i - 1], "lu plan: sizes not sorted");
    std::vector<int32_t> act;
    std::vector<int64_t> pfx;
    const int64_t maxn = nsys ? n_sorted[0] : 0;
    for (int64_t k = 0; k < maxn; k += GK) {
        LuStep S;
        S.k = k;
        S.act_off = (int64_t)act.size();
        int cnt = 0;
        while (cnt < nsys && n_sorted[cnt] > k) cnt++;
        for (int i = 0; i < cnt; i++) act.push_back(i);
        S.n_panel = cnt;
        for (int e = 0; e < 2; e++) {
            const int64_t es = e == 0 ? 4 : 8;
            const int64_t lim = PANEL_SMEM_BYTES / (GK * es);
            int tall = 0;
            while (tall < cnt && n_sorted[tall] - k > lim) tall++;
            S.n_tall_by_elem[e] = tall;
            S.n_tall_rows[e] = tall > 0 ? n_sorted[0] - k : 0;
            S.smem_rows[e] = tall < cnt ? n_sorted[tall] - k : 0;
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
        plan.steps.push_back(S);
    }
    if (!act.empty()) {
        GB_CUDA(cudaMalloc(&plan.d_act, act.size() * sizeof(int32_t)));
        GB_CUDA(cudaMemcpyAsync(plan.d_act, act.data(), act.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    if (!pfx.empty()) {
        GB_CUDA(cudaMalloc(&plan.d_pfx, pfx.size() * sizeof(int64_t)));
        GB_CUDA(cudaMemcpyAsync(plan.d_pfx, pfx.data(), pfx.size() * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    }
    GB_CUDA(cudaStreamSynchronize(st));
    return GBVLM_OK;
}

void LuPlan::release() {
    if (d_act) cudaFree(d_act);
    if (d_pfx) cudaFree(d_pfx);
    d_act = nullptr;
    d_pfx = nullptr;
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
    if (*work_bytes < sizeof(Tab)) {
        if (*work) cudaFree(*work);
        *work = nullptr;
        GB_CUDA(cudaMalloc(work, 256));
        *work_bytes = 256;
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
};

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
    rc = lu_batch_factor<T>(B, h->plan, st);
    if (rc) return rc;
    int32_t* hi = (int32_t*)host_scratch(sizeof(int32_t));
    GB_CUDA(cudaMemcpyAsync(hi, h->d_info, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (*hi != 0) {
        set_error("LU: exactly zero pivot at column %d", *hi);
        return GBVLM_ERR_SINGULAR;
    }
    return GBVLM_OK;
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
    return lu_batch_solve<T>(B, 1, (int32_t)nrhs, n, st);
}

extern "C" {

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
