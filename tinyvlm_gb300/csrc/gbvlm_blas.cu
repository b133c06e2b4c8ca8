// The rest of the vlm::Backend contract (vlm/include/vlm_backend.hpp:72-133,
// vlm/include/vlm_memory.hpp:22-37): device memory, the BLAS subset the
// drivers call, a least-squares solver, the strided 2-D sum, and the stream
// and event plumbing a host without PyTorch needs.  All kernels are plain
// SIMT: none of these calls is on the batched hot path (the drivers use fused
// kernels), so they are written for exactness and fixed summation order, not
// for peak throughput.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include "gbvlm_internal.h"
#include "gbvlm_math.cuh"

using namespace gbvlm;

namespace {

constexpr int BT = 256;  // threads of the reduction kernels

template <class T>
__device__ __forceinline__ double block_sum_d(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];  // every thread, same order
    __syncthreads();
    return r;
}

// ---------------------------------------------------------------------------
// Memory (vlm_memory.hpp:22-37): strided fill
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_fill_strided(T* p, int64_t stride, T v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i * stride] = v;
}

// ---------------------------------------------------------------------------
// BLAS (vlm_backend.hpp:78-97): column-major, BLAS argument meaning
// ---------------------------------------------------------------------------
// y = alpha op(A) x + beta y, no transpose: one thread per row (coalesced
// down the columns), the row's terms summed in column order
template <class T>
__global__ void k_gemv_n(int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x, int64_t incx, T beta,
                         T* y, int64_t incy) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        T acc = 0;
        for (int64_t j = 0; j < n; j++) acc += A[i + j * lda] * x[j * incx];
        T* yi = y + i * incy;
        *yi = beta == (T)0 ? alpha * acc : alpha * acc + beta * *yi;
    }
}

// transpose: one warp per output (a column of A), shuffle sum in a fixed order
template <class T>
__global__ void k_gemv_t(int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x, int64_t incx, T beta,
                         T* y, int64_t incy) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = w0; j < n; j += nw) {
        T acc = 0;
        for (int64_t i = lane; i < m; i += 32) acc += A[i + j * lda] * x[i * incx];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            T* yj = y + j * incy;
            *yj = beta == (T)0 ? alpha * acc : alpha * acc + beta * *yj;
        }
    }
}

// C = alpha op(A) op(B) + beta C: 64 x 64 tiles of C, 16-deep slices of K
// staged in shared memory, 4 x 4 outputs per thread (256 threads)
constexpr int GM = 64, GK = 16;
template <class T>
__global__ void __launch_bounds__(256) k_gemm(int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda,
                                              int ta, const T* B, int64_t ldb, int tb, T beta, T* C, int64_t ldc) {
    __shared__ T sa[GK][GM + 1];
    __shared__ T sb[GK][GM + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t r0 = (int64_t)blockIdx.x * GM, c0 = (int64_t)blockIdx.y * GM;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = 0;
    for (int64_t kk = 0; kk < k; kk += GK) {
        for (int e = threadIdx.x; e < GK * GM; e += 256) {
            const int r = e % GM, q = e / GM;  // element (r0 + r, kk + q) of op(A)
            const int64_t gi = r0 + r, gq = kk + q;
            T va = 0;
            if (gi < m && gq < k) va = ta ? A[gq + gi * lda] : A[gi + gq * lda];
            sa[q][r] = va;
            const int64_t gj = c0 + r;  // element (kk + q, c0 + r) of op(B)
            T vb = 0;
            if (gj < n && gq < k) vb = tb ? B[gj + gq * ldb] : B[gq + gj * ldb];
            sb[q][r] = vb;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < GK; q++) {
            T av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; a++) av[a] = sa[q][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; b++) bv[b] = sb[q][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) acc[a][b] += av[a] * bv[b];
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int64_t i = r0 + tx + 16 * a, j = c0 + ty + 16 * b;
            if (i < m && j < n) {
                T* c = C + i + j * ldc;
                *c = beta == (T)0 ? alpha * acc[a][b] : alpha * acc[a][b] + beta * *c;
            }
        }
}

template <class T>
__global__ void k_axpy2d(int64_t m, int64_t n, T alpha, const T* x, int64_t sx0, int64_t sx1, T* y, int64_t sy0,
                         int64_t sy1) {
    const int64_t tot = m * n;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < tot; g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = g % m, j = g / m;
        y[i * sy0 + j * sy1] += alpha * x[i * sx0 + j * sx1];
    }
}

template <class T>
__global__ void k_scal(int64_t n, T alpha, T* x, int64_t incx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i * incx] *= alpha;
}

// Euclidean norm in one block: the largest magnitude first, then the sum of
// squares of the scaled entries in double (no overflow or underflow for any
// finite input of either precision); out[0] = the norm
template <class T>
__global__ void __launch_bounds__(BT) k_nrm2(int64_t n, const T* x, int64_t incx, double* out) {
    __shared__ double sh[32];
    double mx = 0;
    for (int64_t i = threadIdx.x; i < n; i += BT) mx = fmax(mx, fabs((double)x[i * incx]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = 0;
    for (int k = 0; k < BT / 32; k++) mx = fmax(mx, sh[k]);
    __syncthreads();
    CSum s;
    if (mx > 0)
        for (int64_t i = threadIdx.x; i < n; i += BT) {
            const double v = (double)x[i * incx] / mx;
            s.add(v * v);
        }
    const double tot = block_sum_d<T>(s.value(), sh);
    if (threadIdx.x == 0) out[0] = mx > 0 ? mx * sqrt(tot) : 0.0;
}

// sum of an (m, n) view with element strides (s0, s1), compensated in double
template <class T>
__global__ void __launch_bounds__(BT) k_sum2d(int64_t m, int64_t n, const T* x, int64_t s0, int64_t s1, double* out) {
    __shared__ double sh[32];
    CSum s;
    const int64_t tot = m * n;
    for (int64_t g = threadIdx.x; g < tot; g += BT) s.add((double)x[(g % m) * s0 + (g / m) * s1]);
    const double r = block_sum_d<T>(s.value(), sh);
    if (threadIdx.x == 0) out[0] = r;
}

// ---------------------------------------------------------------------------
// LSQ (vlm_backend.hpp:121-133; LAPACK ?gels with trans = 'N', m >= n):
// Householder QR of A (m x n) in one block, Q^T applied to the right-hand
// sides as each reflector is formed, then R x = (Q^T B)[0:n] by back
// substitution.  The first n rows of B receive the solution, rows n..m-1
// the components of the residual, A is overwritten by R (upper triangle) and
// the reflectors (below).  status[0] = 1-based column of an exactly zero
// diagonal of R (rank deficiency), else 0.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(BT) k_lsq_qr(int64_t m, int64_t n, T* A, int64_t lda, T* B, int64_t nrhs,
                                                int64_t ldb, int32_t* status) {
    __shared__ double sh[32];
    __shared__ double s_tau, s_beta;
    for (int64_t j = 0; j < n; j++) {
        T* aj = A + j * lda;
        // norm of A[j+1:m, j]
        CSum s;
        for (int64_t i = j + 1 + threadIdx.x; i < m; i += BT) s.add((double)aj[i] * (double)aj[i]);
        const double sig = block_sum_d<T>(s.value(), sh);
        if (threadIdx.x == 0) {
            const double alpha = (double)aj[j];
            if (sig == 0.0) {  // nothing below the diagonal: H = I
                s_tau = 0.0;
                s_beta = alpha;
            } else {
                const double nrm = sqrt(alpha * alpha + sig);
                const double beta = alpha >= 0 ? -nrm : nrm;
                s_tau = (beta - alpha) / beta;
                s_beta = beta;
                aj[j] = (T)(alpha - beta);  // v0 before scaling
            }
        }
        __syncthreads();
        const double tau = s_tau;
        if (tau != 0.0) {
            const double v0 = (double)aj[j];
            for (int64_t i = j + 1 + threadIdx.x; i < m; i += BT) aj[i] = (T)((double)aj[i] / v0);  // v = [1, ...]
            __syncthreads();
            // apply H = I - tau v v^T to the later columns of A and to B
            for (int64_t c = j + 1; c < n + nrhs; c++) {
                T* col = c < n ? A + c * lda : B + (c - n) * ldb;
                CSum w;
                if (threadIdx.x == 0) w.add((double)col[j]);
                for (int64_t i = j + 1 + threadIdx.x; i < m; i += BT) w.add((double)aj[i] * (double)col[i]);
                const double dot = tau * block_sum_d<T>(w.value(), sh);
                if (threadIdx.x == 0) col[j] = (T)((double)col[j] - dot);
                for (int64_t i = j + 1 + threadIdx.x; i < m; i += BT) col[i] = (T)((double)col[i] - dot * (double)aj[i]);
                __syncthreads();
            }
        }
        if (threadIdx.x == 0) aj[j] = (T)s_beta;  // R(j, j)
        __syncthreads();
    }
    // back substitution, one thread per right-hand side
    for (int64_t r = threadIdx.x; r < nrhs; r += BT) {
        T* b = B + r * ldb;
        for (int64_t i = n - 1; i >= 0; i--) {
            double acc = (double)b[i];
            for (int64_t c = i + 1; c < n; c++) acc -= (double)A[i + c * lda] * (double)b[c];
            const double d = (double)A[i + i * lda];
            if (d == 0.0) {
                atomicCAS(status, 0, (int32_t)(i + 1));
                b[i] = (T)0;
            } else {
                b[i] = (T)(acc / d);
            }
        }
    }
}

inline unsigned grid_for(int64_t n, int threads = 256) {
    int64_t g = cdiv(n > 0 ? n : 1, threads);
    return (unsigned)(g < 65535 * 8 ? g : 65535 * 8);
}

int sync_scalar(const double* d, double* host, cudaStream_t st) {
    double* h = (double*)host_scratch(sizeof(double));
    GB_REQUIRE(h != nullptr, "pinned host allocation failed");
    GB_CUDA(cudaMemcpyAsync(h, d, sizeof(double), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    *host = *h;
    return GBVLM_OK;
}

template <class T>
int gemv(int32_t trans, int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x, int64_t incx, T beta, T* y,
         int64_t incy, cudaStream_t st) {
    GB_REQUIRE(m >= 0 && n >= 0 && lda >= (m > 1 ? m : 1) && incx >= 1 && incy >= 1, "bad gemv sizes");
    GB_REQUIRE((m == 0 || n == 0) || (A && x && y), "null gemv operand");
    const int64_t rows = trans ? n : m;
    if (rows == 0) return GBVLM_OK;
    if (!trans) {
        k_gemv_n<T><<<grid_for(m), 256, 0, st>>>(m, n, alpha, A, lda, x, incx, beta, y, incy);
    } else {
        k_gemv_t<T><<<grid_for(32 * n), 256, 0, st>>>(m, n, alpha, A, lda, x, incx, beta, y, incy);
    }
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

template <class T>
int gemm(int32_t ta, int32_t tb, int64_t m, int64_t n, int64_t k, T alpha, const T* A, int64_t lda, const T* B,
         int64_t ldb, T beta, T* C, int64_t ldc, cudaStream_t st) {
    GB_REQUIRE(m >= 0 && n >= 0 && k >= 0, "bad gemm sizes");
    GB_REQUIRE(lda >= ((ta ? k : m) > 1 ? (ta ? k : m) : 1) && ldb >= ((tb ? n : k) > 1 ? (tb ? n : k) : 1) &&
                   ldc >= (m > 1 ? m : 1),
               "gemm leading dimension too small");
    if (m == 0 || n == 0) return GBVLM_OK;
    GB_REQUIRE(C && (k == 0 || (A && B)), "null gemm operand");
    GB_REQUIRE(cdiv(n, GM) <= 65535, "gemm: n too large");
    dim3 grid((unsigned)cdiv(m, GM), (unsigned)cdiv(n, GM));
    k_gemm<T><<<grid, 256, 0, st>>>(m, n, k, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc);
    GB_LAUNCH_CHECK();
    return GBVLM_OK;
}

template <class T>
int lsq(int64_t m, int64_t n, T* A, int64_t lda, T* B, int64_t nrhs, int64_t ldb, cudaStream_t st) {
    GB_REQUIRE(n >= 1 && m >= n && nrhs >= 1, "least squares needs m >= n >= 1 and nrhs >= 1 (m=%lld n=%lld)",
               (long long)m, (long long)n);
    GB_REQUIRE(A && B && lda >= m && ldb >= m, "bad least-squares operands");
    void* d = nullptr;
    int rc = device_scratch(sizeof(int32_t), &d, st);
    if (rc) return rc;
    GB_CUDA(cudaMemsetAsync(d, 0, sizeof(int32_t), st));
    k_lsq_qr<T><<<1, BT, 0, st>>>(m, n, A, lda, B, nrhs, ldb, (int32_t*)d);
    GB_LAUNCH_CHECK();
    int32_t* h = (int32_t*)host_scratch(sizeof(int32_t));
    GB_REQUIRE(h != nullptr, "pinned host allocation failed");
    GB_CUDA(cudaMemcpyAsync(h, d, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (*h != 0) {
        set_error("least squares: R(%d, %d) is exactly zero (A is rank deficient)", *h, *h);
        return GBVLM_ERR_SINGULAR;
    }
    return GBVLM_OK;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Memory
// ---------------------------------------------------------------------------
int gbvlm_mem_alloc(int32_t location, int64_t bytes, void** out) {
    GB_REQUIRE(out && bytes >= 0, "bad allocation arguments");
    GB_REQUIRE(location == GBVLM_LOC_DEVICE || location == GBVLM_LOC_HOST, "unknown location %d", location);
    *out = nullptr;
    if (bytes == 0) return GBVLM_OK;
    cudaError_t e = location == GBVLM_LOC_DEVICE ? cudaMalloc(out, (size_t)bytes) : cudaMallocHost(out, (size_t)bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("%s of %lld bytes failed: %s", location == GBVLM_LOC_DEVICE ? "cudaMalloc" : "cudaMallocHost",
                  (long long)bytes, cudaGetErrorString(e));
        *out = nullptr;
        return GBVLM_ERR_NOMEM;
    }
    return GBVLM_OK;
}

int gbvlm_mem_free(int32_t location, void* ptr) {
    GB_REQUIRE(location == GBVLM_LOC_DEVICE || location == GBVLM_LOC_HOST, "unknown location %d", location);
    if (!ptr) return GBVLM_OK;
    GB_CUDA(location == GBVLM_LOC_DEVICE ? cudaFree(ptr) : cudaFreeHost(ptr));
    return GBVLM_OK;
}

int gbvlm_mem_copy(int32_t dst_loc, void* dst, int64_t dst_stride, int32_t src_loc, const void* src,
                   int64_t src_stride, int64_t elem_size, int64_t size, gbvlm_stream stream) {
    GB_REQUIRE(elem_size >= 1 && size >= 0 && dst_stride >= 1 && src_stride >= 1, "bad copy sizes");
    GB_REQUIRE((dst_loc == GBVLM_LOC_DEVICE || dst_loc == GBVLM_LOC_HOST) &&
                   (src_loc == GBVLM_LOC_DEVICE || src_loc == GBVLM_LOC_HOST),
               "unknown location");
    if (size == 0) return GBVLM_OK;
    GB_REQUIRE(dst && src, "null copy operand");
    cudaStream_t st = to_cuda(stream);
    if (dst_loc == GBVLM_LOC_HOST && src_loc == GBVLM_LOC_HOST) {
        char* d = (char*)dst;
        const char* s = (const char*)src;
        for (int64_t i = 0; i < size; i++) memcpy(d + i * dst_stride * elem_size, s + i * src_stride * elem_size, elem_size);
        return GBVLM_OK;
    }
    if (dst_stride == 1 && src_stride == 1) {
        GB_CUDA(cudaMemcpyAsync(dst, src, (size_t)(size * elem_size), cudaMemcpyDefault, st));
    } else {
        GB_CUDA(cudaMemcpy2DAsync(dst, (size_t)(dst_stride * elem_size), src, (size_t)(src_stride * elem_size),
                                  (size_t)elem_size, (size_t)size, cudaMemcpyDefault, st));
    }
    // a host side makes the copy synchronous for the caller (the reference's
    // Memory::copy returns with the data in place, vlm_backend_cuda.cu:109-126)
    if (dst_loc == GBVLM_LOC_HOST || src_loc == GBVLM_LOC_HOST) GB_CUDA(cudaStreamSynchronize(st));
    return GBVLM_OK;
}

#define DEF_FILL(sfx, T)                                                                                      \
    int gbvlm_mem_fill_##sfx(int32_t location, T* ptr, int64_t stride, T value, int64_t size, gbvlm_stream stream) { \
        GB_REQUIRE(size >= 0 && stride >= 1, "bad fill sizes");                                               \
        if (size == 0) return GBVLM_OK;                                                                       \
        GB_REQUIRE(ptr != nullptr, "null fill pointer");                                                      \
        if (location == GBVLM_LOC_HOST) {                                                                     \
            for (int64_t i = 0; i < size; i++) ptr[i * stride] = value;                                       \
            return GBVLM_OK;                                                                                  \
        }                                                                                                     \
        GB_REQUIRE(location == GBVLM_LOC_DEVICE, "unknown location %d", location);                            \
        k_fill_strided<T><<<grid_for(size), 256, 0, to_cuda(stream)>>>(ptr, stride, value, size);             \
        GB_LAUNCH_CHECK();                                                                                    \
        return GBVLM_OK;                                                                                      \
    }
DEF_FILL(f32, float)
DEF_FILL(f64, double)

// ---------------------------------------------------------------------------
// BLAS, LSQ, strided sum
// ---------------------------------------------------------------------------
#define DEF_BLAS(sfx, T)                                                                                      \
    int gbvlm_blas_gemv_##sfx(int32_t trans, int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x, \
                              int64_t incx, T beta, T* y, int64_t incy, gbvlm_stream stream) {                \
        return gemv<T>(trans, m, n, alpha, A, lda, x, incx, beta, y, incy, to_cuda(stream));                  \
    }                                                                                                         \
    int gbvlm_blas_gemm_##sfx(int32_t trans_a, int32_t trans_b, int64_t m, int64_t n, int64_t k, T alpha,     \
                              const T* A, int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc,    \
                              gbvlm_stream stream) {                                                          \
        return gemm<T>(trans_a, trans_b, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, to_cuda(stream));      \
    }                                                                                                         \
    int gbvlm_blas_axpy_##sfx(int64_t n, T alpha, const T* x, int64_t incx, T* y, int64_t incy,               \
                              gbvlm_stream stream) {                                                          \
        GB_REQUIRE(n >= 0 && incx >= 1 && incy >= 1, "bad axpy sizes");                                      \
        if (n == 0) return GBVLM_OK;                                                                          \
        GB_REQUIRE(x && y, "null axpy operand");                                                              \
        k_axpy2d<T><<<grid_for(n), 256, 0, to_cuda(stream)>>>(n, 1, alpha, x, incx, 0, y, incy, 0);            \
        GB_LAUNCH_CHECK();                                                                                    \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_blas_axpy2d_##sfx(int64_t m, int64_t n, T alpha, const T* x, int64_t x_s0, int64_t x_s1, T* y,  \
                                int64_t y_s0, int64_t y_s1, gbvlm_stream stream) {                            \
        GB_REQUIRE(m >= 0 && n >= 0, "bad axpy sizes");                                                       \
        if (m == 0 || n == 0) return GBVLM_OK;                                                                \
        GB_REQUIRE(x && y, "null axpy operand");                                                              \
        k_axpy2d<T><<<grid_for(m * n), 256, 0, to_cuda(stream)>>>(m, n, alpha, x, x_s0, x_s1, y, y_s0, y_s1);  \
        GB_LAUNCH_CHECK();                                                                                    \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_blas_scal_##sfx(int64_t n, T alpha, T* x, int64_t incx, gbvlm_stream stream) {                  \
        GB_REQUIRE(n >= 0 && incx >= 1, "bad scal sizes");                                                    \
        if (n == 0) return GBVLM_OK;                                                                          \
        GB_REQUIRE(x != nullptr, "null scal operand");                                                        \
        k_scal<T><<<grid_for(n), 256, 0, to_cuda(stream)>>>(n, alpha, x, incx);                               \
        GB_LAUNCH_CHECK();                                                                                    \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_blas_nrm2_##sfx(int64_t n, const T* x, int64_t incx, T* out, gbvlm_stream stream) {             \
        GB_REQUIRE(n >= 0 && incx >= 1 && out, "bad nrm2 arguments");                                        \
        if (n == 0) {                                                                                         \
            *out = (T)0;                                                                                      \
            return GBVLM_OK;                                                                                  \
        }                                                                                                     \
        GB_REQUIRE(x != nullptr, "null nrm2 operand");                                                        \
        cudaStream_t st = to_cuda(stream);                                                                    \
        void* d = nullptr;                                                                                    \
        int rc = device_scratch(sizeof(double), &d, st);                                                      \
        if (rc) return rc;                                                                                    \
        k_nrm2<T><<<1, BT, 0, st>>>(n, x, incx, (double*)d);                                                  \
        GB_LAUNCH_CHECK();                                                                                    \
        double h;                                                                                             \
        if ((rc = sync_scalar((const double*)d, &h, st))) return rc;                                          \
        *out = (T)h;                                                                                          \
        return GBVLM_OK;                                                                                      \
    }                                                                                                         \
    int gbvlm_lsq_solve_##sfx(int64_t m, int64_t n, T* A, int64_t lda, T* B, int64_t nrhs, int64_t ldb,       \
                              gbvlm_stream stream) {                                                          \
        return lsq<T>(m, n, A, lda, B, nrhs, ldb, to_cuda(stream));                                           \
    }                                                                                                         \
    int gbvlm_sum2d_##sfx(const T* x, int64_t m, int64_t n, int64_t stride0, int64_t stride1, T* out,         \
                          gbvlm_stream stream) {                                                              \
        GB_REQUIRE(m >= 0 && n >= 0 && out, "bad sum arguments");                                             \
        if (m == 0 || n == 0) {                                                                               \
            *out = (T)0;                                                                                      \
            return GBVLM_OK;                                                                                  \
        }                                                                                                     \
        GB_REQUIRE(x != nullptr, "null sum operand");                                                         \
        cudaStream_t st = to_cuda(stream);                                                                    \
        void* d = nullptr;                                                                                    \
        int rc = device_scratch(sizeof(double), &d, st);                                                      \
        if (rc) return rc;                                                                                    \
        k_sum2d<T><<<1, BT, 0, st>>>(m, n, x, stride0, stride1, (double*)d);                                  \
        GB_LAUNCH_CHECK();                                                                                    \
        double h;                                                                                             \
        if ((rc = sync_scalar((const double*)d, &h, st))) return rc;                                          \
        *out = (T)h;                                                                                          \
        return GBVLM_OK;                                                                                      \
    }
DEF_BLAS(f32, float)
DEF_BLAS(f64, double)

// ---------------------------------------------------------------------------
// Streams, events, device queries
// ---------------------------------------------------------------------------
int gbvlm_stream_create(gbvlm_stream* out) {
    GB_REQUIRE(out != nullptr, "null stream pointer");
    cudaStream_t s = nullptr;
    GB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    *out = (gbvlm_stream)s;
    return GBVLM_OK;
}

int gbvlm_stream_destroy(gbvlm_stream s) {
    if (s) GB_CUDA(cudaStreamDestroy(to_cuda(s)));
    return GBVLM_OK;
}

int gbvlm_stream_synchronize(gbvlm_stream s) {
    GB_CUDA(cudaStreamSynchronize(to_cuda(s)));
    return GBVLM_OK;
}

int gbvlm_device_synchronize(void) {
    GB_CUDA(cudaDeviceSynchronize());
    return GBVLM_OK;
}

int gbvlm_event_create(gbvlm_event* out) {
    GB_REQUIRE(out != nullptr, "null event pointer");
    cudaEvent_t e = nullptr;
    GB_CUDA(cudaEventCreate(&e));
    *out = (gbvlm_event)e;
    return GBVLM_OK;
}

int gbvlm_event_destroy(gbvlm_event e) {
    if (e) GB_CUDA(cudaEventDestroy((cudaEvent_t)e));
    return GBVLM_OK;
}

int gbvlm_event_record(gbvlm_event e, gbvlm_stream s) {
    GB_REQUIRE(e != nullptr, "null event");
    GB_CUDA(cudaEventRecord((cudaEvent_t)e, to_cuda(s)));
    return GBVLM_OK;
}

int gbvlm_event_synchronize(gbvlm_event e) {
    GB_REQUIRE(e != nullptr, "null event");
    GB_CUDA(cudaEventSynchronize((cudaEvent_t)e));
    return GBVLM_OK;
}

int gbvlm_event_elapsed_ms(gbvlm_event start, gbvlm_event end, float* ms) {
    GB_REQUIRE(start && end && ms, "null event argument");
    GB_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)start, (cudaEvent_t)end));
    return GBVLM_OK;
}

int gbvlm_device_info(int32_t* sm_count, int64_t* free_bytes, int64_t* total_bytes) {
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    if (sm_count) {
        int v = 0;
        GB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
        *sm_count = v;
    }
    if (free_bytes || total_bytes) {
        size_t f = 0, t = 0;
        GB_CUDA(cudaMemGetInfo(&f, &t));
        if (free_bytes) *free_bytes = (int64_t)f;
        if (total_bytes) *total_bytes = (int64_t)t;
    }
    return GBVLM_OK;
}

}  // extern "C"
