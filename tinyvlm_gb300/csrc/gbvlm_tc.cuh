// Tensor-core (tcgen05, TF32) trailing update of the blocked LU:
//
//     C[r, c] -= sum_kk L[r, kk] * U[kk, c]
//
// over 128 x 128 output tiles, for every active system of a step.  L, U and
// C live in the system's column-major matrix (leading dimension ld).
//
// Precision: each fp32 operand x is split as hi = tf32(x) (round to nearest)
// and lo = x - hi; the product is accumulated in fp32 in tensor memory as
// hi*hi + hi*lo + lo*hi ("3xTF32"), which keeps the update at fp32 accuracy
// (the dropped lo*lo term is ~2^-22 relative).  PASSES = 1 keeps hi*hi only
// (plain TF32).
//
// Per CTA (256 threads, one output tile of 128 x 128 or 128 x 256, two CTAs
// per SM; a wide tile moves twice the C bytes per operand-load round trip):
//   * operands are staged in shared memory per 32-wide K chunk, in the
//     K-major, 128-byte-swizzled layout the MMA reads: row r of a chunk is
//     128 bytes (32 tf32), its 16-byte pieces permuted by XOR with r % 8,
//     8-row groups 1024 bytes apart.  With STAGES = 2 threads fill chunk
//     c+1 while the tensor core works on chunk c; with one stage the other
//     CTA on the SM fills that time;
//   * one thread issues tcgen05.mma (M = 128, N = tile width, K = 8 per
//     instruction) into an fp32 accumulator of that many tensor-memory
//     columns and commits each chunk to that stage's mbarrier;
//   * epilogue: warp w reads accumulator lanes 32(w%4)..+31 (tile rows) and
//     the (w/4) half of the columns with tcgen05.ld and subtracts them from C,
//     a warp covering 32 consecutive rows of one column per store.
// Every wait on an mbarrier is bounded in time; a CTA that runs out sets the
// error word, skips its epilogue and still frees its tensor memory.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbvlm {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int BN_WIDE = 256;                    // wide tiles: 128 x 256, the A chunk serves twice the columns
constexpr int THREADS = 256;
constexpr int CHUNK_BYTES = BM * BK * 4;        // one operand chunk, 16 KB
constexpr int STAGE_BYTES = 4 * CHUNK_BYTES;    // A hi, A lo, B hi, B lo
constexpr int STAGES = 1;                       // one stage: two CTAs share an SM and hide each other's latency
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;  // + alignment slack
constexpr int TMEM_COLS = BN;
// a tile of TBN columns: A hi/lo chunks of 128 rows, B hi/lo chunks of TBN rows
template <int TBN> constexpr int stage_bytes() { return 2 * CHUNK_BYTES + 2 * TBN * BK * 4; }
template <int TBN> constexpr int smem_bytes() { return STAGES * stage_bytes<TBN>() + 1024; }
static_assert(smem_bytes<BN>() == SMEM_BYTES, "tile shared-memory layout");
constexpr unsigned long long WAIT_NS = 2000000000ull;  // 2 s bound on any wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// wait for the phase of the given parity to complete; false after WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > WAIT_NS) return false;
    return true;
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D (tensor memory) (+)= A (smem) * B (smem)^T, kind::tf32
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive on the mbarrier once every MMA issued so far by this thread is done
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart; `saddr` is the chunk's (1024-aligned) address plus the
// byte offset of the K step inside the 128-byte row
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
    d |= (uint64_t)1 << 16;                     // leading-dimension offset (not used by swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;           // stride-dimension offset
    d |= (uint64_t)1 << 46;                     // descriptor version
    d |= (uint64_t)2 << 61;                     // 128-byte swizzle
    return d;
}

// instruction descriptor: fp32 accumulator, tf32 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// byte offset of element (row, kk) in a 128-row x 32-column swizzled chunk
__device__ __forceinline__ uint32_t sw128_off(int row, int kk) {
    return (uint32_t)((row >> 3) * 1024 + (row & 7) * 128 + ((((kk >> 2) ^ (row & 7)) & 7) << 4) + ((kk & 3) << 2));
}

__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, float a, float b, float c, float d) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}
__device__ __forceinline__ void st_shared_f32(uint32_t addr, float a) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(a) : "memory");
}

// One 128 x 128 tile: C(r0.., c0..) -= L(r0.., 0..K) * U(0..K, c0..).
//   L(r, kk) = Lp[r + kk * ldl], U(kk, c) = Up[kk + c * ldu], C(r, c) = Cp[r + c * ldc];
//   rows r < m_rows and columns c < n_cols exist (tile-relative bounds).
// WITHHOLD (a test hook's instantiation only): the MMA thread issues and
// commits nothing, so the bounded mbarrier waits must run out; no MMA is
// ever in flight, the CTA frees its tensor memory and sets the error word.
// TBN: tile columns, 128 or 256 (one MMA of N = TBN per K step; TBN
// accumulator columns of tensor memory; shared memory smem_bytes<TBN>()).
template <int PASSES, bool WITHHOLD = false, int TBN = BN>
__device__ __forceinline__ void update_tile(const float* Lp, int64_t ldl, const float* Up, int64_t ldu, float* Cp,
                                            int64_t ldc, int m_rows, int n_cols, int K, unsigned char* smem_raw,
                                            uint64_t* bar, uint32_t* tslot, int* err) {
    static_assert(TBN == 128 || TBN == 256, "tile width");
    constexpr int SB = stage_bytes<TBN>();
    constexpr int BCHUNK = TBN * BK * 4;
    constexpr int BP = TBN / 32;       // B loads per thread: (column, 4 consecutive K) pairs
    constexpr int EQ = TBN / 64;       // 32-column accumulator groups per thread in the epilogue
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    // the tile's C lines into L2 while the K loop runs, so the epilogue's
    // reads of C hit L2: the first and last row of each 32-row run of each
    // column (a run may straddle two 128-byte lines)
    for (int e = tid; e < TBN * 8; e += THREADS) {
        const int col = e >> 3, row = 32 * ((e >> 1) & 3) + 31 * (e & 1);
        if (col < n_cols && row < m_rows) prefetch_l2(Cp + row + (int64_t)col * ldc);
    }
    constexpr uint32_t idesc = idesc_tf32(BM, TBN);
    const int nchunks = (K + BK - 1) / BK;
    bool ok = true;
    int committed = -1;  // last chunk whose MMAs were committed
    // operand chunks pass through registers: chunk c + 1 is loaded from global
    // memory while the MMAs of chunk c run (one shared-memory stage)
    const int arow = tid & (BM - 1), akh = (tid >> 7) * 16;
    // B: pair j of this thread is column (tid + 256 j) / 8 and K values
    // 4 ((tid + 256 j) % 8) .. +3, consecutive in memory (U is K-contiguous):
    // a warp reads four columns' 128-byte runs, and each pair lands in the
    // swizzled tile as one 16-byte store
    const int bk = 4 * (tid & 7), bc = tid >> 3;
    float va[16], vb[BP][4];
    auto load_chunk = [&](int c) {
        const int kc = c * BK;
        const bool rv = arow < m_rows;  // A: thread = tile row, 16 K values of its half
#pragma unroll
        for (int kk = 0; kk < 16; kk++)
            va[kk] = (rv && kc + akh + kk < K) ? Lp[arow + (int64_t)(kc + akh + kk) * ldl] : 0.f;
#pragma unroll
        for (int j = 0; j < BP; j++) {
            const int col = bc + 32 * j;
            const bool cv = col < n_cols;
#pragma unroll
            for (int e = 0; e < 4; e++)
                vb[j][e] = (cv && kc + bk + e < K) ? Up[(kc + bk + e) + (int64_t)col * ldu] : 0.f;
        }
    };
    // the first chunk's loads in flight while tensor memory and the barrier are set up
    if (nchunks > 0) load_chunk(0);
    if (wid == 0) {
        tmem_alloc(tslot, TBN);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < STAGES; i++) mbar_init(&bar[i], 1);
        fence_mbar_init();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    for (int c = 0; c < nchunks; c++) {
        const int s = c % STAGES;
        // stage s is free once the MMAs of chunk c - STAGES are done
        const bool free_ = c < STAGES || mbar_wait(&bar[s], ((c - STAGES) / STAGES) & 1);
        const uint32_t a_hi = base + s * SB, a_lo = a_hi + CHUNK_BYTES;
        const uint32_t b_hi = a_hi + 2 * CHUNK_BYTES, b_lo = b_hi + BCHUNK;
        if (free_) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const uint32_t off = sw128_off(arow, akh + 4 * j);
                const float h0 = tf32_hi(va[4 * j]), h1 = tf32_hi(va[4 * j + 1]);
                const float h2 = tf32_hi(va[4 * j + 2]), h3 = tf32_hi(va[4 * j + 3]);
                st_shared_v4(a_hi + off, h0, h1, h2, h3);
                if (PASSES > 1)
                    st_shared_v4(a_lo + off, va[4 * j] - h0, va[4 * j + 1] - h1, va[4 * j + 2] - h2,
                                 va[4 * j + 3] - h3);
            }
#pragma unroll
            for (int j = 0; j < BP; j++) {
                const uint32_t off = sw128_off(bc + 32 * j, bk);
                const float h0 = tf32_hi(vb[j][0]), h1 = tf32_hi(vb[j][1]);
                const float h2 = tf32_hi(vb[j][2]), h3 = tf32_hi(vb[j][3]);
                st_shared_v4(b_hi + off, h0, h1, h2, h3);
                if (PASSES > 1)
                    st_shared_v4(b_lo + off, vb[j][0] - h0, vb[j][1] - h1, vb[j][2] - h2, vb[j][3] - h3);
            }
            if (c + 1 < nchunks) load_chunk(c + 1);
        }
        fence_async_smem();  // generic-proxy stores visible to the tensor core
        fence_before_sync();
        ok = __syncthreads_and(free_) != 0;  // uniform over the CTA
        if (!ok) break;
        if (tid == 0 && !WITHHOLD) {
            fence_after_sync();
#pragma unroll
            for (int ks = 0; ks < BK / 8; ks++) {
                const uint64_t ah = sw128_desc(a_hi + ks * 32), bh = sw128_desc(b_hi + ks * 32);
                mma_tf32(tmem, ah, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
                if (PASSES > 1) {
                    const uint64_t al = sw128_desc(a_lo + ks * 32), bl = sw128_desc(b_lo + ks * 32);
                    mma_tf32(tmem, ah, bl, idesc, 1u);
                    mma_tf32(tmem, al, bh, idesc, 1u);
                }
            }
            mma_commit(&bar[s]);
        }
        committed = c;
    }
    // the first 32 columns of this thread's C in flight while the last MMAs finish
    const int erow = 32 * (wid & 3) + lane;
    const bool erv = erow < m_rows;
    float cpre[32];
    {
        const int cb = (TBN / 2) * (wid >> 2);
#pragma unroll
        for (int j = 0; j < 32; j++) cpre[j] = (ok && erv && cb + j < n_cols) ? Cp[erow + (int64_t)(cb + j) * ldc] : 0.f;
    }
    // every committed MMA done (the last commit covers all earlier ones)
    bool done = committed < 0 || mbar_wait(&bar[committed % STAGES], (committed / STAGES) & 1);
    done = __syncthreads_and(done) != 0;
    fence_after_sync();
    if (ok && done) {
#pragma unroll
        for (int q = 0; q < EQ; q++) {
            const int cb = (TBN / 2) * (wid >> 2) + 32 * q;
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(32 * (wid & 3)) << 16) + (uint32_t)cb, v);
            if (erv) {
                // all 32 loads before the stores: a load may not pass a store to the same array
                float c[32];
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const int col = cb + j;
                    c[j] = q == 0 ? cpre[j] : (col < n_cols ? Cp[erow + (int64_t)col * ldc] : 0.f);
                }
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const int col = cb + j;
                    if (col < n_cols) Cp[erow + (int64_t)col * ldc] = c[j] - v[j];
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    fence_before_sync();
    __syncthreads();
    if (wid == 0) tmem_dealloc(tmem, TBN);
}

}  // namespace tc
}  // namespace gbvlm

namespace gbvlm {

// ===========================================================================
// Persistent, warp-specialised form of the same update.  One CTA per SM walks
// the tiles blockIdx.x, blockIdx.x + gridDim.x, ...; its warps split the work
//   warps 0-7   producers in two groups of four: group g fills stage g for
//               the chunks g, g+2, ... (hi/lo split into shared memory)
//   warp 8      one thread issues the MMAs of a tile into one of two
//               accumulators in tensor memory (tfull/tempty per accumulator)
//   warps 9-12  epilogue: the tile's C is copied to shared memory with
//               cp.async while the MMAs run; then C - acc is stored and the
//               accumulator released
// so operand loads, MMAs and the C read-modify-write overlap, with the C
// reads in flight as asynchronous copies.  Every wait is bounded; a role that
// gives up raises a shared abort flag that ends the others' waits, the MMA
// thread drains its MMAs, and the CTA frees its tensor memory and sets the
// error word.
// ===========================================================================
namespace tc {

constexpr int PSTAGES = 2;  // one per producer group
constexpr int P_GROUP_WARPS = 4;
constexpr int P_PROD_WARPS = PSTAGES * P_GROUP_WARPS, P_EPI_WARPS = 4;
constexpr int P_MMA_WARP = P_PROD_WARPS;
constexpr int P_THREADS = (P_PROD_WARPS + 1 + P_EPI_WARPS) * 32;
constexpr int C_TILE_BYTES = BM * BN * 4;  // C staged column-major, [col][row]
constexpr int P_SMEM_BYTES = PSTAGES * STAGE_BYTES + C_TILE_BYTES + 1024;
constexpr int P_TMEM_COLS = 2 * BN;

// C(r, c) -= sum_kk L(r, kk) U(kk, c) for r < m_rows, c < n_cols (tile-relative)
struct TileJob {
    const float* Lp;
    int64_t ldl;
    const float* Up;
    int64_t ldu;
    float* Cp;
    int64_t ldc;
    int m_rows, n_cols, K;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ float ld_shared_f32(uint32_t addr) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

// bounded wait that also ends when another role has aborted
__device__ __forceinline__ bool pwait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (global_ns() - t0 > WAIT_NS) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

template <int PASSES, class JobOf>
__device__ __forceinline__ void update_persistent(int64_t ntiles, JobOf job_of, unsigned char* smem_raw, int* err) {
    __shared__ __align__(8) uint64_t full[PSTAGES], empty[PSTAGES], tfull[2], tempty[2], drain;
    __shared__ uint32_t tslot;
    __shared__ int abort_flag;
    const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    const uint32_t cbuf = base + PSTAGES * STAGE_BYTES;
    if (wid == 0) {
        tmem_alloc(&tslot, P_TMEM_COLS);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int i = 0; i < PSTAGES; i++) {
            mbar_init(&full[i], P_GROUP_WARPS * 32);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], P_EPI_WARPS * 32);
        }
        mbar_init(&drain, 1);
        abort_flag = 0;
        fence_mbar_init();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tslot;
    constexpr uint32_t idesc = idesc_tf32(BM, BN);

    if (wid < P_PROD_WARPS) {
        // ---- producers: group pg fills stage pg for the chunks pg, pg+2, ... ----
        const int pg = wid / P_GROUP_WARPS, pw = wid % P_GROUP_WARPS, ptid = tid % (P_GROUP_WARPS * 32);
        const uint32_t a_hi = base + pg * STAGE_BYTES, a_lo = a_hi + CHUNK_BYTES;
        const uint32_t b_hi = a_hi + 2 * CHUNK_BYTES, b_lo = a_hi + 3 * CHUNK_BYTES;
        int g = 0;    // chunk counter over all tiles
        int use = 0;  // this group's uses of its stage
        bool ok = true;
        for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
            const TileJob J = job_of(t);
            const int nch = (J.K + BK - 1) / BK;
            for (int c = 0; c < nch; c++, g++) {
                if (g % PSTAGES != pg) continue;
                if (!pwait(&empty[pg], (use & 1) ^ 1, &abort_flag)) {
                    ok = false;
                    break;
                }
                use++;
                const int kc = c * BK;
                // A chunk: thread = tile row, its 32 K values (coalesced across the warp per K)
                {
                    float va[BK];
                    const bool rv = ptid < J.m_rows;
#pragma unroll
                    for (int kk = 0; kk < BK; kk++)
                        va[kk] = (rv && kc + kk < J.K) ? J.Lp[ptid + (int64_t)(kc + kk) * J.ldl] : 0.f;
#pragma unroll
                    for (int j = 0; j < BK / 4; j++) {
                        const uint32_t off = sw128_off(ptid, 4 * j);
                        const float h0 = tf32_hi(va[4 * j]), h1 = tf32_hi(va[4 * j + 1]);
                        const float h2 = tf32_hi(va[4 * j + 2]), h3 = tf32_hi(va[4 * j + 3]);
                        st_shared_v4(a_hi + off, h0, h1, h2, h3);
                        if (PASSES > 1)
                            st_shared_v4(a_lo + off, va[4 * j] - h0, va[4 * j + 1] - h1, va[4 * j + 2] - h2,
                                         va[4 * j + 3] - h3);
                    }
                }
                // B chunk: warp pw covers tile columns 32pw..32pw+31, lane = K index
                {
                    float vb[32];
                    const bool kv = kc + lane < J.K;
#pragma unroll
                    for (int cc = 0; cc < 32; cc++) {
                        const int col = 32 * pw + cc;
                        vb[cc] = (kv && col < J.n_cols) ? J.Up[(kc + lane) + (int64_t)col * J.ldu] : 0.f;
                    }
#pragma unroll
                    for (int cc = 0; cc < 32; cc++) {
                        const uint32_t off = sw128_off(32 * pw + cc, lane);
                        const float h = tf32_hi(vb[cc]);
                        st_shared_f32(b_hi + off, h);
                        if (PASSES > 1) st_shared_f32(b_lo + off, vb[cc] - h);
                    }
                }
                fence_async_smem();  // generic-proxy stores visible to the tensor core
                mbar_arrive(&full[pg]);
            }
        }
    } else if (wid == P_MMA_WARP) {
        // ---- MMA issuer ------------------------------------------------------
        if (lane == 0) {
            int g = 0, li = 0;
            int uses[PSTAGES] = {};
            bool ok = true;
            for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x, li++) {
                const TileJob J = job_of(t);
                const int nch = (J.K + BK - 1) / BK;
                const int acc = li & 1;
                if (!pwait(&tempty[acc], ((li >> 1) & 1) ^ 1, &abort_flag)) break;
                fence_after_sync();
                const uint32_t d = tmem + (uint32_t)(acc * BN);
                for (int c = 0; c < nch; c++, g++) {
                    const int s = g % PSTAGES;
                    if (!pwait(&full[s], uses[s] & 1, &abort_flag)) {
                        ok = false;
                        break;
                    }
                    uses[s]++;
                    fence_after_sync();
                    const uint32_t a_hi = base + s * STAGE_BYTES, a_lo = a_hi + CHUNK_BYTES;
                    const uint32_t b_hi = a_hi + 2 * CHUNK_BYTES, b_lo = a_hi + 3 * CHUNK_BYTES;
#pragma unroll
                    for (int ks = 0; ks < BK / 8; ks++) {
                        const uint64_t ah = sw128_desc(a_hi + ks * 32), bh = sw128_desc(b_hi + ks * 32);
                        mma_tf32(d, ah, bh, idesc, (c > 0 || ks > 0) ? 1u : 0u);
                        if (PASSES > 1) {
                            const uint64_t al = sw128_desc(a_lo + ks * 32), bl = sw128_desc(b_lo + ks * 32);
                            mma_tf32(d, ah, bl, idesc, 1u);
                            mma_tf32(d, al, bh, idesc, 1u);
                        }
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) mma_commit(&tfull[acc]);
            }
            // every MMA issued by this thread done before the CTA tears down
            mma_commit(&drain);
            if (!mbar_wait(&drain, 0)) abort_flag = 1;
        }
    } else {
        // ---- epilogue: thread = tile row (warp w owns tensor-memory lanes 32(w%4)..) ----
        const int quarter = wid & 3;
        const int row = 32 * quarter + lane;
        int li = 0;
        for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, li++) {
            const TileJob J = job_of(t);
            const int acc = li & 1;
            const bool rv = row < J.m_rows;
            float* crow = J.Cp + row;
            // this thread's row of C into shared memory while the MMAs run (each
            // thread reads back only what it copied: no barrier needed)
            if (rv)
                for (int col = 0; col < J.n_cols; col++)
                    cp_async4(cbuf + (uint32_t)((col * BM + row) * 4), crow + (int64_t)col * J.ldc);
            cp_async_wait_all();
            if (!pwait(&tfull[acc], (li >> 1) & 1, &abort_flag)) break;
            fence_after_sync();
#pragma unroll 1
            for (int q = 0; q < BN / 32; q++) {
                const int cb = 32 * q;
                float v[32];
                tmem_ld32(tmem + (uint32_t)(acc * BN) + ((uint32_t)(32 * quarter) << 16) + (uint32_t)cb, v);
                if (rv) {
#pragma unroll
                    for (int j = 0; j < 32; j++)
                        if (cb + j < J.n_cols)
                            crow[(int64_t)(cb + j) * J.ldc] =
                                ld_shared_f32(cbuf + (uint32_t)(((cb + j) * BM + row) * 4)) - v[j];
                }
            }
            fence_before_sync();
            mbar_arrive(&tempty[acc]);
        }
    }
    fence_before_sync();
    __syncthreads();
    if (tid == 0 && abort_flag) atomicExch(err, 1);
    if (wid == 0) tmem_dealloc(tmem, P_TMEM_COLS);
}

}  // namespace tc
}  // namespace gbvlm
