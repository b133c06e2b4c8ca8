// Variable-size batched LU: shared declarations (see gbvlm_lu.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace gbvlm {

constexpr int LU_NB = 32;      // panel width
constexpr int LU_OUTER = 128;  // outer block width with tensor-core updates

// Device tables, one entry per system (systems sorted by n descending).
template <class T>
struct LuBatch {
    const int64_t* n;
    const int64_t* ld;
    T* const* A;
    int32_t* const* ipiv;
    int32_t* info;
    T* const* X;
    const int64_t* ldx;
    const int32_t* nrhs;
    int32_t* const* perm;  // row permutation of the factorisation (perm[r] = original row), n per system
    // float two-level factorisation: the row moves of the last 32-column panel,
    // 64 entries per system at sid * 64: [t] = offset below k of the row that
    // ends at position k + t, [32 + r] = final offset of the row that started
    // at k + r (null: not recorded)
    int32_t* mv = nullptr;
};

// One panel launch: active systems [first, first + count) of a step, each
// factored by a cluster of `csize` CTAs of `nt` threads owning `slab` rows
// apiece, one row per thread in registers (csize 0: the global-memory
// fallback).
struct PanelGroup {
    int32_t first = 0, count = 0;
    int32_t csize = 1, slab = 0, nt = 0;
    // one-CTA panels with several systems per CTA: ctas CTAs, entries
    // (first system of the CTA relative to `first`, systems in it) at
    // LuPlan::d_pack + 2 * pack_off; ctas = 0: one system per CTA
    int32_t ctas = 0;
    int64_t pack_off = 0;
};

struct LuStep {
    int64_t k = 0;
    int64_t act_off = 0;
    int32_t n_panel = 0;
    std::vector<PanelGroup> panels[2];  // panel launches (float, double)
    int64_t swap_pfx = 0, swap_total = 0;
    int64_t trsm_pfx = 0, trsm_blocks = 0;
    int32_t n_upd = 0;
    int64_t upd_act_skip = 0;
    int64_t upd_pfx = 0, upd_blocks = 0;  // whole trailing update (one-level blocking)
    // two-level blocking: outer block [kend - LuPlan::W, kend)
    int64_t kend = 0;
    int32_t n_in = 0;                         // systems with an inner update (a prefix)
    int64_t in_pfx = 0, in_blocks = 0;        // inner update of the outer panel, 64 x 64 tiles
    int64_t ik_pfx = 0, ik_blocks = 0;        // k_inner: row moves and U rows, 16-column chunks of the outer panel
    int32_t bswap_first = 0;                  // systems [bswap_first, n_panel) end the outer block here
    int64_t bswap_pfx = 0, bswap_total = 0;   // the block's swaps on the columns outside it: CTAs per system
    int32_t n_tc = 0;                         // systems with n > kend at the block's last step (a prefix)
    int64_t btrsm_pfx = 0, btrsm_blocks = 0;  // U12 = L11^-1 A12, 32 columns per CTA
    int64_t tc_pfx = 0, tc_blocks = 0;        // outer update, 128 x 128 tensor-core tiles
    int64_t tcn_pfx = 0, tcn_blocks = 0;      // its first column of tiles (the next outer panel)
    int64_t tcr_pfx = 0, tcr_blocks = 0;      // its other columns of tiles (lookahead)
    int64_t tcs_pfx = 0, tcs_blocks = 0;      // U12 on the tensor cores: tiles of 128 rows x the update's tile width
    int64_t inc_pfx = 0, inc_blocks = 0;      // the inner update on the tensor cores: 128-row tiles
};

struct LuPlan {
    std::vector<LuStep> steps;
    int32_t nsys = 0;
    int32_t base = 0;  // the plan's systems are [base, base + nsys) of the batch tables
    int64_t maxn = 0;
    int cluster = 1;  // largest cluster the register panel can be launched with
    int tc_passes = 0;  // float trailing update: 0 CUDA cores, 1 TF32, 3 3xTF32 tensor cores
    bool tc_wide = false;  // the update right of the next outer panel in 128 x 256 tiles (GBVLM_TC_WIDE=0: 128 x 128)
    cudaStream_t mem = nullptr;  // device memory stream-ordered on this stream (dev_alloc), or cudaMalloc
    // U12 = L11^-1 A12 as an explicit inverse (one triangular solve on the
    // identity per system and outer block) and a tensor-core tile product,
    // instead of the triangular solve per 64 columns (GBVLM_TC_TRSM=0)
    bool tc_inner = false;  // inner updates in 128-row tensor-core tiles, K = 32 (GBVLM_TC_INNER=0: CUDA cores)
    bool tc_trsm = false;
    int32_t tc_trsm_min = 1;  // ... for steps with at least this many systems
    float* d_minv = nullptr;  // nsys x 128 x 128: I - L11^-1 of each system's current outer block
    int W = LU_NB;      // outer block width of the float factorisation
    int32_t* d_act = nullptr;
    int32_t* d_pack = nullptr;  // PanelGroup pack entries
    int64_t* d_pfx = nullptr;
    int* d_err = nullptr;  // set by a tensor-core tile whose bounded wait ran out
    // algorithmic work of the outer (tensor-core) updates of one factorisation:
    // 2 m^2 W flops and 8 m^2 + 8 m W bytes (C read and written, L21 and U12
    // read once) per system and outer block, m = n - kend
    double tc_flops = 0, tc_bytes = 0;
    int64_t tc_launches = 0;
    // when set, lu_batch_factor records an event before and after every
    // tensor-core update launch (profiling; not used inside graphs)
    std::vector<cudaEvent_t>* tc_events = nullptr;
    // lookahead: the part of an outer update right of the next outer panel
    // runs on la_stream while the next block's inner steps run
    cudaStream_t la_stream = nullptr;
    cudaEvent_t la_fork = nullptr, la_join = nullptr;
    void release();
    ~LuPlan() { release(); }
    LuPlan() = default;
    LuPlan(const LuPlan&) = delete;
    LuPlan& operator=(const LuPlan&) = delete;
};

// n_sorted: sizes of systems [base, base + n_sorted.size()) of the batch, descending
int lu_plan_build(LuPlan& plan, const std::vector<int64_t>& n_sorted, cudaStream_t st, int32_t base = 0);
// GBVLM_OK, or an error if a tensor-core update gave up waiting (synchronises st)
int lu_plan_check(const LuPlan& plan, cudaStream_t st);
// number of kernel launches lu_batch_factor makes for element size es (4 or 8)
int64_t lu_plan_launches(const LuPlan& plan, int es);
// lookahead: overlap each outer update's right part with the next block's
// inner steps (float, tensor-core plans; ignored while timing launches)
template <class T>
int lu_batch_factor(const LuBatch<T>& B, const LuPlan& plan, cudaStream_t st, bool lookahead);
// err: the tensor-core error word of a plan with tensor cores (a single large
// float system then solves in 128-row blocks on the tensor cores), or null
template <class T>
int lu_batch_solve(const LuBatch<T>& B, int32_t nsys, int32_t max_nrhs, int64_t maxn, cudaStream_t st, int* err);

// Dataflow triangular solves of a float batch (k_trs_flow): one persistent
// launch per 8 right-hand sides runs the forward and backward sweeps of every
// system in 128-row blocks, items handed out in dependency order.
struct TrsFlow {
    int32_t nsys = 0, nfwd = 0, nitems = 0, grid = 0;
    int32_t groups = 1;        // blocks of FL_R right-hand sides solved by one launch
    int2* d_items = nullptr;   // (system, block) in dispatch order
    int32_t* d_ctl = nullptr;  // counter, error word, per-system forward and backward progress
    float* d_y = nullptr;      // per system n x 8 row-major
    float** d_yp = nullptr;    // per-system pointers into d_y
    cudaStream_t mem = nullptr;  // device memory stream-ordered on this stream (dev_alloc), or cudaMalloc
    void release();
    ~TrsFlow() { release(); }
    TrsFlow() = default;
    TrsFlow(const TrsFlow&) = delete;
    TrsFlow& operator=(const TrsFlow&) = delete;
};
// n_sorted: sizes of all systems of the batch, in batch order; groups: how
// many blocks of 8 right-hand sides one launch solves side by side
int trs_flow_build(TrsFlow& f, const std::vector<int64_t>& n_sorted, cudaStream_t st, int32_t groups = 1);
// whether one dataflow solve can take nsys systems with `groups` groups of
// 8 right-hand sides (item words hold the system in 20 bits)
inline bool trs_flow_fits(int64_t nsys, int64_t groups) { return nsys <= (1 << 20) && groups <= 1024; }
int trs_flow_solve(const LuBatch<float>& B, const TrsFlow& f, int32_t max_nrhs, cudaStream_t st);
int64_t trs_flow_launches(int32_t max_nrhs, int32_t groups = 1);
// GBVLM_OK, or an error if a wait of the last solve ran out (synchronises st)
int trs_flow_check(const TrsFlow& f, cudaStream_t st);

// Single-system tables packed in a small device buffer (*work, grown on demand).
template <class T>
int make_single_batch(LuBatch<T>& B, int64_t n, int64_t ld, T* A, int32_t* ipiv, int32_t* perm, int32_t* info, T* X,
                      int64_t ldx, int32_t nrhs, void** work, size_t* work_bytes, cudaStream_t st);

}  // namespace gbvlm
