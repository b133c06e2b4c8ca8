// Variable-size batched LU: shared declarations (see gbvlm_lu.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace gbvlm {

constexpr int LU_NB = 32;  // panel width

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
};

struct LuStep {
    int64_t k = 0;
    int64_t act_off = 0;
    int32_t n_panel = 0;
    int32_t n_tall_by_elem[2] = {0, 0};  // active systems whose panel exceeds shared memory (float, double)
    int64_t smem_rows[2] = {0, 0};       // tallest panel of the rest (float, double)
    int64_t n_tall_rows[2] = {0, 0};     // tallest panel of the tall ones
    int64_t swap_pfx = 0, swap_total = 0;
    int64_t trsm_pfx = 0, trsm_blocks = 0;
    int32_t n_upd = 0;
    int64_t upd_act_skip = 0;
    int64_t upd_pfx = 0, upd_blocks = 0;
};

struct LuPlan {
    std::vector<LuStep> steps;
    int32_t nsys = 0;
    int64_t maxn = 0;
    int cluster = 0;  // CTAs per cluster for tall panels (0: one-CTA global-memory panel)
    int32_t* d_act = nullptr;
    int64_t* d_pfx = nullptr;
    void release();
    ~LuPlan() { release(); }
    LuPlan() = default;
    LuPlan(const LuPlan&) = delete;
    LuPlan& operator=(const LuPlan&) = delete;
};

int lu_plan_build(LuPlan& plan, const std::vector<int64_t>& n_sorted, cudaStream_t st);
template <class T>
int lu_batch_factor(const LuBatch<T>& B, const LuPlan& plan, cudaStream_t st);
template <class T>
int lu_batch_solve(const LuBatch<T>& B, int32_t nsys, int32_t max_nrhs, int64_t maxn, cudaStream_t st);

// Single-system tables packed in a small device buffer (*work, grown on demand).
template <class T>
int make_single_batch(LuBatch<T>& B, int64_t n, int64_t ld, T* A, int32_t* ipiv, int32_t* perm, int32_t* info, T* X,
                      int64_t ldx, int32_t nrhs, void** work, size_t* work_bytes, cudaStream_t st);

}  // namespace gbvlm
