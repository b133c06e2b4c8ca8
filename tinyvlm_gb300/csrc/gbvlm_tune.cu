// Launch-shape parameters of the kernels, one process-wide table the
// autotuner (tinyvlm_gb300/autotune.py) fills per workload shape.  A batch
// plan copies the values it uses when it is created, so a plan keeps its
// shapes whatever is set afterwards; the per-operator calls read them at
// every launch.
#include <cuda_runtime.h>
#include <string.h>

#include <mutex>

#include "gbvlm_internal.h"

namespace gbvlm {

namespace {

struct Param {
    const char* name;
    int64_t TuneParams::*field;
    int64_t lo, hi;
};

// name, field, allowed range (inclusive); defaults in TuneParams
const Param kParams[] = {
    {"wake.waves", &TuneParams::wake_waves, 1, 16},
    {"hbvlm.waves", &TuneParams::hbvlm_waves, 1, 16},
    {"hbvlm.min_rows", &TuneParams::hbvlm_min_rows, 8, 512},
    {"batch.group_hi", &TuneParams::batch_group_hi, 64, 16384},
    {"batch.group_lo", &TuneParams::batch_group_lo, 16, 16384},
    {"batch.group_mid", &TuneParams::batch_group_mid, 0, 16384},
    {"batch.loads_threads", &TuneParams::batch_loads_threads, 0, 256},
    {"batch.assembly_span", &TuneParams::batch_assembly_span, 64, 256},
    {"batch.assembly_rows", &TuneParams::batch_assembly_rows, 1, 4},
};

std::mutex g_mu;
TuneParams g_params;

const Param* find(const char* name) {
    if (!name) return nullptr;
    for (const auto& p : kParams)
        if (strcmp(p.name, name) == 0) return &p;
    return nullptr;
}

}  // namespace

TuneParams tune() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_params;
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 152;
    }
    if (!cached[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
            cudaGetLastError();
            return 152;
        }
        cached[dev] = v;
    }
    return cached[dev];
}

}  // namespace gbvlm

using namespace gbvlm;

extern "C" {

int gbvlm_tune_set(const char* name, int64_t value) {
    const Param* p = find(name);
    GB_REQUIRE(p != nullptr, "unknown tuning parameter '%s'", name ? name : "(null)");
    GB_REQUIRE(value >= p->lo && value <= p->hi, "%s = %lld outside [%lld, %lld]", p->name, (long long)value,
               (long long)p->lo, (long long)p->hi);
    if (strcmp(p->name, "batch.loads_threads") == 0)
        GB_REQUIRE(value == 0 || value == 32 || value == 64 || value == 128 || value == 256,
                   "batch.loads_threads must be 0 (by size), 32, 64, 128 or 256");
    if (strcmp(p->name, "batch.assembly_span") == 0)
        GB_REQUIRE(value == 64 || value == 128 || value == 256, "batch.assembly_span must be 64, 128 or 256");
    std::lock_guard<std::mutex> lk(g_mu);
    g_params.*(p->field) = value;
    return GBVLM_OK;
}

int gbvlm_tune_get(const char* name, int64_t* value) {
    const Param* p = find(name);
    GB_REQUIRE(p != nullptr && value != nullptr, "unknown tuning parameter '%s'", name ? name : "(null)");
    std::lock_guard<std::mutex> lk(g_mu);
    *value = g_params.*(p->field);
    return GBVLM_OK;
}

int gbvlm_tune_reset(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_params = TuneParams();
    return GBVLM_OK;
}

int gbvlm_tune_count(int32_t* n) {
    GB_REQUIRE(n != nullptr, "null argument");
    *n = (int32_t)(sizeof(kParams) / sizeof(kParams[0]));
    return GBVLM_OK;
}

int gbvlm_tune_name(int32_t i, const char** name, int64_t* lo, int64_t* hi) {
    GB_REQUIRE(i >= 0 && i < (int32_t)(sizeof(kParams) / sizeof(kParams[0])) && name, "no tuning parameter %d", i);
    *name = kParams[i].name;
    if (lo) *lo = kParams[i].lo;
    if (hi) *hi = kParams[i].hi;
    return GBVLM_OK;
}

}  // extern "C"
