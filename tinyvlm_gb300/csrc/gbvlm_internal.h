// Host-side helpers shared by the gbvlm translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/gbvlm.h"

namespace gbvlm {

void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define GB_CUDA(call)                                                              \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) return ::gbvlm::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

#define GB_LAUNCH_CHECK() GB_CUDA(cudaGetLastError())

#define GB_REQUIRE(cond, ...)                  \
    do {                                       \
        if (!(cond)) {                         \
            ::gbvlm::set_error(__VA_ARGS__);   \
            return GBVLM_ERR_ARG;              \
        }                                      \
    } while (0)

inline cudaStream_t to_cuda(gbvlm_stream s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Per-thread pinned staging buffer for synchronous scalar read-backs.
void* host_scratch(size_t bytes);
// Per-device small device buffer for reductions (grown on demand).
int device_scratch(size_t bytes, void** out, cudaStream_t s);

}  // namespace gbvlm
