// common.cuh — shared definitions for the gpunear CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gpunear.h"

namespace gn {

// ── status / error plumbing (host) ─────────────────────────────────────────
void set_error(const std::string &msg);
int fail(int status, const std::string &msg);

#define GN_CUDA_TRY(expr)                                                                  \
    do {                                                                                   \
        cudaError_t _e = (expr);                                                           \
        if (_e != cudaSuccess)                                                             \
            return ::gn::fail(_e == cudaErrorMemoryAllocation ? GN_ERR_OOM : GN_ERR_CUDA, \
                              std::string(#expr) + ": " + cudaGetErrorString(_e));         \
    } while (0)

#define GN_TRY(expr)              \
    do {                          \
        int _s = (expr);          \
        if (_s != GN_OK) return _s; \
    } while (0)

// ── metric ids (match gn_metric in gpunear.h) ──────────────────────────────
enum Metric : int { M_L2 = GN_METRIC_L2, M_L1 = GN_METRIC_L1, M_LINF = GN_METRIC_LINF, M_HAMMING = GN_METRIC_HAMMING };

// ── sortable 64-bit keys: (distance bits << 32) | row index ───────────────
// Distances are non-negative floats (their IEEE bits order like unsigned ints)
// or non-negative integers, so comparing keys compares (distance, index)
// lexicographically: the lower index wins a distance tie.
static constexpr uint64_t KEY_EMPTY = ~0ull;

__host__ __device__ __forceinline__ uint64_t make_key(uint32_t dist_bits, uint32_t idx) {
    return ((uint64_t)dist_bits << 32) | (uint64_t)idx;
}
__host__ __device__ __forceinline__ uint32_t key_dist(uint64_t k) { return (uint32_t)(k >> 32); }
__host__ __device__ __forceinline__ uint32_t key_idx(uint64_t k) { return (uint32_t)(k & 0xffffffffu); }

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// Device properties of the current device, cached per device.
struct DevInfo {
    int device = -1;
    int num_sms = 0;
    int max_smem_optin = 0;
};
const DevInfo &dev_info();

}  // namespace gn
