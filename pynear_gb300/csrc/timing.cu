// timing.cu — event bracket used by gn_timing_enable / gn_timing_last.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "timing.cuh"

namespace gn {

static std::atomic<bool> g_on{false};
static std::mutex g_mu;
static cudaEvent_t g_ev[2] = {nullptr, nullptr};
static std::string g_name;
static bool g_have = false;

bool timing_on() { return g_on.load(std::memory_order_relaxed); }

void timing_begin(cudaStream_t st, const char *kernel_name) {
    if (!timing_on()) return;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ev[0]) {
        cudaEventCreate(&g_ev[0]);
        cudaEventCreate(&g_ev[1]);
    }
    g_name = kernel_name;
    cudaEventRecord(g_ev[0], st);
}

void timing_end(cudaStream_t st) {
    if (!timing_on()) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEventRecord(g_ev[1], st);
    g_have = true;
}

}  // namespace gn

using namespace gn;

extern "C" int gn_timing_enable(int on) {
    g_on.store(on != 0);
    return GN_OK;
}

extern "C" int gn_timing_last(float *ms, char *name, int name_len) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_have) return fail(GN_ERR_INVALID, "no timed kernel recorded");
    GN_CUDA_TRY(cudaEventSynchronize(g_ev[1]));
    float t = 0.f;
    GN_CUDA_TRY(cudaEventElapsedTime(&t, g_ev[0], g_ev[1]));
    if (ms) *ms = t;
    if (name && name_len > 0) {
        std::strncpy(name, g_name.c_str(), (size_t)name_len - 1);
        name[name_len - 1] = 0;
    }
    return GN_OK;
}
