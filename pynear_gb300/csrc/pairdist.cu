// pairdist.cu — the distance between two vectors: the reference's module-level
// dist_l2 / dist_l1 / dist_chebyshev / dist_hamming (pynear/src/
// PythonBindings.cpp, over DistanceFunctions.hpp), computed on the GPU in the
// exact arithmetic of the flat scans.  Callers use it one pair at a time (the
// reference's own tests build their brute-force answers from millions of such
// calls), so a call costs one small kernel and nothing else: the operands are
// written to mapped pinned host memory that the kernel reads directly, and the
// result comes back the same way; the buffers and the stream are kept per
// device and only grow.
#include <cstring>
#include <mutex>

#include "distance.cuh"
#include "index.cuh"

namespace gn {

template <int M>
__global__ void pair_fdist_kernel(const float *__restrict__ a, const float *__restrict__ b, int d,
                                  double *__restrict__ out) {
    if (threadIdx.x == 0) *out = (double)fdist<M>(a, b, d);
}

__global__ void pair_hdist_kernel(const uint4 *__restrict__ a, const uint4 *__restrict__ b, int w4,
                                  double *__restrict__ out) {
    if (threadIdx.x == 0) *out = (double)hdist(a, b, w4);
}

struct PairCtx {
    cudaStream_t st = nullptr;
    uint8_t *h = nullptr;   // mapped pinned host memory: [a | b | result]
    uint8_t *dp = nullptr;  // its device address
    size_t cap = 0;
};

static std::mutex g_pair_mu;
static PairCtx g_pair[64];

}  // namespace gn

using namespace gn;

extern "C" int gn_dist(int32_t metric, const void *a, const void *b, int64_t d, double *out) {
    if (!out) return fail(GN_ERR_INVALID, "dist: NULL output");
    if (d < 0 || d > ((int64_t)1 << 28)) return fail(GN_ERR_INVALID, "dist: bad vector length");
    if (d > 0 && (!a || !b)) return fail(GN_ERR_INVALID, "dist: NULL vector");
    if (metric != GN_METRIC_L2 && metric != GN_METRIC_L1 && metric != GN_METRIC_LINF && metric != GN_METRIC_HAMMING)
        return fail(GN_ERR_INVALID, "dist: unknown metric");
    const bool ham = metric == GN_METRIC_HAMMING;
    // padded row bytes: floats to a multiple of 4 (16 bytes), bytes to a multiple of 16
    const size_t raw = (size_t)d * (ham ? 1 : 4);
    const size_t row = (raw + 15) & ~(size_t)15;
    int dev = 0;
    GN_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(GN_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(g_pair_mu);
    PairCtx &c = g_pair[dev];
    if (!c.st) GN_CUDA_TRY(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
    const size_t need = 2 * row + 16;
    if (c.cap < need) {
        if (c.h) cudaFreeHost(c.h);
        c.h = nullptr;
        c.cap = 0;
        const size_t cap = std::max<size_t>(need, 4096);
        void *p = nullptr;
        GN_CUDA_TRY(cudaHostAlloc(&p, cap, cudaHostAllocMapped | cudaHostAllocPortable));
        void *dptr = nullptr;
        GN_CUDA_TRY(cudaHostGetDevicePointer(&dptr, p, 0));
        c.h = reinterpret_cast<uint8_t *>(p);
        c.dp = reinterpret_cast<uint8_t *>(dptr);
        c.cap = cap;
    }
    std::memset(c.h, 0, 2 * row);
    if (raw) {
        std::memcpy(c.h, a, raw);
        std::memcpy(c.h + row, b, raw);
    }
    double *res_d = reinterpret_cast<double *>(c.dp + 2 * row);
    const float *fa = reinterpret_cast<const float *>(c.dp), *fb = reinterpret_cast<const float *>(c.dp + row);
    switch (metric) {
    case GN_METRIC_L2: pair_fdist_kernel<M_L2><<<1, 32, 0, c.st>>>(fa, fb, (int)d, res_d); break;
    case GN_METRIC_L1: pair_fdist_kernel<M_L1><<<1, 32, 0, c.st>>>(fa, fb, (int)d, res_d); break;
    case GN_METRIC_LINF: pair_fdist_kernel<M_LINF><<<1, 32, 0, c.st>>>(fa, fb, (int)d, res_d); break;
    default:
        pair_hdist_kernel<<<1, 32, 0, c.st>>>(reinterpret_cast<const uint4 *>(c.dp),
                                              reinterpret_cast<const uint4 *>(c.dp + row), (int)(row / 16), res_d);
        break;
    }
    GN_CUDA_TRY(cudaGetLastError());
    GN_CUDA_TRY(cudaStreamSynchronize(c.st));
    *out = *reinterpret_cast<volatile double *>(c.h + 2 * row);
    return GN_OK;
}
