// noalloc.cu — exact Hamming k-NN that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at search time — a serving
// process whose device memory is already reserved by another allocator (for
// example a framework's caching allocator that owns the whole HBM pool), or a
// latency-critical loop that cannot afford cudaMalloc's device-wide
// synchronisation.  They pass their own device buffers for the database, the
// queries and the results; the only other memory the scan needs (its per-slice
// partial top-k lists) lives in the fixed array below, which every GPU that
// loads this library holds until the process exits.
#include <mutex>

#include "flat_scan.cuh"
#include "index.cuh"

namespace gn {

// Scratch of the allocation-free scan: 2 Mi keys (16 MB) per device.
constexpr size_t NOALLOC_SCRATCH_KEYS = (size_t)2 << 20;
static __device__ __align__(256) uint64_t g_noalloc_scratch[NOALLOC_SCRATCH_KEYS];

// Device address of g_noalloc_scratch on the current device.  The host-side
// name is only a stand-in, so the address is looked up once per device (with
// that device current) and cached.
static int noalloc_scratch(uint64_t **out) {
    static std::mutex mu;
    static uint64_t *addr[64] = {nullptr};
    int dev = 0;
    GN_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(GN_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(GN_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        }
        addr[dev] = reinterpret_cast<uint64_t *>(p);
    }
    *out = addr[dev];
    return GN_OK;
}

}  // namespace gn

using namespace gn;

extern "C" int gn_hamming_knn_noalloc(const uint8_t *d_db, int64_t n, int64_t nbytes, const uint8_t *d_queries,
                                      int64_t nq, int64_t k, int64_t *d_idx, int64_t *d_dist, void *stream) {
    if (!d_db || !d_queries || !d_idx || !d_dist) return fail(GN_ERR_INVALID, "hamming_knn_noalloc: NULL pointer");
    if (n <= 0 || n >= 0x7fffffffLL) return fail(GN_ERR_INVALID, "hamming_knn_noalloc: n must be in [1, 2^31-2]");
    if (nbytes <= 0 || nbytes % 16 != 0)
        return fail(GN_ERR_INVALID, "hamming_knn_noalloc: row width must be a positive multiple of 16 bytes");
    if (nq < 0) return fail(GN_ERR_INVALID, "hamming_knn_noalloc: negative query count");
    if (k <= 0 || k > FLAT_MAX_K_WARP) return fail(GN_ERR_INVALID, "hamming_knn_noalloc: k must be in [1, 256]");
    if ((uint64_t)nq * (uint64_t)k > NOALLOC_SCRATCH_KEYS)
        return fail(GN_ERR_INVALID, "hamming_knn_noalloc: nq * k = " + std::to_string(nq * k) +
                                        " exceeds the fixed scratch of " + std::to_string(NOALLOC_SCRATCH_KEYS) +
                                        " keys; split the queries into smaller calls");
    uint64_t *scratch = nullptr;
    GN_TRY(noalloc_scratch(&scratch));
    if (nq == 0) return GN_OK;
    FlatScanArgs a;
    a.metric = M_HAMMING;
    a.db = d_db;
    a.n = n;
    a.d = (int)nbytes;
    a.stride4 = (int)(nbytes / 16);
    a.q = d_queries;
    a.nq = nq;
    a.k = (int)k;
    a.out_idx = d_idx;
    a.out_dist = d_dist;
    flat_plan(a);
    // fewer database slices when the partial lists would overflow the scratch
    const int64_t max_slices = (int64_t)(NOALLOC_SCRATCH_KEYS / ((uint64_t)nq * (uint64_t)k));
    if (a.n_slices > max_slices) {
        a.slice_rows = round_up(ceil_div(n, max_slices), 32);
        a.n_slices = (int)ceil_div(n, a.slice_rows);
    }
    if (!flat_smem_ok(a)) return fail(GN_ERR_UNSUPPORTED, "hamming_knn_noalloc: rows too wide for the scan");
    flat_launch(a, scratch, (cudaStream_t)stream);
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}
