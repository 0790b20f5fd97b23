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
//
// Set-up: the library's kernels and this array live in modules that the CUDA
// driver loads lazily (the default since CUDA 12.2), so the FIRST call on a
// device loads them, and that load is when the CUDA driver reserves the array's
// 16 MB and the kernels' code.  A caller that must not allocate later makes
// one call at set-up time (nq = 0 is enough: it loads everything and scans
// nothing), with that device current and before any stream capture.  After
// that, calls allocate nothing.
#include <mutex>

#include "flat_scan.cuh"
#include "index.cuh"

namespace gn {

// Scratch of the allocation-free scan: 2 Mi keys (16 MB) per device.
constexpr size_t NOALLOC_SCRATCH_KEYS = (size_t)2 << 20;
static __device__ __align__(256) uint64_t g_noalloc_scratch[NOALLOC_SCRATCH_KEYS];

// Device address of g_noalloc_scratch on the current device.  The host-side
// name is only a stand-in, so the address is looked up on every call, with
// the caller's device current (cheap once the module is loaded; nothing is
// cached, so a cudaDeviceReset between calls leaves no stale pointer).  The
// same call loads the scan kernels (see the set-up note above).
static int noalloc_setup(uint64_t **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(GN_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    }
    GN_TRY(flat_preload_hamming());
    *out = reinterpret_cast<uint64_t *>(p);
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
    // rows are read as 16-byte vectors: both bases must be 16-byte aligned
    if (((uintptr_t)d_db | (uintptr_t)d_queries) & 15)
        return fail(GN_ERR_INVALID, "hamming_knn_noalloc: d_db and d_queries must be 16-byte aligned");
    if (nq < 0) return fail(GN_ERR_INVALID, "hamming_knn_noalloc: negative query count");
    if (k <= 0 || k > FLAT_MAX_K_WARP) return fail(GN_ERR_INVALID, "hamming_knn_noalloc: k must be in [1, 256]");
    // nq * k <= the scratch, tested without forming the (possibly wrapping) product
    if ((uint64_t)nq > NOALLOC_SCRATCH_KEYS / (uint64_t)k)
        return fail(GN_ERR_INVALID, "hamming_knn_noalloc: nq * k (nq = " + std::to_string(nq) +
                                        ", k = " + std::to_string(k) + ") exceeds the fixed scratch of " +
                                        std::to_string(NOALLOC_SCRATCH_KEYS) +
                                        " keys; split the queries into smaller calls");
    uint64_t *scratch = nullptr;
    GN_TRY(noalloc_setup(&scratch));
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
    // (nq * k >= 1 and <= the scratch here, so max_slices >= 1)
    const int64_t max_slices = (int64_t)(NOALLOC_SCRATCH_KEYS / ((uint64_t)nq * (uint64_t)k));
    if (a.n_slices > max_slices) {
        a.slice_rows = round_up(ceil_div(n, max_slices), 32);
        a.n_slices = (int)ceil_div(n, a.slice_rows);
    }
    if (!flat_smem_ok(a)) return fail(GN_ERR_UNSUPPORTED, "hamming_knn_noalloc: rows too wide for the scan");
    GN_TRY(flat_launch(a, scratch, (cudaStream_t)stream));
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}
