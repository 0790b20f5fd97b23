// api.cu — C ABI: status plumbing, device buffers and the exact flat index.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>

#include "flat_scan.cuh"
#include "index.cuh"

namespace gn {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}

const DevInfo &dev_info() {
    static thread_local DevInfo cache[64];
    int dev = 0;
    cudaGetDevice(&dev);
    DevInfo &di = cache[dev & 63];
    if (di.device != dev) {
        cudaDeviceGetAttribute(&di.num_sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&di.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        di.device = dev;
    }
    return di;
}

static std::atomic<uint64_t> g_dbuf_gen{1};
uint64_t dbuf_generation() { return g_dbuf_gen.load(std::memory_order_relaxed); }

int DBuf::ensure(size_t bytes) {
    if (bytes <= cap && p) return GN_OK;
    if (!own) return fail(GN_ERR_INVALID, "a buffer shared with a parent index cannot be reallocated");
    g_dbuf_gen.fetch_add(1, std::memory_order_relaxed);  // device pointers held elsewhere may go stale
    release();
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        cap = 0;
        cudaGetLastError();
        return fail(GN_ERR_OOM, "device allocation of " + std::to_string(want) + " bytes failed: " + cudaGetErrorString(e));
    }
    cap = want;
    return GN_OK;
}
void DBuf::release() {
    if (p && own) cudaFree(p);
    p = nullptr;
    cap = 0;
    own = true;
}

static std::mutex g_fork_mu;

void fork_attach(gn_index *child, gn_index *parent) {
    std::lock_guard<std::mutex> g(g_fork_mu);
    child->fork_parent = parent;
    parent->fork_count++;
}

bool has_forks(gn_index *ix) {
    std::lock_guard<std::mutex> g(g_fork_mu);
    return ix->fork_count > 0;
}

int HBuf::ensure(size_t bytes) {
    if (bytes <= cap && p) return GN_OK;
    release();
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMallocHost(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        cap = 0;
        cudaGetLastError();
        return fail(GN_ERR_OOM, "pinned host allocation failed");
    }
    cap = want;
    return GN_OK;
}
void HBuf::release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
}

int make_stream(gn_index *ix) {
    if (ix->stream) return GN_OK;
    GN_CUDA_TRY(cudaStreamCreateWithFlags(&ix->stream, cudaStreamNonBlocking));
    return GN_OK;
}

// Page-locked host memory (allocated or registered with CUDA)?
static bool host_pinned(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

void begin_blocking(gn_index *ix) {
    ix->pending.clear();
    ix->pending_bytes = 0;
}

int stage_queries(gn_index *ix, const void *src, size_t bytes, cudaStream_t st, const void **out) {
    *out = src;
    if (bytes == 0 || bytes > STAGE_BYTES || host_pinned(src)) return GN_OK;
    GN_TRY(ix->stage_in.ensure(STAGE_BYTES));  // one fixed size: never reallocated under a queued copy
    // a search that ended early (an error) may have left a copy from it queued
    if (ix->stage_in_busy) GN_CUDA_TRY(cudaStreamSynchronize(st));
    std::memcpy(ix->stage_in.p, src, bytes);
    ix->stage_in_busy = true;
    *out = ix->stage_in.p;
    return GN_OK;
}

int upload_queries(gn_index *ix, DBuf &dst, const void *src, int64_t n, int64_t row_bytes, int stride4,
                   cudaStream_t st) {
    const void *s = src;
    if (n > 0) GN_TRY(stage_queries(ix, src, (size_t)n * (size_t)row_bytes, st, &s));
    return upload_rows(dst, s, n, row_bytes, stride4, st);
}

int download_result(gn_index *ix, void *dst, const void *dsrc, size_t bytes, cudaStream_t st) {
    if (bytes == 0) return GN_OK;
    const size_t off = ix->pending_bytes, span = (bytes + 255) & ~(size_t)255;
    if (off + span <= STAGE_BYTES && !host_pinned(dst)) {
        GN_TRY(ix->stage_out.ensure(STAGE_BYTES));
        GN_CUDA_TRY(cudaMemcpyAsync(static_cast<char *>(ix->stage_out.p) + off, dsrc, bytes, cudaMemcpyDeviceToHost,
                                    st));
        ix->pending.push_back({dst, off, bytes});
        ix->pending_bytes = off + span;
        return GN_OK;
    }
    GN_CUDA_TRY(cudaMemcpyAsync(dst, dsrc, bytes, cudaMemcpyDeviceToHost, st));
    return GN_OK;
}

int finish_blocking(gn_index *ix, int *d_err, cudaStream_t st, const char *what) {
    int *h = nullptr;
    if (d_err) {
        GN_TRY(ix->hstatus.ensure(sizeof(int)));
        h = static_cast<int *>(ix->hstatus.p);
        *h = 0;  // no copy into it is pending: every blocking search ends synchronised
        GN_CUDA_TRY(cudaMemcpyAsync(h, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    const cudaError_t se = cudaStreamSynchronize(st);
    if (ix->stage_in_busy) ix->stage_in_busy = false;
    if (!ix->pending.empty()) {  // (the entry points that stage hold the index's lock throughout)
        if (se == cudaSuccess)
            for (const auto &pd : ix->pending)
                std::memcpy(pd.dst, static_cast<const char *>(ix->stage_out.p) + pd.off, pd.bytes);
        begin_blocking(ix);
    }
    GN_CUDA_TRY(se);
    if (h && *h) {
        GN_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        return fail(GN_ERR_TIMEOUT, what);
    }
    return GN_OK;
}

int upload_rows(DBuf &dst, const void *src, int64_t n, int64_t row_bytes, int stride4, cudaStream_t st,
                bool src_on_device) {
    const size_t pitch = (size_t)stride4 * 16;
    GN_TRY(dst.ensure(std::max<size_t>(1, (size_t)n * pitch)));
    if (n == 0) return GN_OK;
    const cudaMemcpyKind kind = src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if ((size_t)row_bytes == pitch) {
        GN_CUDA_TRY(cudaMemcpyAsync(dst.p, src, (size_t)n * pitch, kind, st));
    } else {
        GN_CUDA_TRY(cudaMemsetAsync(dst.p, 0, (size_t)n * pitch, st));
        GN_CUDA_TRY(cudaMemcpy2DAsync(dst.p, pitch, src, (size_t)row_bytes, (size_t)row_bytes, (size_t)n, kind, st));
    }
    return GN_OK;
}

}  // namespace gn

gn_index::~gn_index() {
    gn::ivf_free(this);
    if (stream) cudaStreamSynchronize(stream);
    if (ext && ext_free) ext_free(ext);
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
}

using namespace gn;

extern "C" {

int gn_version(void) { return 100; }

const char *gn_last_error(void) { return g_last_error.c_str(); }

int gn_device_info(int *num_sms, int *cc_major, int *cc_minor) {
    int dev = 0, count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(GN_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    GN_CUDA_TRY(cudaGetDevice(&dev));
    if (num_sms) GN_CUDA_TRY(cudaDeviceGetAttribute(num_sms, cudaDevAttrMultiProcessorCount, dev));
    if (cc_major) GN_CUDA_TRY(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
    if (cc_minor) GN_CUDA_TRY(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    return GN_OK;
}

int gn_flat_create(int metric, gn_index **out) {
    if (!out) return fail(GN_ERR_INVALID, "gn_flat_create: out is NULL");
    if (metric < GN_METRIC_L2 || metric > GN_METRIC_HAMMING) return fail(GN_ERR_INVALID, "gn_flat_create: unknown metric");
    gn_index *ix = new gn_index();
    ix->kind = K_FLAT;
    ix->metric = metric;
    *out = ix;
    return GN_OK;
}

int gn_index_destroy(gn_index *ix) {
    if (!ix) return GN_OK;
    gn_index *parent_done = nullptr;
    {
        std::lock_guard<std::mutex> g(g_fork_mu);
        if (ix->fork_count > 0) {  // forks still read its lists: deleted with the last fork
            ix->destroy_pending = true;
            return GN_OK;
        }
        if (gn_index *p = ix->fork_parent)
            if (--p->fork_count == 0 && p->destroy_pending) parent_done = p;
    }
    delete ix;  // a fork's views of the parent's lists are not freed
    delete parent_done;
    return GN_OK;
}

int gn_index_size(gn_index *ix, int64_t *n, int64_t *dim) {
    if (!ix) return fail(GN_ERR_INVALID, "index is NULL");
    if (n) *n = ix->n;
    if (dim) *dim = ix->dim;
    return GN_OK;
}

static int row_stride4(int metric, int64_t dim) {
    const int64_t bytes = (metric == GN_METRIC_HAMMING) ? dim : dim * 4;
    return (int)ceil_div(bytes, 16);
}

int gn_flat_set(gn_index *ix, const void *data, int64_t n, int64_t dim) {
    if (!ix || ix->kind != K_FLAT) return fail(GN_ERR_INVALID, "gn_flat_set: not a flat index");
    if (n < 0 || dim < 0) return fail(GN_ERR_INVALID, "gn_flat_set: negative shape");
    if (n > 0 && dim <= 0) return fail(GN_ERR_INVALID, "gn_flat_set: dimension must be positive");
    if (n > 0 && !data) return fail(GN_ERR_INVALID, "gn_flat_set: data is NULL");
    if (n >= 0x7fffffffLL) return fail(GN_ERR_UNSUPPORTED, "gn_flat_set: at most 2^31-2 rows");
    std::lock_guard<std::mutex> lk(ix->mu);
    GN_TRY(make_stream(ix));
    ix->n = 0;
    ix->dim = 0;
    if (n == 0) return GN_OK;  // an empty index: searches raise GN_ERR_EMPTY
    const int s4 = row_stride4(ix->metric, dim);
    const int64_t row_bytes = (ix->metric == GN_METRIC_HAMMING) ? dim : dim * 4;
    GN_TRY(upload_rows(ix->data, data, n, row_bytes, s4, ix->stream));
    GN_CUDA_TRY(cudaStreamSynchronize(ix->stream));
    ix->n = n;
    ix->dim = dim;
    ix->stride4 = s4;
    return GN_OK;
}

// Shared search body.  queries/out are device pointers here.
static int flat_search_dev(gn_index *ix, const void *d_q, int64_t nq, int64_t k, int64_t *d_idx, void *d_dist,
                           cudaStream_t st) {
    FlatScanArgs a;
    a.metric = ix->metric;
    a.db = ix->data.p;
    a.n = ix->n;
    a.d = (int)ix->dim;
    a.stride4 = ix->stride4;
    a.q = d_q;
    a.nq = nq;
    a.k = (int)k;
    a.out_idx = d_idx;
    a.out_dist = d_dist;
    if (nq == 0) return GN_OK;
    if (k <= FLAT_MAX_K_WARP) {
        flat_plan(a);
        if (!flat_smem_ok(a)) return fail(GN_ERR_UNSUPPORTED, "dimension too large for the exact flat scan");
        GN_TRY(ix->part.ensure(flat_part_bytes(a)));
        if (a.metric != M_HAMMING) {
            if (!ix->err.p) {
                GN_TRY(ix->err.ensure(4));
                GN_CUDA_TRY(cudaMemsetAsync(ix->err.p, 0, 4, st));
            }
            a.err = ix->err.as<int>();
        }
        GN_TRY(flat_launch(a, ix->part.as<uint64_t>(), st));
    } else {
        // materialise keys for chunks of queries (<= 512 MB of keys per chunk)
        const int64_t p2 = next_pow2(k);
        int64_t qc = std::max<int64_t>(1, std::min<int64_t>(nq, (int64_t)(512ll << 20) / (8 * std::max<int64_t>(ix->n, 1))));
        GN_TRY(ix->keys.ensure((size_t)qc * ix->n * 8));
        GN_TRY(ix->sorted.ensure((size_t)qc * p2 * 8));
        for (int64_t q0 = 0; q0 < nq; q0 += qc)
            flat_large_k_launch(a, q0, std::min(qc, nq - q0), ix->keys.as<uint64_t>(), ix->sorted.as<uint64_t>(), st);
    }
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

static int flat_check(gn_index *ix, int64_t nq, int64_t k) {
    if (!ix || ix->kind != K_FLAT) return fail(GN_ERR_INVALID, "not a flat index");
    if (ix->n == 0)
        return fail(GN_ERR_EMPTY, "index must be first initialized with .set() function and non empty dataset");
    if (nq < 0) return fail(GN_ERR_INVALID, "negative query count");
    if (k <= 0) return fail(GN_ERR_INVALID, "k must be positive");
    if (k > 0x7fffffffLL) return fail(GN_ERR_INVALID, "k too large");
    return GN_OK;
}

int gn_flat_search_knn(gn_index *ix, const void *queries, int64_t nq, int64_t k, int64_t *out_idx, void *out_dist) {
    GN_TRY(flat_check(ix, nq, k));
    if (nq > 0 && (!queries || !out_idx || !out_dist)) return fail(GN_ERR_INVALID, "NULL pointer argument");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (nq == 0) return GN_OK;
    cudaStream_t st = ix->stream;
    begin_blocking(ix);
    const int64_t row_bytes = (ix->metric == GN_METRIC_HAMMING) ? ix->dim : ix->dim * 4;
    GN_TRY(upload_queries(ix, ix->q, queries, nq, row_bytes, ix->stride4, st));
    GN_TRY(ix->out_idx.ensure((size_t)nq * k * 8));
    GN_TRY(ix->out_dist.ensure((size_t)nq * k * 8));
    GN_TRY(flat_search_dev(ix, ix->q.p, nq, k, ix->out_idx.as<int64_t>(), ix->out_dist.p, st));
    const size_t dist_bytes = (size_t)nq * k * (ix->metric == GN_METRIC_HAMMING ? 8 : 4);
    GN_TRY(download_result(ix, out_idx, ix->out_idx.p, (size_t)nq * k * 8, st));
    GN_TRY(download_result(ix, out_dist, ix->out_dist.p, dist_bytes, st));
    // a float scan's pipeline wait that ran out (reported once, then cleared)
    return finish_blocking(ix, ix->err.p ? ix->err.as<int>() : nullptr, st,
                           "flat scan: a pipeline wait timed out; results are invalid");
}

int gn_flat_search_1nn(gn_index *ix, const void *queries, int64_t nq, int64_t *out_idx, void *out_dist) {
    return gn_flat_search_knn(ix, queries, nq, 1, out_idx, out_dist);
}

int gn_flat_search_knn_device(gn_index *ix, const void *d_queries, int64_t nq, int64_t k, int64_t *d_idx,
                              void *d_dist, void *stream) {
    GN_TRY(flat_check(ix, nq, k));
    std::lock_guard<std::mutex> lk(ix->mu);
    // device queries must already use the index's padded row layout
    return flat_search_dev(ix, d_queries, nq, k, d_idx, d_dist, (cudaStream_t)stream);
}

}  // extern "C"
