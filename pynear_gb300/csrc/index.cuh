// index.cuh — host-side index object shared by the C ABI translation units.
#pragma once

#include <mutex>
#include <vector>

#include "common.cuh"

namespace gn {

// Growable device allocation owned by an index (freed in the destructor), or
// a view of another index's allocation (a fork's shared list data: never
// freed or grown through the view).
struct DBuf {
    void *p = nullptr;
    size_t cap = 0;
    bool own = true;
    int ensure(size_t bytes);
    void release();
    void view(const DBuf &o) {
        release();
        p = o.p;
        cap = o.cap;
        own = false;
    }
    template <typename T>
    T *as() const { return reinterpret_cast<T *>(p); }
    ~DBuf() { release(); }
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
};

// Pinned host staging buffer.
struct HBuf {
    void *p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
    ~HBuf() { release(); }
    HBuf() = default;
    HBuf(const HBuf &) = delete;
    HBuf &operator=(const HBuf &) = delete;
};

enum IndexKind { K_FLAT = 1, K_IVFL2 = 2, K_IVFBIN = 3, K_TCFLAT = 4, K_PROBER = 5, K_MIH = 6 };

struct IvfL2State;
struct IvfBinState;

}  // namespace gn

struct gn_index {
    int kind = 0;
    int metric = 0;
    int64_t n = 0;        // rows
    int64_t dim = 0;      // floats (float metrics) or bytes (binary)
    int stride4 = 0;      // row stride in 16-byte units
    gn::DBuf data;        // n * stride4 * 16 bytes, zero padded
    cudaStream_t stream = nullptr;
    std::mutex mu;
    // per-call scratch (reused across calls)
    gn::DBuf q, part, out_idx, out_dist, keys, sorted;
    gn::DBuf err;         // float flat scans: error word of their bounded pipeline waits
    gn::HBuf hstatus;     // pinned: a blocking search's error word, copied behind its results
    // pinned staging of a blocking search's small pageable copies (queries in,
    // results out); staged results reach the caller's buffers after the sync
    gn::HBuf stage_in, stage_out;
    struct Pending {
        void *dst;
        size_t off, bytes;
    };
    std::vector<Pending> pending;
    size_t pending_bytes = 0;
    bool stage_in_busy = false;  // a copy from stage_in may still be queued
    // kind-specific state
    gn::IvfL2State *ivfl2 = nullptr;
    gn::IvfBinState *ivfbin = nullptr;
    void *ext = nullptr;                  // other engines' state
    void (*ext_free)(void *) = nullptr;
    // forks (concurrent search contexts over one index's lists): a fork points
    // at its parent; a parent counts its live forks and, when destroyed while
    // some are alive, is deleted with the last of them (guarded by a global
    // mutex in api.cu)
    gn_index *fork_parent = nullptr;
    int fork_count = 0;
    bool destroy_pending = false;
    ~gn_index();
};

namespace gn {

int make_stream(gn_index *ix);
// Blocking searches (the host-buffer entry points), in this order:
// begin_blocking, then upload_queries / download_result for the caller's
// buffers, then finish_blocking.  Pageable buffers of up to STAGE_BYTES go
// through the index's pinned stage_in / stage_out, so that each copy is one
// asynchronous DMA instead of the CUDA driver's staged pageable copy (about
// 19 us of a 76 us one-query call measured); pinned or larger buffers are
// copied directly.
constexpr size_t STAGE_BYTES = (size_t)1 << 20;
void begin_blocking(gn_index *ix);
// Host -> device copy of n query rows in upload_rows' layout.
int upload_queries(gn_index *ix, DBuf &dst, const void *src, int64_t n, int64_t row_bytes, int stride4,
                   cudaStream_t st);
// Host staging of query rows for a copy the caller issues: returns src, or
// the pinned stage_in holding a copy of its `bytes`.
int stage_queries(gn_index *ix, const void *src, size_t bytes, cudaStream_t st, const void **out);
// Device -> host copy of `bytes` of results into the caller's dst.
int download_result(gn_index *ix, void *dst, const void *dsrc, size_t bytes, cudaStream_t st);
// End of a blocking search on stream st: the device error word d_err (may be
// null) is copied into the index's pinned status word behind the results'
// copies, the stream is synchronised once, staged results are copied to the
// caller's buffers, and a pipeline wait that ran out is reported as
// GN_ERR_TIMEOUT with message `what` (the word is cleared).
int finish_blocking(gn_index *ix, int *d_err, cudaStream_t st, const char *what);
// Register a new fork of `parent` / ask whether an index has live forks
// (under the fork mutex).
void fork_attach(gn_index *child, gn_index *parent);
bool has_forks(gn_index *ix);
// Counter bumped whenever any DBuf (re)allocates: captured CUDA graphs that
// hold device pointers compare it to know whether they are still valid.
uint64_t dbuf_generation();
void ivf_free(gn_index *ix);
// Copy n rows of `dim` elements of `elem` bytes from host into a device buffer
// with row stride stride4*16 bytes, zero padding the tail of each row.
int upload_rows(DBuf &dst, const void *src, int64_t n, int64_t row_bytes, int stride4, cudaStream_t st,
                bool src_on_device = false);

}  // namespace gn
