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
// End of a blocking search on stream st: the device error word d_err (may be
// null) is copied into the index's pinned status word behind the results'
// copies, the stream is synchronised once, and a pipeline wait that ran out
// is reported as GN_ERR_TIMEOUT with message `what` (the word is cleared).
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
