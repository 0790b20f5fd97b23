// ivf.cuh — IVF index state and device search plumbing.
#pragma once

#include <vector>

#include "index.cuh"

namespace gn {

// Per-batch scratch of an IVF search (device resident, reused).
struct IvfScratch {
    DBuf q, qn, probes, probes64, pdist, bcnt, boff, bucket, fill, slot_rel, qcount, qslot, item_off, counter, part,
        cpart;
};

// Float IVF (forest.py IVFFlatL2Index semantics, squared L2).
struct IvfL2State {
    int32_t nlist_req = 100, nprobe = 10;
    int d = 0, dp = 0;           // dp = round_up(d, 16) floats per row
    int32_t nc = 0;              // non-empty lists, ordered by descending size
    int64_t n = 0;
    DBuf cent, cnorm;            // nc*dp, nc
    DBuf list_off;               // int64 nc+1
    DBuf vecs, vnorm, ids;       // n*dp (list order), n, n (int32 original row)
    std::vector<int64_t> h_off;  // host copy of list_off
    std::vector<int64_t> top_rows;  // top_rows[p] = rows in the p largest lists
    int rc = 1024;               // rows per scan work item
    IvfScratch s;
};

// Binary IVF (IVFFlatBinaryIndex semantics).
struct IvfBinState {
    int32_t nlist = 256, nprobe = 8, max_iter = 20;
    uint32_t seed = 42;
    int nbytes = 0, w4 = 0;      // row = w4 uint4 words
    int32_t kc = 0;              // centroids built = min(nlist, n)
    int64_t n = 0;
    DBuf cent;                   // kc*w4*16 bytes, in the reference's cluster order
    DBuf vecs, ids;              // CSR rows (list order) and original ids
    DBuf list_off;               // int64 kc+1, lists in cluster order
    std::vector<int64_t> h_off;
    std::vector<int64_t> top_rows;
    std::vector<int32_t> h_labels;
    int rc = 4096;
    IvfScratch s;
};

}  // namespace gn
