// ivf.cuh — IVF index state and device search plumbing.
#pragma once

#include <vector>

#include "index.cuh"

namespace gn {

constexpr int IVF_RHO = 64;  // per list: radii of its rows nearest the centroid kept (>= the largest shortlist)

// Per-batch scratch of an IVF search (device resident, reused).
struct IvfScratch {
    DBuf q, qn, probes, probes64, pdist, bcnt, boff, bucket, fill, slot_rel, qcount, qslot, item_off, counter, part,
        cpart, nprobed, qbound,  // qbound: per query, the ordered score bound of the tensor-core list scan
        mh1, mcand, mcb, mqn;    // batched prober MLP: first-layer outputs, candidates, their bounds, |q|^2
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
    // tensor-core engine (mode 1): BF16 rows in list order, shortlist + re-rank
    int mode = 0;                // 0 FP32 CUDA-core scan, 1 BF16 tcgen05 shortlist + exact FP32 re-rank
    int shortlist = 40;
    int K = 0;                   // BF16 row length, round_up(d, 64)
    DBuf x16;                    // BF16 rows in list order, tiled: every list padded to a multiple of
                                 // 128 rows (list l from padded row xoff[l]); the 128 rows of a tile
                                 // stored K-slice by K-slice, each slice (128 rows x 64 values, 16 KB)
                                 // contiguous, so one TMA box is one contiguous block
    DBuf xoff;                   // int64 nc + 1: padded start row of each list in x16
    int64_t x16_rows = 0;        // padded rows
    DBuf qb, aslot, abound, units, nunits, err, scores;
    // score bound of the tensor-core list scan: per list, the distances |x - c|
    // of its 64 rows nearest the centroid (ascending, slightly rounded up;
    // +inf past the list's size), and the largest row norm of the index
    DBuf rho;
    float xmax = 0.f;
    DBuf sel_part, sel_done;     // split selection: partial best-S lists, per-query arrival counters
    DBuf sched;                  // unit counters of the tensor-core scans (coarse, lists)
    DBuf tmin;                   // per (score slot, 32-row quarter): minimum ordered score
    int drill = 0;               // failure drill armed for the next tensor-core list scan (tests)
    DBuf q16, c16, cunits, cnunits, caslot, cscores;  // tensor-core coarse stage
    // learned probing (prober.cu): attached model and logit threshold
    gn_index *prober = nullptr;
    float prober_tau = 0.f;
    // launch choices of the tensor-core engine per batch-size bucket (ivf_tune.cu):
    // 0 = built-in heuristic
    struct TcTune {
        int32_t rc = 0;    // list rows per work unit (256, 1024, 4096)
        int32_t bmax = 0;  // most blocks one query's selection is split over (1..16)
        int32_t nt = 0;    // selector threads per block (128, 256)
        int32_t qc = 0;    // queries per list-scan work unit, the MMA's N (32, 64, 128)
    } tune[7];
    // search configuration version (bumped by every setter); CUDA graphs
    // captured for one configuration are replayed only under it
    uint64_t cfg = 1;
    struct IvfGraphs *graphs = nullptr;
};

// Captured batch pipelines of a float IVF index (ivf_graph.cu), one per batch
// size, replayed on fixed staging buffers.
struct IvfGraphs {
    int64_t max_batch = 0;
    int k = 0, dp = 0;
    DBuf gq, gidx, gdist, gcnt;  // staging: queries (pitch dp), indices, distances, counts
    std::vector<std::pair<int64_t, cudaGraphExec_t>> execs;  // batch size -> graph
    uint64_t cfg = 0, gen = 0;
    int64_t replays = 0, capture_failures = 0;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;  // order the index's stream after / before the caller's
    void clear();
    ~IvfGraphs();
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

// slot_rc: rows per partial slot (defaults to rc); 1 makes every (query, probe)
// own a segment of one entry per list row (the tensor-core store mode).
int ivf_plan(IvfScratch &S, int64_t nq, int np, int nc, const int64_t *d_list_off, int rc, int qchunk,
             cudaStream_t st, int slot_rc = 0);
int64_t ivf_max_slots_per_query(const std::vector<int64_t> &top, int np, int rc);
int ivfl2_coarse(gn_index *ix, const float *dQ, int64_t nq, int np, cudaStream_t st);
int ivfl2_coarse_run(gn_index *ix, const float *dQ, int64_t nq, int np, bool keep_keys, int *nsplit_out,
                     cudaStream_t st);
int ivfl2_coarse_sorted_keys(gn_index *ix, const float *dQ, int64_t nq, int np, uint64_t *keys, cudaStream_t st);
int ivfl2_probes(gn_index *ix, const float *dQ, int64_t nq, int *np_out, cudaStream_t st);
int ivfl2_search_core(gn_index *ix, const float *dQ, int64_t nq, int k, int64_t *d_idx, float *d_dist, int64_t *d_cnt,
                      cudaStream_t st);
// batch-size bucket of the tuning table: [1,4) [4,16) [16,64) [64,256) [256,1024) [1024,4096) [4096,..)
inline int tune_bucket(int64_t nq) {
    int b = 0;
    for (int64_t x = nq; x >= 4 && b < 6; x >>= 2) ++b;
    return b;
}
// Graph-replayed search; queries/results on the host or the device.
int ivfl2_search_graph(gn_index *ix, const float *q, bool q_host, int64_t nq, int k, int64_t *idx, float *dist,
                       int64_t *cnt, bool out_host, cudaStream_t user);
int ivfl2_search_tc(gn_index *ix, const float *dQ, int64_t nq, int k, int64_t *d_idx, float *d_dist, int64_t *d_cnt,
                    cudaStream_t st);
int ivfl2_prepare_tc(gn_index *ix, cudaStream_t st);

}  // namespace gn
