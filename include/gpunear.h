/*
 * gpunear.h — C ABI of the GB300 search library (libgpunear.so).
 *
 * Plain pointers and sizes only.  Every call returns a gn_status; on failure
 * gn_last_error() gives a message for the calling thread.  Results are always
 * nearest-first; a distance tie is broken by the lower database row index.
 *
 * Host-pointer entry points (the drop-in surface) copy inputs to the device and
 * results back inside the call.  *_device entry points take device pointers and
 * a cudaStream_t passed as void*, and return without synchronising.
 *
 * Each declaration names the reference interface it replaces, as
 * file:line within the PyNear 2.2.0 source tree.
 */
#ifndef GPUNEAR_H
#define GPUNEAR_H

#include <stdint.h>

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GN_OK = 0,
    GN_ERR_INVALID = 1,     /* bad argument: shape, k, dtype width (maps to ValueError) */
    GN_ERR_EMPTY = 2,       /* search on an index without data (maps to RuntimeError) */
    GN_ERR_CUDA = 3,        /* CUDA runtime failure */
    GN_ERR_OOM = 4,         /* device allocation failed */
    GN_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    GN_ERR_UNSUPPORTED = 6  /* valid request outside the implemented limits */
} gn_status;

typedef enum {
    GN_METRIC_L2 = 0,      /* Euclidean (sqrt) distance, float32 */
    GN_METRIC_L1 = 1,      /* Manhattan distance, float32 */
    GN_METRIC_LINF = 2,    /* Chebyshev distance, float32 */
    GN_METRIC_HAMMING = 3  /* popcount(a ^ b) over uint8 rows, int64 */
} gn_metric;

typedef struct gn_index gn_index;

/* library / device info */
int gn_version(void);
const char *gn_last_error(void);
int gn_device_info(int *num_sms, int *cc_major, int *cc_minor);
/* Kernel timing (no reference counterpart; used by the benchmark): while
 * enabled, each search brackets its dominant kernel with CUDA events on the
 * stream it launches on; gn_timing_last waits for the last bracket and reports
 * its duration and the kernel's name. */
int gn_timing_enable(int on);
int gn_timing_last(float *ms, char *name, int name_len);

/* Distance between two vectors of d floats (L2: Euclidean, L1, L-inf) or d
 * bytes (Hamming), host pointers, the result in *out.  Replaces the module
 * functions dist_l2 / dist_l1 / dist_chebyshev / dist_hamming
 * (pynear/src/PythonBindings.cpp, DistanceFunctions.hpp:304-448): float values
 * bit for bit those of dist_*_f_avx2; Hamming the true bit count.  Computed on
 * the GPU by one small kernel per call (operands in mapped pinned memory). */
int gn_dist(int32_t metric, const void *a, const void *b, int64_t d, double *out);

/* ── exact flat index ─────────────────────────────────────────────────────
 * Replaces the VP-tree indexes bound in pynear/src/PythonBindings.cpp:344-408
 * (VPTreeNumpyAdapter::set / searchKNN / search1NN, :36-90, and the binary
 * adapter VPTreeNumpyAdapterBinary, :147-176) with an exhaustive scan that
 * returns the exact k nearest rows.  Distances are the reference's
 * dist_l2_f_avx2 / dist_l1_f_avx2 / dist_chebyshev_f_avx2 values bit for bit
 * (pynear/include/DistanceFunctions.hpp:304-420) and exact Hamming counts.
 */
int gn_flat_create(int metric, gn_index **out);
/* data: n rows of dim floats (float metrics) or dim bytes (Hamming); copied. */
int gn_flat_set(gn_index *ix, const void *data, int64_t n, int64_t dim);
/* out_idx: nq*k int64; out_dist: nq*k float32 (float metrics) or int64
 * (Hamming).  When k > n the trailing entries of each row are -1 / 0.
 * Host-buffer searches (this one, gn_ivfl2_search_knn, gn_ivfbin_search_knn,
 * gn_tcflat_search_knn) block until the results are in the caller's buffers;
 * they accept pageable or page-locked memory (pageable buffers of up to 1 MB
 * are staged through the index's own page-locked buffers). */
int gn_flat_search_knn(gn_index *ix, const void *queries, int64_t nq, int64_t k, int64_t *out_idx, void *out_dist);
/* 1-NN shortcut (VPTree::search1NN, pynear/include/VPTree.hpp:169-191) */
int gn_flat_search_1nn(gn_index *ix, const void *queries, int64_t nq, int64_t *out_idx, void *out_dist);
int gn_flat_search_knn_device(gn_index *ix, const void *d_queries, int64_t nq, int64_t k, int64_t *d_idx,
                              void *d_dist, void *stream);
int gn_index_size(gn_index *ix, int64_t *n, int64_t *dim);
/* Exact Hamming k-NN that allocates no device memory.  No counterpart in the
 * reference: it is for callers that cannot call cudaMalloc at search time (a
 * process whose device memory is already owned by another allocator, or a
 * latency-critical loop that cannot take cudaMalloc's synchronisation).  All
 * arguments are device buffers: d_db n rows of nbytes (a multiple of 16)
 * packed bytes, d_queries nq rows of the same width (both 16-byte aligned),
 * d_idx / d_dist nq*k int64 results (nearest first, ties to the lower row).
 * The only other memory used is a fixed 16 MB array per device inside the
 * library, so nq * k must be at most 2 Mi (larger requests fail with
 * GN_ERR_INVALID); 1 <= k <= 256.  Set-up: the first call on a device loads
 * the library's scan kernels and that array (the CUDA driver loads modules lazily,
 * and reserves their memory then) and looks up the array's address
 * (cudaGetSymbolAddress); make that first call (nq = 0 is enough) at set-up
 * time, with the device current and before any stream capture; later calls
 * allocate nothing.  Every call uses the same array: calls that overlap on
 * the GPU (other streams, other threads) race and must be serialised by the
 * caller.  Returns without synchronising `stream`. */
int gn_hamming_knn_noalloc(const uint8_t *d_db, int64_t n, int64_t nbytes, const uint8_t *d_queries, int64_t nq,
                           int64_t k, int64_t *d_idx, int64_t *d_dist, void *stream);
int gn_index_destroy(gn_index *ix);

/* ── exact L2 via a tensor-core shortlist ─────────────────────────────────
 * Same contract as gn_flat_search_knn for GN_METRIC_L2 (the exact Euclidean
 * k nearest rows, the reference's dist_l2_f_avx2 values), computed in two
 * stages: a BF16 tcgen05 GEMM scores |x|^2 - 2 q.x with FP32 accumulation and
 * keeps the `shortlist` best rows per query, then those are re-ranked with the
 * reference's FP32 distance.  Exact whenever the true k nearest rows are inside
 * the shortlist.  Shortlist: 16, 32, 40, 48, 56 or 64; k <= min(32, shortlist).
 * Replaces VPTreeL2Index (pynear/src/PythonBindings.cpp:344-350) for
 * large batches.
 */
int gn_tcflat_create(int32_t shortlist, gn_index **out);
int gn_tcflat_set(gn_index *ix, const float *data, int64_t n, int64_t d);
int gn_tcflat_search_knn(gn_index *ix, const float *queries, int64_t nq, int64_t k, int64_t *out_idx,
                         float *out_dist);
/* d_queries: nq rows of round_up(d, 4) floats (zero padded) on the device */
int gn_tcflat_search_knn_device(gn_index *ix, const float *d_queries, int64_t nq, int64_t k, int64_t *d_idx,
                                float *d_dist, void *stream);
/* operand precision of the shortlist GEMM: 0 = BF16 (default), 1 = FP8 E4M3
 * with one FP32 scale per row (max |x| -> 448), scored as
 * |x|^2 - 2 s_q s_x (q8 . x8); FP8 takes shortlists of 16 to 56.  May be
 * called before or after set() (the low-precision copy is rebuilt on the GPU). */
int gn_tcflat_set_precision(gn_index *ix, int32_t precision);
/* error word of the last tensor-core launch (nonzero: a bounded wait expired) */
int gn_tc_error(gn_index *ix, int32_t *err_out);

/* ── float k-means coarse quantiser ───────────────────────────────────────
 * Replaces kmeans_l2 (pynear/include/KMeans.hpp:25-126, bound as
 * _pynear.kmeans_l2 at pynear/src/PythonBindings.cpp:305-329): k-means++
 * seeding, Lloyd iterations with the assignment done as a GEMM on the device
 * and FP64 centroid sums; stops when no label changes or after max_iter.
 * labels: n int32; centroids: k*d float32; iters_out may be NULL.
 */
int gn_kmeans_l2(const float *data, int64_t n, int64_t d, int64_t k, int64_t max_iter, uint32_t seed,
                 int32_t *labels, float *centroids, int64_t *iters_out);

/* ── IVF-flat L2 index ────────────────────────────────────────────────────
 * Replaces IVFFlatL2Index (pynear/forest.py:167-194; set :36-59, searchKNN
 * :63-111).  Lists are a device-resident CSR (offsets, permuted rows, original
 * ids); distances are squared L2; a query may get fewer than k results when
 * its probed lists hold fewer than k rows (out_cnt gives the count).
 */
int gn_ivfl2_create(int32_t n_clusters, int32_t n_probe, gn_index **out);
int gn_ivfl2_set(gn_index *ix, const float *data, int64_t n, int64_t d);
/* build from given centroids and labels (no k-means), e.g. to reproduce an
 * index built elsewhere; empty clusters are dropped as forest.py:51-53 does */
int gn_ivfl2_set_assigned(gn_index *ix, const float *data, int64_t n, int64_t d, const float *centroids,
                          int32_t n_centroids, const int32_t *labels);
int gn_ivfl2_search_knn(gn_index *ix, const float *queries, int64_t nq, int64_t k, int64_t *out_idx,
                        float *out_dist, int64_t *out_cnt);
/* Concurrent search contexts (no reference counterpart; results unchanged):
 * a fork views the parent's lists (centroids, CSR offsets, rows, ids; nothing
 * is copied) and owns its scratch, stream, error word and captured graphs, so
 * searches on the parent and its forks may run at the same time, each on its
 * own stream.  Settings (n_probe, engine, shortlist, prober, tuning) start as
 * the parent's.  While forks live, set / set_assigned on the parent fail with
 * GN_ERR_INVALID; gn_index_destroy of the parent defers its release to the
 * last fork's.  Forks of forks are refused. */
int gn_ivfl2_fork(gn_index *parent, gn_index **out);
/* device variant: queries [nq x d] row-major on the device; results written
 * to device buffers in stream order (no synchronisation).  Searches of one
 * index share its scratch: issue them on one stream, or order them (with
 * graphs enabled they run on the index's own stream and are ordered) */
int gn_ivfl2_search_knn_device(gn_index *ix, const float *d_queries, int64_t nq, int64_t k, int64_t *d_idx,
                               float *d_dist, int64_t *d_cnt, void *stream);
int gn_ivfl2_set_n_probe(gn_index *ix, int32_t n_probe);
/* CUDA-graph replay (no reference counterpart; same results): searches of
 * 1..max_batch queries with this k run as one captured graph per batch size,
 * replayed on fixed staging buffers; a configuration change or a scratch
 * reallocation drops the cached graphs.  max_batch 0 disables.  The call runs
 * one search of max_batch queries to size the scratch. */
int gn_ivfl2_enable_graphs(gn_index *ix, int64_t max_batch, int32_t k);
/* out[0] max_batch (0: disabled), out[1] cached graphs, out[2] replays,
 * out[3] captures that failed (those batches ran uncaptured) */
int gn_ivfl2_graph_info(gn_index *ix, int64_t *out);
/* Autotuner of the tensor-core engine (no reference counterpart; results
 * unchanged): for each batch-size bucket [1,4) [4,16) [16,64) [64,256)
 * [256,1024) [1024,4096) [4096,..) that the nq sample queries reach, times
 * every combination of rows per list-scan work unit (256/1024/4096), most
 * blocks per query selection (1/4/16) and selector threads per query (32 =
 * one warp, 128/256 = a block), reps
 * runs each, and keeps the fastest; then, with those fixed, the tile shape:
 * queries per list-scan work unit, the MMA's N (32/64/128).
 * table: 7 x {rc, bmax, nt, qc}; zeros = the built-in choice. */
int gn_ivfl2_autotune(gn_index *ix, const float *queries, int64_t nq, int64_t k, int32_t reps, int32_t *table_out);
int gn_ivfl2_get_tuning(gn_index *ix, int32_t *table_out);
int gn_ivfl2_set_tuning(gn_index *ix, const int32_t *table);
/* Search engine (no reference counterpart; same result contract):
 *   mode 0  FP32 CUDA-core scan, distances |q|^2 + |x|^2 - 2 q.x clamped at 0,
 *           the formula of forest.py:189-194;
 *   mode 1  BF16 tcgen05 GEMM keeps `shortlist` candidates per query over the
 *           probed lists, re-ranked with the exact squared L2 in FP32
 *           (compensated sum); k <= min(32, shortlist). */
int gn_ivfl2_set_mode(gn_index *ix, int32_t mode, int32_t shortlist);
/* error word of the last tensor-core launch (nonzero: a bounded wait expired) */
int gn_ivfl2_error(gn_index *ix, int32_t *err_out);
/* (gn_ivfl2_error reads the error word after the device has drained and
 * clears it; gn_ivfl2_search_knn reports it itself as GN_ERR_TIMEOUT.)
 * Failure drill, for tests (no reference counterpart; it exercises on the GPU
 * the error path whose host-side analogue is the reference's search exception,
 * VPTree.hpp:145-147): the next tensor-core list scan of this index issues no
 * tile copies and bounds its pipeline waits to 200,000 cycles, so they run
 * out; the launch ends with the error word set and its tensor memory freed,
 * and the search reports GN_ERR_TIMEOUT.  The drill disarms itself after that
 * one launch. */
int gn_ivfl2_failure_drill(gn_index *ix);
/* Work of the last search, for throughput accounting (no reference
 * counterpart): out[0] (query, probe) pairs, out[1] scored (pair, row)
 * entries, out[2] rows of the distinct lists probed, out[3] tensor-core units. */
int gn_ivfl2_last_work(gn_index *ix, int64_t *out);
int gn_ivfl2_info(gn_index *ix, int32_t *n_clusters_built, int32_t *n_probe, int64_t *n, int64_t *d);
/* copy out the built state: centroids (n_clusters_built*d), list offsets
 * (n_clusters_built+1, int64), original ids in list order (n, int64) */
int gn_ivfl2_export(gn_index *ix, float *centroids, int64_t *offsets, int64_t *ids);

/* ── MIHBinaryIndex (pynear/include/MIH.hpp:58-175,
 *    pynear/src/PythonBindings.cpp:253-271,468-481) ───────────────────────────
 * Multi-index hashing: m sub-strings of nbytes/m <= 8 bytes, one hash table
 * each (built on the host at set()).  A query's candidates are the rows whose
 * t-th sub-string is within radius/m bits of the query's for some t; they are
 * verified on the GPU (exact Hamming, top-k by (distance, lower row)),
 * nearest first; out_cnt < k when fewer rows are candidates.  An empty index
 * returns no results.  k <= 256. */
int gn_mih_create(int32_t m, gn_index **out);
int gn_mih_set(gn_index *ix, const uint8_t *data, int64_t n, int64_t nbytes);
int gn_mih_search_knn(gn_index *ix, const uint8_t *queries, int64_t nq, int64_t k, int32_t radius, int64_t *out_idx,
                      int64_t *out_dist, int64_t *out_cnt);
int gn_mih_info(gn_index *ix, int32_t *m, int64_t *n, int64_t *nbytes);

/* ── learned probing (no reference counterpart) ───────────────────────────
 * An MLP (64 -> 256 -> 256 -> one logit per list; BF16 weights, FP32
 * accumulation at inference) scores a query's 64 nearest lists by the
 * probability that they hold one of its exact 10 nearest neighbours; the index
 * probes the lists whose logit reaches a threshold (always the nearest one),
 * instead of a fixed n_probe.  Trained on the GPU by the library's own forward,
 * backward and Adam kernels against labels from exact search.
 * Parameters are one flat FP32 array: W1 [nlist x 256] | b1 [256] |
 * W2 [256 x 256] | b2 [256] | W3 [nlist x 256] | b3 [nlist].
 */
int gn_prober_create(int32_t nlist, uint32_t seed, gn_index **out);
int gn_prober_num_params(gn_index *pr, int64_t *n);
int gn_prober_get_params(gn_index *pr, float *out);
int gn_prober_set_params(gn_index *pr, const float *in);
/* mean binary cross-entropy and its gradient for B explicit examples:
 * cand [B x 64] list ids (-1 = none), feat [B x 64], lab [B x 64] in {0,1} */
int gn_prober_loss_grad(gn_index *pr, int64_t B, const int32_t *cand, const float *feat, const float *lab,
                        float *loss_out, float *grads_out);
/* queries: nq host rows of the index dimension; gt: [nq x k] exact neighbour
 * ids; loss_out: one mean loss per epoch */
int gn_prober_train(gn_index *pr, gn_index *ivf, const float *queries, int64_t nq, const int64_t *gt, int32_t k,
                    int32_t epochs, int32_t batch, float lr, float *loss_out);
int gn_ivfl2_set_prober(gn_index *ivf, gn_index *pr, float logit_tau);
int gn_ivfl2_last_nprobed(gn_index *ivf, int64_t nq, int32_t *out);

/* ── IVF-flat binary index ────────────────────────────────────────────────
 * Replaces IVFFlatBinaryIndex (pynear/include/BinaryIVF.hpp:34-227, bound at
 * pynear/src/PythonBindings.cpp:454-466): binary k-means++ and majority-vote
 * Lloyd iterations reproduce the reference's centroids exactly (same mt19937
 * stream, same integer arithmetic); the search returns the lexicographic
 * (distance, index) top-k of the probed lists.
 */
int gn_ivfbin_create(int32_t nlist, int32_t nprobe, int32_t max_iter, uint32_t seed, gn_index **out);
int gn_ivfbin_set(gn_index *ix, const uint8_t *data, int64_t n, int64_t nbytes);
int gn_ivfbin_search_knn(gn_index *ix, const uint8_t *queries, int64_t nq, int64_t k, int64_t *out_idx,
                         int64_t *out_dist, int64_t *out_cnt);
int gn_ivfbin_get_params(gn_index *ix, int32_t *nlist, int32_t *nprobe);
int gn_ivfbin_set_nprobe(gn_index *ix, int32_t nprobe);
/* copy out centroids (k*nbytes) and labels (n); k_out gets min(nlist, n) */
int gn_ivfbin_export(gn_index *ix, uint8_t *centroids, int32_t *labels, int32_t *k_out);

/* ── headless Voronoi raster (demo/voronoi.py:84-110) ─────────────────────
 * Replaces the reference's pixel-grid search1NN (VPTreeL2Index over the
 * n_seeds 2-D seeds, queried with every pixel (xs[c], ys[r])) and palette
 * lookup.  seeds: n_seeds x 2 floats (x, y); xs: width floats; ys: height
 * floats.  Outputs, row-major height x width, each optional (NULL = skip, at
 * least one given): out_ids the nearest seed (ties to the lower index, the
 * exact flat search1NN answer), out_dist its L2 distance, out_rgba 4 bytes per
 * pixel = palette[(id % n_palette)] (palette: n_palette x 4 bytes).  The
 * _device form takes device pointers and launches on `stream` without
 * synchronising (seeds 8-byte, palette and out_rgba 4-byte aligned). */
int gn_voronoi_raster(const float *seeds, int64_t n_seeds, const float *xs, int64_t width, const float *ys,
                      int64_t height, int32_t *out_ids, float *out_dist, const uint8_t *palette, int64_t n_palette,
                      uint8_t *out_rgba);
int gn_voronoi_raster_device(const float *d_seeds, int64_t n_seeds, const float *d_xs, int64_t width,
                             const float *d_ys, int64_t height, int32_t *d_ids, float *d_dist,
                             const uint8_t *d_palette, int64_t n_palette, uint8_t *d_rgba, void *stream);

#ifdef __cplusplus
}
#endif

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#endif /* GPUNEAR_H */
