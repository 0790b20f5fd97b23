// ivf_tune.cu — autotuner of the tensor-core IVF engine's launch choices.
//
// The tensor-core engine has four launch choices whose best values depend on
// the batch size, the list-length distribution, the probe width and the GPU:
//   rc    list rows per work unit of the list scan (256, 1024, 4096): short
//         units spread a small batch's few lists over all SMs, long ones cut
//         per-unit overhead;
//   bmax  most blocks one query's selection is split over (1, 4, 16): splitting
//         shortens a small batch's critical path, at the price of a merge;
//   nt    selector threads per query (32, 128, 256): 32 is one warp per query
//         (no block barriers, for large batches), 128 and 256 a block of that
//         many threads per query (part);
//   qc    queries per list-scan work unit, the MMA's N side (32, 64, 128): the
//         tile shape; smaller units spread a mid-size batch's lists over more
//         SMs at the price of more reads of each list's rows.
// The first three are timed jointly with qc = 128, then qc with the best of them.
// gn_ivfl2_autotune times every combination on the caller's sample queries,
// for each batch-size bucket the sample covers ([1,4) [4,16) ... [4096,..)),
// with CUDA events on the index's stream, and keeps the fastest per bucket in
// the index's tuning table; the table can be read out and set back (kept with
// a pickled index), and a cleared entry (zeros) restores the built-in choice.
#include <algorithm>
#include <vector>

#include "ivf.cuh"

namespace gn {

static const int TUNE_RC[] = {256, 1024, 4096};
static const int TUNE_BMAX[] = {1, 4, 16};
static const int TUNE_NT[] = {32, 128, 256};  // 32: one warp per query
static const int TUNE_QC[] = {32, 64};  // besides the built-in 128
constexpr int TUNE_COLS = 4;
static const int64_t TUNE_NQ[7] = {2, 8, 32, 128, 512, 2048, 4096};  // representative batch per bucket

}  // namespace gn

using namespace gn;

extern "C" int gn_ivfl2_autotune(gn_index *ix, const float *queries, int64_t nq, int64_t k, int32_t reps,
                                 int32_t *table_out) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    IvfL2State &S = *ix->ivfl2;
    if (S.nc == 0) return fail(GN_ERR_EMPTY, "Index is empty — call set() first");
    if (S.mode != 1) return fail(GN_ERR_INVALID, "autotune applies to the tensor-core engine (mode 1)");
    if (nq <= 0 || !queries) return fail(GN_ERR_INVALID, "autotune needs sample queries");
    if (k <= 0 || k > 32 || k > S.shortlist) return fail(GN_ERR_INVALID, "k must be in [1, min(32, shortlist)]");
    if (reps <= 0) reps = 3;
    std::lock_guard<std::mutex> lk(ix->mu);
    GN_TRY(make_stream(ix));
    cudaStream_t st = ix->stream;
    const int64_t nmax = std::min<int64_t>(nq, TUNE_NQ[6]);
    DBuf dq, di, dd, dc;
    GN_TRY(upload_rows(dq, queries, nmax, S.d * 4, S.dp / 4, st));
    GN_TRY(di.ensure((size_t)nmax * k * 8));
    GN_TRY(dd.ensure((size_t)nmax * k * 4));
    GN_TRY(dc.ensure((size_t)nmax * 8));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    GN_CUDA_TRY(cudaEventCreate(&e0));
    GN_CUDA_TRY(cudaEventCreate(&e1));
    struct Ev {
        cudaEvent_t a, b;
        ~Ev() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } ev{e0, e1};
    const int nsm = dev_info().num_sms;
    for (int b = 0; b < 7; ++b) {
        const int64_t lo = b == 0 ? 1 : ((int64_t)1 << (2 * b));
        const int64_t nb = std::min<int64_t>(TUNE_NQ[b], nmax);
        if (nb < lo) continue;  // the sample does not reach this bucket: keep its entry
        float best = 0.f;
        IvfL2State::TcTune best_t;
        for (int rc : TUNE_RC)
            for (int bm : TUNE_BMAX)
                for (int nt : TUNE_NT) {
                    // a split the batch never uses would time the same launch again (the
                    // warp-per-query selector never splits)
                    if (bm > 1 && (nb * 2 > (int64_t)nsm * 4 || nt == 32)) continue;
                    S.tune[b].rc = rc;
                    S.tune[b].bmax = bm;
                    S.tune[b].nt = nt;
                    GN_TRY(ivfl2_search_core(ix, dq.as<float>(), nb, (int)k, di.as<int64_t>(), dd.as<float>(),
                                             dc.as<int64_t>(), st));  // warm-up (sizes the scratch)
                    GN_CUDA_TRY(cudaEventRecord(e0, st));
                    for (int r = 0; r < reps; ++r)
                        GN_TRY(ivfl2_search_core(ix, dq.as<float>(), nb, (int)k, di.as<int64_t>(),
                                                 dd.as<float>(), dc.as<int64_t>(), st));
                    GN_CUDA_TRY(cudaEventRecord(e1, st));
                    GN_CUDA_TRY(cudaEventSynchronize(e1));
                    float ms = 0.f;
                    GN_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
                    if (best_t.rc == 0 || ms < best) {
                        best = ms;
                        best_t = S.tune[b];
                    }
                }
        // the tile shape, with the other choices fixed at their best (timed above
        // with the built-in 128 queries per unit)
        for (int qc : TUNE_QC) {
            S.tune[b] = best_t;
            S.tune[b].qc = qc;
            GN_TRY(ivfl2_search_core(ix, dq.as<float>(), nb, (int)k, di.as<int64_t>(), dd.as<float>(),
                                     dc.as<int64_t>(), st));
            GN_CUDA_TRY(cudaEventRecord(e0, st));
            for (int r = 0; r < reps; ++r)
                GN_TRY(ivfl2_search_core(ix, dq.as<float>(), nb, (int)k, di.as<int64_t>(), dd.as<float>(),
                                         dc.as<int64_t>(), st));
            GN_CUDA_TRY(cudaEventRecord(e1, st));
            GN_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0.f;
            GN_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) {
                best = ms;
                best_t.qc = qc;
            }
        }
        if (best_t.qc == 0) best_t.qc = 128;
        S.tune[b] = best_t;
    }
    S.cfg++;  // captured graphs hold the old choices
    if (table_out)
        for (int b = 0; b < 7; ++b) {
            table_out[TUNE_COLS * b] = S.tune[b].rc;
            table_out[TUNE_COLS * b + 1] = S.tune[b].bmax;
            table_out[TUNE_COLS * b + 2] = S.tune[b].nt;
            table_out[TUNE_COLS * b + 3] = S.tune[b].qc;
        }
    return GN_OK;
}

extern "C" int gn_ivfl2_get_tuning(gn_index *ix, int32_t *table_out) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2 || !table_out) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    std::lock_guard<std::mutex> lk(ix->mu);
    for (int b = 0; b < 7; ++b) {
        table_out[TUNE_COLS * b] = ix->ivfl2->tune[b].rc;
        table_out[TUNE_COLS * b + 1] = ix->ivfl2->tune[b].bmax;
        table_out[TUNE_COLS * b + 2] = ix->ivfl2->tune[b].nt;
        table_out[TUNE_COLS * b + 3] = ix->ivfl2->tune[b].qc;
    }
    return GN_OK;
}

extern "C" int gn_ivfl2_set_tuning(gn_index *ix, const int32_t *table) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2 || !table) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    for (int b = 0; b < 7; ++b) {
        const int32_t rc = table[TUNE_COLS * b], bm = table[TUNE_COLS * b + 1], nt = table[TUNE_COLS * b + 2],
                      qc = table[TUNE_COLS * b + 3];
        if (rc && (rc < 256 || rc % 128)) return fail(GN_ERR_INVALID, "tuning: rc must be 0 or a multiple of 128 >= 256");
        if (bm < 0 || bm > 16) return fail(GN_ERR_INVALID, "tuning: bmax must be in [0, 16]");
        if (nt && nt != 32 && nt != 128 && nt != 256)
            return fail(GN_ERR_INVALID, "tuning: nt must be 0, 32, 128 or 256");
        if (qc && qc != 32 && qc != 64 && qc != 128) return fail(GN_ERR_INVALID, "tuning: qc must be 0, 32, 64 or 128");
    }
    std::lock_guard<std::mutex> lk(ix->mu);
    for (int b = 0; b < 7; ++b) {
        ix->ivfl2->tune[b].rc = table[TUNE_COLS * b];
        ix->ivfl2->tune[b].bmax = table[TUNE_COLS * b + 1];
        ix->ivfl2->tune[b].nt = table[TUNE_COLS * b + 2];
        ix->ivfl2->tune[b].qc = table[TUNE_COLS * b + 3];
    }
    ix->ivfl2->cfg++;
    return GN_OK;
}
