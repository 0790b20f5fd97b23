// ivf_tc.cu — tensor-core engine of the float IVF index.
//
// Same bucketing and work plan as the FP32 scan (ivf.cu), then:
//   1. Qb      the BF16 copy of each (query, probe) pair's query, rows grouped by
//              list (bucket order), so one TMA box covers a work unit's queries;
//   2. units   one tensor-core work unit per (list, 128-query chunk, row chunk);
//   3. scan    tc_ivf_kernel: BF16 tcgen05 GEMM of the list's rows (M = 128
//              per tile) against the unit's queries (N = 32..256) with FP32
//              accumulation; the score |x|^2 - 2 q.x (exact FP32 |x|^2) of
//              every (pair, row) goes to the pair's segment of a score buffer;
//   4. select  one warp per query walks its probed lists' segments with a
//              register top-S (S = shortlist), recomputes the S candidates'
//              squared L2 exactly in FP32 with a compensated sum (two-product
//              + two-sum) and returns the k nearest, ties to the lower
//              original index.
// Work units are short (a list holds ~1k rows), so selection is kept out of
// the tensor-core kernel: a per-unit top-S would pay its warm-up on every
// unit.
// Everything stays on the device; the batch has no host round trip.
#include <cuda_bf16.h>

#include <algorithm>
#include <vector>

#include "ivf.cuh"
#include "kmeans.cuh"
#include "tc_ivf.cuh"
#include "tc_scan.cuh"
#include "timing.cuh"
#include "gemm_topk.cuh"
#include "topk.cuh"

namespace gn {

constexpr int TC_QCHUNK = 256;  // queries per tensor-core work unit (MMA N <= 256)

__global__ void qb_fill_kernel(const float *__restrict__ Q, int d, int dp, int K, int np,
                               const int64_t *__restrict__ bucket, const int64_t *__restrict__ boff_end,
                               const int64_t *__restrict__ qslot, const int64_t *__restrict__ slot_rel,
                               __nv_bfloat16 *__restrict__ qb, int64_t *__restrict__ aslot, int64_t max_pairs) {
    const int64_t pos = (int64_t)blockIdx.x;
    if (pos >= max_pairs || pos >= *boff_end) return;
    const int64_t pair = bucket[pos];
    const int64_t q = pair / np;
    for (int j = threadIdx.x; j < K; j += blockDim.x)
        qb[pos * K + j] = __float2bfloat16_rn(j < d ? Q[q * dp + j] : 0.f);
    if (threadIdx.x == 0) aslot[pos] = qslot[q] + slot_rel[pair];
}

__device__ __forceinline__ int find_list_tc(const int64_t *item_off, int nc, int64_t item) {
    int lo = 0, hi = nc;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (item_off[mid] <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void tc_units_kernel(const int64_t *__restrict__ item_off, int nc, const int64_t *__restrict__ boff,
                                const int64_t *__restrict__ list_off, int rc, int64_t max_units,
                                TcUnit *__restrict__ units, int64_t *__restrict__ n_units) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = item_off[nc];
    if (i == 0) *n_units = min(total, max_units);
    if (i >= total || i >= max_units) return;
    const int l = find_list_tc(item_off, nc, i);
    const int64_t lb = list_off[l], le = list_off[l + 1];
    const int64_t nrc = (le - lb + rc - 1) / rc;
    const int64_t local = i - item_off[l];
    const int64_t qc = local / nrc, rch = local % nrc;
    TcUnit u;
    u.a0 = boff[l] + qc * TC_QCHUNK;
    u.na = (int32_t)min((int64_t)TC_QCHUNK, boff[l + 1] - u.a0);
    u.r0 = lb + rch * rc;
    u.r1 = min(le, u.r0 + rc);
    u.rbase = lb;
    u.rch = (int32_t)rch;
    units[i] = u;
}

// Squared L2 with a compensated FP32 sum: each (q_i - x_i)^2 is split into its
// rounded product and the product's exact error (fma), the running sum keeps
// its rounding error (two-sum); the errors are added back at the end.
__device__ __forceinline__ float l2sq_compensated(const float *__restrict__ q, const float *__restrict__ x, int d) {
    float s = 0.f, c = 0.f;
    for (int i = 0; i < d; ++i) {
        const float t = __fsub_rn(q[i], x[i]);
        const float p = __fmul_rn(t, t);
        const float e = __fmaf_rn(t, t, -p);
        const float s2 = __fadd_rn(s, p);
        const float bp = __fsub_rn(s2, s);
        const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(s2, bp)), __fsub_rn(p, bp));
        s = s2;
        c = __fadd_rn(c, __fadd_rn(err, e));
    }
    return __fadd_rn(s, c);
}

// Selection over a query's score segments.  W warps share one query (W = 1
// for large batches, up to 16 for small ones): warp w takes every W-th block
// of 128 scores, keeps a register top-S, the partial lists meet in shared
// memory and warp 0 merges them, re-ranks the S candidates exactly and writes
// the k nearest.
template <int RS>
__global__ void ivf_tc_select_kernel(const float *__restrict__ scores, const int32_t *__restrict__ probes, int np,
                                     const int64_t *__restrict__ qseg, const int64_t *__restrict__ seg_rel,
                                     const int64_t *__restrict__ list_off, int S, const float *__restrict__ Q,
                                     const float *__restrict__ X, int d, int dp, const int32_t *__restrict__ ids,
                                     int64_t nq, int k, int W, int64_t *__restrict__ out_idx,
                                     float *__restrict__ out_dist, int64_t *__restrict__ out_cnt) {
    extern __shared__ uint64_t sel_smem[];  // [blockDim/32][32*RS] partial lists
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int qpb = (blockDim.x >> 5) / W;  // queries per block
    const int64_t q = (int64_t)blockIdx.x * qpb + warp / W;
    const int wq = warp % W;
    const bool active = q < nq;
    const float INF = __int_as_float(0x7f800000);
    WarpTopK<RS> L;
    L.init();
    uint64_t thr = KEY_EMPTY;
    float thr_f = INF;
    if (active) {
        int64_t blk = 0;  // running index of 128-score blocks over the query's segments
        for (int p = 0; p < np; ++p) {
            const int64_t pair = q * np + p;
            const int32_t l = probes[pair];
            if (l < 0) continue;
            const int64_t lb = list_off[l], len = list_off[l + 1] - lb;
            const float *sc = scores + qseg[q] + seg_rel[pair];
            const int64_t nblk = (len + 127) / 128;
            // first block of this segment owned by warp wq
            int64_t b0 = (wq - blk % W + W) % W;
            for (int64_t b = b0; b < nblk; b += W) {
                const int64_t i0 = b * 128;
                float v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t i = i0 + u * 32 + lane;
                    v[u] = (i < len) ? __ldg(sc + i) : INF;
                }
                const float m = fminf(fminf(v[0], v[1]), fminf(v[2], v[3]));
                if (!__any_sync(0xffffffffu, m <= thr_f)) continue;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int64_t i = i0 + u * 32 + lane;
                    const uint64_t key = (i < len) ? make_key(f2ord(v[u]), (uint32_t)(lb + i)) : KEY_EMPTY;
                    L.offer(key, thr, S);
                    thr_f = (thr == KEY_EMPTY) ? INF : ord2f(key_dist(thr));
                }
            }
            blk += nblk;
        }
    }
    if (W > 1) {
        uint64_t *mine = sel_smem + (size_t)warp * 32 * RS;
#pragma unroll
        for (int r = 0; r < RS; ++r) mine[r * 32 + lane] = L.v[r];
        __syncthreads();
        if (wq == 0 && active) {
            for (int w = 1; w < W; ++w) {
                const uint64_t *other = sel_smem + (size_t)(warp + w) * 32 * RS;
#pragma unroll
                for (int r = 0; r < RS; ++r) L.offer(other[r * 32 + lane], thr, S);
            }
        }
    }
    if (!active || wq != 0) return;
    WarpTopK<1> F;
    F.init();
    uint64_t fthr = KEY_EMPTY;
#pragma unroll
    for (int r = 0; r < RS; ++r) {
        const int pos = r * 32 + lane;
        const uint64_t key = L.v[r];
        uint64_t fk = KEY_EMPTY;
        if (pos < S && key != KEY_EMPTY) {
            const int64_t row = key_idx(key);
            const float dd = l2sq_compensated(Q + q * dp, X + row * dp, d);
            fk = make_key(__float_as_uint(dd), (uint32_t)ids[row]);
        }
        F.offer(fk, fthr, k);
    }
    const uint64_t key = F.v[0];
    const bool e = key == KEY_EMPTY;
    if (lane < k) {
        out_idx[q * k + lane] = e ? -1 : (int64_t)key_idx(key);
        out_dist[q * k + lane] = e ? 0.f : __uint_as_float(key_dist(key));
    }
    const int cnt = __popc(__ballot_sync(0xffffffffu, lane < k && !e));
    if (lane == 0 && out_cnt) out_cnt[q] = cnt;
}

int ivfl2_prepare_tc(gn_index *ix, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    S.K = (int)round_up(S.d, 64);
    const int64_t rows = std::max<int64_t>(S.n, 256);  // at least one 256-row TMA box
    GN_TRY(S.x16.ensure((size_t)rows * S.K * 2));
    GN_CUDA_TRY(cudaMemsetAsync(S.x16.p, 0, (size_t)rows * S.K * 2, st));
    to_bf16_rows(S.vecs.as<float>(), S.n, S.d, S.dp, S.x16.p, S.K, st);
    GN_TRY(S.err.ensure(4));
    GN_CUDA_TRY(cudaMemsetAsync(S.err.p, 0, 4, st));
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

int ivfl2_search_tc(gn_index *ix, const float *dQ, int64_t nq, int k, int64_t *d_idx, float *d_dist, int64_t *d_cnt,
                    cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    IvfScratch &T = S.s;
    if (k > 32 || k > S.shortlist) return fail(GN_ERR_UNSUPPORTED, "tensor-core IVF supports k <= min(32, shortlist)");
    if (S.K == 0) GN_TRY(ivfl2_prepare_tc(ix, st));
    int np = 1;
    GN_TRY(ivfl2_probes(ix, dQ, nq, &np, st));
    // work items of rc rows (short items for small batches so that their few
    // lists still spread over all SMs); every pair owns a score segment
    const int rc = nq >= 512 ? S.rc_tc : (nq >= 64 ? 1024 : 256);
    GN_TRY(ivf_plan(T, nq, np, S.nc, S.list_off.as<int64_t>(), rc, TC_QCHUNK, st, 1));
    const int64_t npairs = nq * np;
    const int64_t qb_rows = std::max<int64_t>(npairs, 256);  // >= one 256-row TMA box
    GN_TRY(S.qb.ensure((size_t)qb_rows * S.K * 2));
    GN_TRY(S.aslot.ensure((size_t)npairs * 8));
    qb_fill_kernel<<<(unsigned)npairs, 128, 0, st>>>(dQ, S.d, S.dp, S.K, np, T.bucket.as<int64_t>(),
                                                     T.boff.as<int64_t>() + S.nc, T.qslot.as<int64_t>(),
                                                     T.slot_rel.as<int64_t>(), S.qb.as<__nv_bfloat16>(),
                                                     S.aslot.as<int64_t>(), npairs);
    const int64_t maxlen = S.top_rows.size() > 1 ? S.top_rows[1] : 0;
    const int64_t max_units = (ceil_div(npairs, TC_QCHUNK) + S.nc) * (ceil_div(maxlen, rc) + 1);
    GN_TRY(S.units.ensure((size_t)max_units * sizeof(TcUnit)));
    GN_TRY(S.nunits.ensure(8));
    tc_units_kernel<<<(unsigned)ceil_div(max_units, 256), 256, 0, st>>>(
        T.item_off.as<int64_t>(), S.nc, T.boff.as<int64_t>(), S.list_off.as<int64_t>(), rc, max_units,
        S.units.as<TcUnit>(), S.nunits.as<int64_t>());
    // score segments: at most the rows of the np largest lists per query
    const int64_t seg_total = nq * S.top_rows[(size_t)std::min<int64_t>(np, (int64_t)S.top_rows.size() - 1)];
    GN_TRY(S.scores.ensure((size_t)std::max<int64_t>(seg_total, 1) * 4));
    TcIvfLaunch a;
    a.X = S.x16.p;
    a.x_rows = std::max<int64_t>(S.n, 256);
    a.Q = S.qb.p;
    a.q_rows = qb_rows;
    a.K = S.K;
    a.units = S.units.as<TcUnit>();
    a.n_units = S.nunits.as<int64_t>();
    a.xnorm = S.vnorm.as<float>();
    a.aslot = S.aslot.as<int64_t>();
    a.scores = S.scores.as<float>();
    a.err = S.err.as<int>();
    a.grid = dev_info().num_sms;
    timing_begin(st, "tc_ivf_kernel");
    GN_TRY(tc_ivf_launch(a, st));
    timing_end(st);
    // warps per query: enough warps in flight for small batches
    int W = 1;
    while (W < 16 && nq * W * 2 <= (int64_t)dev_info().num_sms * 32) W *= 2;
    const int qpb = std::max(1, 8 / W);
    const int threads = 32 * W * qpb;
    const unsigned blocks = (unsigned)ceil_div(nq, qpb);
    auto sel = [&](auto RC) {
        constexpr int R = decltype(RC)::value;
        const size_t smem = W > 1 ? (size_t)(threads / 32) * 32 * R * 8 : 0;
        ivf_tc_select_kernel<R><<<blocks, threads, smem, st>>>(
            S.scores.as<float>(), T.probes.as<int32_t>(), np, T.qslot.as<int64_t>(), T.slot_rel.as<int64_t>(),
            S.list_off.as<int64_t>(), S.shortlist, dQ, S.vecs.as<float>(), S.d, S.dp, S.ids.as<int32_t>(), nq, k, W,
            d_idx, d_dist, d_cnt);
    };
    if (S.shortlist <= 32) sel(std::integral_constant<int, 1>());
    else sel(std::integral_constant<int, 2>());
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

}  // namespace gn

using namespace gn;

extern "C" int gn_ivfl2_set_mode(gn_index *ix, int32_t mode, int32_t shortlist) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    if (mode != 0 && mode != 1) return fail(GN_ERR_INVALID, "mode must be 0 (FP32 scan) or 1 (tensor-core shortlist)");
    if (mode == 1 && shortlist != 16 && shortlist != 32 && shortlist != 40 && shortlist != 64)
        return fail(GN_ERR_INVALID, "shortlist must be 16, 32, 40 or 64");
    std::lock_guard<std::mutex> lk(ix->mu);
    ix->ivfl2->mode = mode;
    if (mode == 1) ix->ivfl2->shortlist = shortlist;
    return GN_OK;
}

extern "C" int gn_ivfl2_error(gn_index *ix, int32_t *err_out) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    int herr = 0;
    if (ix->ivfl2->err.p) GN_CUDA_TRY(cudaMemcpy(&herr, ix->ivfl2->err.p, 4, cudaMemcpyDeviceToHost));
    if (err_out) *err_out = herr;
    return GN_OK;
}

// Work of the last search (benchmark accounting; computed on demand):
// out[0] (query, probe) pairs, out[1] scored (pair, row) entries, out[2] rows
// of the distinct lists probed, out[3] tensor-core work units.
extern "C" int gn_ivfl2_last_work(gn_index *ix, int64_t *out) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    IvfL2State &S = *ix->ivfl2;
    IvfScratch &T = S.s;
    std::lock_guard<std::mutex> lk(ix->mu);
    if (!T.bcnt.p || S.nc == 0) return fail(GN_ERR_INVALID, "no search has run");
    std::vector<int32_t> cnt((size_t)S.nc);
    GN_CUDA_TRY(cudaMemcpy(cnt.data(), T.bcnt.p, (size_t)S.nc * 4, cudaMemcpyDeviceToHost));
    int64_t pairs = 0, scored = 0, rows = 0;
    for (int32_t l = 0; l < S.nc; ++l) {
        const int64_t len = S.h_off[(size_t)l + 1] - S.h_off[(size_t)l];
        pairs += cnt[(size_t)l];
        scored += (int64_t)cnt[(size_t)l] * len;
        if (cnt[(size_t)l] > 0) rows += len;
    }
    int64_t units = 0;
    if (S.mode == 1 && S.nunits.p) GN_CUDA_TRY(cudaMemcpy(&units, S.nunits.p, 8, cudaMemcpyDeviceToHost));
    out[0] = pairs;
    out[1] = scored;
    out[2] = rows;
    out[3] = units;
    return GN_OK;
}
