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
#include "prober.cuh"
#include "flat_scan.cuh"
#include "tc_ivf.cuh"
#include "tc_scan.cuh"
#include "timing.cuh"
#include "gemm_topk.cuh"
#include "topk.cuh"

namespace gn {

constexpr int TC_QCHUNK = 256;  // queries per tensor-core work unit (MMA N <= 256)

// Qb row pos = BF16 row of the query of the pair bucket[pos]; warp per row.
__global__ void qb_fill_kernel(const uint4 *__restrict__ q16, int K8, int np, const int64_t *__restrict__ bucket,
                               const int64_t *__restrict__ boff_end, const int64_t *__restrict__ qslot,
                               const int64_t *__restrict__ slot_rel, uint4 *__restrict__ qb,
                               int64_t *__restrict__ aslot, int64_t max_pairs) {
    const int lane = threadIdx.x & 31;
    const int64_t pos = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (pos >= max_pairs || pos >= *boff_end) return;
    const int64_t pair = bucket[pos];
    const int64_t q = pair / np;
    for (int j = lane; j < K8; j += 32) qb[pos * K8 + j] = q16[q * K8 + j];
    if (lane == 0) aslot[pos] = qslot[q] + slot_rel[pair];
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
        int64_t blk = 0;  // running index of 256-score blocks over the query's segments
        for (int p0 = 0; p0 < np; p0 += 32) {
            // lane p holds probe p0 + p's list start, length and score segment
            const int p = p0 + lane;
            int64_t m_lb = 0, m_len = 0;
            const float *m_sc = nullptr;
            if (p < np) {
                const int64_t pair = q * np + p;
                const int32_t l = probes[pair];
                if (l >= 0) {
                    m_lb = list_off[l];
                    m_len = list_off[l + 1] - m_lb;
                    m_sc = scores + qseg[q] + seg_rel[pair];
                }
            }
            const int cnt = min(32, np - p0);
            for (int pp = 0; pp < cnt; ++pp) {
                const int64_t len = __shfl_sync(0xffffffffu, m_len, pp);
                if (len == 0) continue;
                const int64_t lb = __shfl_sync(0xffffffffu, m_lb, pp);
                const float *sc = reinterpret_cast<const float *>(
                    __shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(m_sc), pp));
                const int nblk = (int)((len + 255) / 256);
                const int ilen = (int)len;
                const int b0 = (int)((wq - blk % W + W) % W);  // first block of this segment owned by warp wq
                for (int b = b0; b < nblk; b += W) {
                    const int i0 = b * 256 + lane;
                    float v[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) v[u] = (i0 + u * 32 < ilen) ? __ldg(sc + i0 + u * 32) : INF;
                    float m = v[0];
#pragma unroll
                    for (int u = 1; u < 8; ++u) m = fminf(m, v[u]);
                    if (!__any_sync(0xffffffffu, m <= thr_f)) continue;
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const int i = i0 + u * 32;
                        const uint64_t key = (i < ilen) ? make_key(f2ord(v[u]), (uint32_t)(lb + i)) : KEY_EMPTY;
                        L.offer(key, thr, S);
                        thr_f = (thr == KEY_EMPTY) ? INF : ord2f(key_dist(thr));
                    }
                }
                blk += nblk;
            }
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

// ── tensor-core coarse stage ──────────────────────────────────────────────
// Units of the centroid scan: every query chunk of 256 against every chunk of
// 128 centroids; aslot[q] = q * nc so the scores land row-major [nq x nc].
__global__ void coarse_units_kernel(int64_t nq, int nc, TcUnit *__restrict__ units, int64_t *__restrict__ n_units,
                                    int64_t *__restrict__ aslot) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nqc = (nq + 255) / 256, ncc = (nc + 127) / 128;
    if (t == 0) *n_units = nqc * ncc;
    if (t < nq) aslot[t] = t * nc;
    if (t >= nqc * ncc) return;
    const int64_t qc = t / ncc, cc = t % ncc;
    TcUnit u;
    u.a0 = qc * 256;
    u.na = (int32_t)min((int64_t)256, nq - u.a0);
    u.r0 = cc * 128;
    u.r1 = min((int64_t)nc, u.r0 + 128);
    u.rbase = 0;
    u.rch = 0;
    units[t] = u;
}

constexpr int PROBE_MAX_D = 2048;  // query row staged in shared memory

// Per query (block of 256 threads): the 64 best centroids by BF16 score, their
// exact squared distances (FP32), sorted nearest first; then either the first
// np of them (fixed probing) or the learned prober's choice (MLP fused here).
template <bool MLP>
__global__ void __launch_bounds__(256) coarse_probe_kernel(const float *__restrict__ scores, int nc, int ncp2,
                                                           const float *__restrict__ Q, int d, int dp,
                                                           const float *__restrict__ C, int64_t nq, int np,
                                                           ProberWeights w, float logit_tau,
                                                           int32_t *__restrict__ probes,
                                                           int32_t *__restrict__ nprobed) {
    constexpr int NC = PROBER_CAND, H = PROBER_HIDDEN;
    __shared__ int32_t sc[NC];
    __shared__ float sd[NC], sf[NC], sh1[H], sh2[H], sz[NC];
    __shared__ int s_cnt0;
    __shared__ __align__(16) float sqr[PROBE_MAX_D];
    extern __shared__ uint64_t skeys[];  // next_pow2(nc) keys
    const int64_t q = blockIdx.x;
    const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
    const float *sq = scores + q * nc;
    for (int t = j; t < d; t += 256) sqr[t] = Q[q * dp + t];
    // block-wide bitonic sort of the BF16 scores; the first 64 are the candidates
    for (int c = j; c < ncp2; c += 256) skeys[c] = c < nc ? make_key(f2ord(sq[c]), (uint32_t)c) : KEY_EMPTY;
    __syncthreads();
    for (int size = 2; size <= ncp2; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = j; i < ncp2 / 2; i += 256) {
                const int lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
                const bool up = (lo & size) == 0;
                const uint64_t a = skeys[lo], b = skeys[hi];
                if ((a > b) == up) { skeys[lo] = b; skeys[hi] = a; }
            }
            __syncthreads();
        }
    if (j < NC) sc[j] = skeys[j] == KEY_EMPTY ? -1 : (int32_t)key_idx(skeys[j]);
    __syncthreads();
    {   // exact squared distances: 4 threads per candidate, float4 strides
        const int i = j >> 2, part = j & 3;
        const int c = sc[i];
        float s0 = 0.f, s1 = 0.f;
        if (c >= 0) {
            const float4 *cr = reinterpret_cast<const float4 *>(C + (int64_t)c * dp);
            const float4 *qr = reinterpret_cast<const float4 *>(sqr);
            const int n4 = d >> 2;
#pragma unroll 4
            for (int t = part; t < n4; t += 8) {
                const float4 a = __ldg(cr + t), b = qr[t];
                float e0 = b.x - a.x, e1 = b.y - a.y, e2 = b.z - a.z, e3 = b.w - a.w;
                s0 = fmaf(e0, e0, s0); s1 = fmaf(e1, e1, s1); s0 = fmaf(e2, e2, s0); s1 = fmaf(e3, e3, s1);
                if (t + 4 < n4) {
                    const float4 a2 = __ldg(cr + t + 4), b2 = qr[t + 4];
                    e0 = b2.x - a2.x; e1 = b2.y - a2.y; e2 = b2.z - a2.z; e3 = b2.w - a2.w;
                    s0 = fmaf(e0, e0, s0); s1 = fmaf(e1, e1, s1); s0 = fmaf(e2, e2, s0); s1 = fmaf(e3, e3, s1);
                }
            }
            for (int t = (n4 << 2) + part; t < d; t += 4) {  // d % 4 tail
                const float e = sqr[t] - C[(int64_t)c * dp + t];
                s0 = fmaf(e, e, s0);
            }
        }
        float s = s0 + s1;
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (part == 0) sd[i] = s;
    }
    __syncthreads();
    if (j < NC) skeys[j] = sc[j] >= 0 ? make_key(__float_as_uint(sd[j]), (uint32_t)sc[j]) : KEY_EMPTY;
    __syncthreads();
    for (int size = 2; size <= NC; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (j < NC / 2) {
                const int lo = 2 * j - (j & (stride - 1)), hi = lo + stride;
                const bool up = (lo & size) == 0;
                const uint64_t a = skeys[lo], b = skeys[hi];
                if ((a > b) == up) { skeys[lo] = b; skeys[hi] = a; }
            }
            __syncthreads();
        }
    if (j < NC) {
        const uint64_t k = skeys[j];
        const bool e = k == KEY_EMPTY;
        const float d1 = __uint_as_float(key_dist(skeys[0]));
        sc[j] = e ? -1 : (int32_t)key_idx(k);
        sf[j] = e ? 0.f : fmaxf(0.f, 1.f - (__uint_as_float(key_dist(k)) - d1) / fmaxf(d1, 1e-12f));
    }
    __syncthreads();
    if (!MLP) {
        if (j < np) probes[q * np + j] = sc[j];
        return;
    }
    const __nv_bfloat16 *W1 = reinterpret_cast<const __nv_bfloat16 *>(w.W1);
    const __nv_bfloat16 *W2 = reinterpret_cast<const __nv_bfloat16 *>(w.W2);
    const __nv_bfloat16 *W3 = reinterpret_cast<const __nv_bfloat16 *>(w.W3);
    float a = w.b1[j];
    for (int i = 0; i < NC; ++i)
        if (sc[i] >= 0) a = fmaf(sf[i], __bfloat162float(W1[(size_t)sc[i] * H + j]), a);
    sh1[j] = fmaxf(a, 0.f);
    __syncthreads();
    for (int o = warp * 32; o < warp * 32 + 32; ++o) {
        float s = 0.f;
#pragma unroll
        for (int k = lane; k < H; k += 32) s = fmaf(__bfloat162float(W2[(size_t)o * H + k]), sh1[k], s);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) sh2[o] = fmaxf(s + w.b2[o], 0.f);
    }
    __syncthreads();
    for (int i = warp; i < NC; i += 8) {
        const int c = sc[i];
        float s = 0.f;
        if (c >= 0) {
#pragma unroll
            for (int k = lane; k < H; k += 32) s = fmaf(__bfloat162float(W3[(size_t)c * H + k]), sh2[k], s);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        }
        if (lane == 0) sz[i] = c >= 0 ? s + w.b3[c] : -INFINITY;
    }
    __syncthreads();
    bool keep = false;
    unsigned m = 0;
    const int i = warp * 32 + lane;
    if (warp < NC / 32) {
        keep = sc[i] >= 0 && (i == 0 || sz[i] >= logit_tau);
        m = __ballot_sync(0xffffffffu, keep);
        if (warp == 0 && lane == 0) s_cnt0 = __popc(m);
    }
    __syncthreads();
    if (warp < NC / 32) {
        const int pos = (warp == 0 ? 0 : s_cnt0) + __popc(m & ((1u << lane) - 1u));
        if (keep) probes[q * NC + pos] = sc[i];
        if (warp == 1) {
            const int total = s_cnt0 + __popc(m);
            for (int t = total + lane; t < NC; t += 32) probes[q * NC + t] = -1;
            if (lane == 0 && nprobed) nprobed[q] = total;
        }
    }
}

// Probes of the tensor-core engine: BF16 centroid scores on the tensor cores,
// exact re-rank of the 64 best, then fixed n_probe or the learned prober.
static int ivfl2_probes_tc(gn_index *ix, const float *dQ, int64_t nq, int *np_out, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    IvfScratch &T = S.s;
    if (S.nc < PROBER_CAND || S.d > PROBE_MAX_D || S.nc > 8192) {  // outside the 64-candidate stage's limits
        if (S.prober) return fail(GN_ERR_INVALID, "learned probing needs at least 64 lists");
        int np = std::min<int32_t>(S.nprobe, S.nc);
        *np_out = np;
        return ivfl2_coarse(ix, dQ, nq, np, st);
    }
    const bool mlp = S.prober != nullptr;
    const int np = mlp ? PROBER_CAND : std::min<int32_t>(std::min<int32_t>(S.nprobe, S.nc), PROBER_CAND);
    if (!mlp && S.nprobe > PROBER_CAND) {  // wider fixed probing: the FP32 coarse stage
        *np_out = std::min<int32_t>(S.nprobe, S.nc);
        return ivfl2_coarse(ix, dQ, nq, *np_out, st);
    }
    *np_out = np;
    const int64_t units = ceil_div(nq, 256) * ceil_div(S.nc, 128);
    GN_TRY(S.cunits.ensure((size_t)units * sizeof(TcUnit)));
    GN_TRY(S.cnunits.ensure(8));
    GN_TRY(S.caslot.ensure((size_t)nq * 8));
    GN_TRY(S.cscores.ensure((size_t)nq * S.nc * 4));
    GN_TRY(T.probes.ensure((size_t)nq * np * 4));
    coarse_units_kernel<<<(unsigned)ceil_div(std::max<int64_t>(units, nq), 256), 256, 0, st>>>(
        nq, S.nc, S.cunits.as<TcUnit>(), S.cnunits.as<int64_t>(), S.caslot.as<int64_t>());
    TcIvfLaunch a;
    a.X = S.c16.p;
    a.x_rows = std::max<int64_t>(S.nc, 128);
    a.Q = S.q16.p;
    a.q_rows = std::max<int64_t>(nq, 256);
    a.K = S.K;
    a.units = S.cunits.as<TcUnit>();
    a.n_units = S.cnunits.as<int64_t>();
    a.xnorm = S.cnorm.as<float>();
    a.aslot = S.caslot.as<int64_t>();
    a.scores = S.cscores.as<float>();
    a.err = S.err.as<int>();
    a.grid = (int)std::min<int64_t>(dev_info().num_sms, units);
    GN_TRY(tc_ivf_launch(a, st));
    const int ncp2 = (int)next_pow2(S.nc);
    const size_t ksm = (size_t)ncp2 * 8;
    if (ksm > 48 * 1024) {
        GN_CUDA_TRY(cudaFuncSetAttribute(coarse_probe_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ksm));
        GN_CUDA_TRY(cudaFuncSetAttribute(coarse_probe_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ksm));
    }
    ProberWeights w;
    if (mlp) {
        GN_TRY(prober_weights(S.prober, &w));
        GN_TRY(T.nprobed.ensure((size_t)nq * 4));
        coarse_probe_kernel<true><<<(unsigned)nq, 256, ksm, st>>>(S.cscores.as<float>(), S.nc, ncp2, dQ, S.d, S.dp,
                                                               S.cent.as<float>(), nq, np, w, S.prober_tau,
                                                               T.probes.as<int32_t>(), T.nprobed.as<int32_t>());
    } else {
        coarse_probe_kernel<false><<<(unsigned)nq, 256, ksm, st>>>(S.cscores.as<float>(), S.nc, ncp2, dQ, S.d, S.dp,
                                                                S.cent.as<float>(), nq, np, w, 0.f,
                                                                T.probes.as<int32_t>(), nullptr);
    }
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

int ivfl2_prepare_tc(gn_index *ix, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    S.K = (int)round_up(S.d, 64);
    const int64_t rows = std::max<int64_t>(S.n, 256);  // at least one 256-row TMA box
    GN_TRY(S.x16.ensure((size_t)rows * S.K * 2));
    GN_CUDA_TRY(cudaMemsetAsync(S.x16.p, 0, (size_t)rows * S.K * 2, st));
    to_bf16_rows(S.vecs.as<float>(), S.n, S.d, S.dp, S.x16.p, S.K, st);
    const int64_t crows = std::max<int64_t>(S.nc, 128);  // at least one 128-row TMA box
    GN_TRY(S.c16.ensure((size_t)crows * S.K * 2));
    GN_CUDA_TRY(cudaMemsetAsync(S.c16.p, 0, (size_t)crows * S.K * 2, st));
    to_bf16_rows(S.cent.as<float>(), S.nc, S.d, S.dp, S.c16.p, S.K, st);
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
    GN_TRY(S.q16.ensure((size_t)std::max<int64_t>(nq, 256) * S.K * 2));
    to_bf16_rows(dQ, nq, S.d, S.dp, S.q16.p, S.K, st);
    int np = 1;
    GN_TRY(ivfl2_probes_tc(ix, dQ, nq, &np, st));
    // work items of rc rows (short items for small batches so that their few
    // lists still spread over all SMs); every pair owns a score segment
    const int rc = nq >= 512 ? S.rc_tc : (nq >= 64 ? 1024 : 256);
    GN_TRY(ivf_plan(T, nq, np, S.nc, S.list_off.as<int64_t>(), rc, TC_QCHUNK, st, 1));
    const int64_t npairs = nq * np;
    const int64_t qb_rows = std::max<int64_t>(npairs, 256);  // >= one 256-row TMA box
    GN_TRY(S.qb.ensure((size_t)qb_rows * S.K * 2));
    GN_TRY(S.aslot.ensure((size_t)npairs * 8));
    qb_fill_kernel<<<(unsigned)ceil_div(npairs, 8), 256, 0, st>>>(
        S.q16.as<uint4>(), S.K / 8, np, T.bucket.as<int64_t>(), T.boff.as<int64_t>() + S.nc, T.qslot.as<int64_t>(),
        T.slot_rel.as<int64_t>(), S.qb.as<uint4>(), S.aslot.as<int64_t>(), npairs);
    const int64_t maxlen = S.top_rows.size() > 1 ? S.top_rows[1] : 0;
    // sized for the shortest row chunk (256) so that a smaller batch never needs more
    const int64_t max_units = (ceil_div(npairs, TC_QCHUNK) + S.nc) * (ceil_div(maxlen, 256) + 1);
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
    while (W < 16 && nq * W <= (int64_t)dev_info().num_sms * 64) W *= 2;
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
    ix->ivfl2->cfg++;
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
