// ivf_tc.cu — tensor-core engine of the float IVF index.
//
//   0. probes  coarse_probe_kernel: BF16 centroid scores (tc_ivf_kernel over
//              the centroids), radix select of the 64 best, exact FP32
//              distances, then the first n_probe or the learned prober's
//              choice (its MLP fused here; from 1,024 queries its layers 2
//              and 3 run in mlp_probe_kernel over 8 queries per block), and
//              each query's score bound for the scan;
//   1. plan    the same bucketing and work plan as the FP32 scan (ivf.cu),
//              score segments in 128-row slots;
//   2. Qb      the BF16 copy of each (query, probe) pair's query, rows grouped by
//              list (bucket order), so one TMA box covers a work unit's queries;
//   3. units   one tensor-core work unit per (list, row chunk, 128-query chunk);
//   4. scan    tc_ivf_kernel: BF16 tcgen05 GEMM of the list's rows (M = 128
//              per tile) against the unit's queries (N = 32..128) with FP32
//              accumulation; the minimum score |x|^2 - 2 q.x (exact FP32
//              |x|^2) of every 32-row quarter goes to the slot's four minima,
//              and the quarter's scores to the pair's slots when that minimum
//              is within the query's bound;
//   5. select  per query: a threshold from the quarter minima, only the
//              quarters below it are read, the S best keys (S = shortlist) by
//              radix select, their squared L2 recomputed exactly in FP32 with a
//              compensated sum, the k nearest returned, ties to the lower
//              original index.
// Work units are short (a list holds ~1k rows), so selection is kept out of
// the tensor-core kernel: a per-unit top-S would pay its warm-up on every
// unit.  Everything stays on the device; the batch has no host round trip.
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

constexpr int TC_QCHUNK = 128;  // queries per tensor-core work unit (MMA N <= 128)

__device__ __forceinline__ int find_list_tc(const int64_t *item_off, int nc, int64_t item) {
    int lo = 0, hi = nc;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (item_off[mid] <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ void tc_units_body(int64_t i, const int64_t *__restrict__ item_off, int nc,
                              const int64_t *__restrict__ boff, const int64_t *__restrict__ list_off,
                              const int64_t *__restrict__ xoff, int rc, int qch, int64_t max_units,
                              TcUnit *__restrict__ units, int64_t *__restrict__ n_units) {
    const int64_t total = item_off[nc];
    if (i == 0) *n_units = min(total, max_units);
    if (i >= total || i >= max_units) return;
    const int l = find_list_tc(item_off, nc, i);
    const int64_t lb = list_off[l], le = list_off[l + 1];
    const int64_t nrc = (le - lb + rc - 1) / rc;
    const int64_t nqc = nrc > 0 ? (item_off[l + 1] - item_off[l]) / nrc : 1;
    const int64_t local = i - item_off[l];
    // the query chunks of one row chunk are adjacent: taken together by
    // different SMs, their second and later reads of the rows hit L2
    const int64_t rch = local / nqc, qc = local % nqc;
    TcUnit u;
    u.a0 = boff[l] + qc * qch;
    u.na = (int32_t)min((int64_t)qch, boff[l + 1] - u.a0);
    u.r0 = lb + rch * rc;
    u.r1 = min(le, u.r0 + rc);
    u.rbase = lb;
    u.xrow = xoff[l] + (u.r0 - lb);  // rc is a multiple of 128: stays tile-aligned
    u.rch = (int32_t)rch;
    units[i] = u;
}

// One launch for both: blocks [0, qb_blocks) fill Qb — row pos = the BF16 row
// of the query of the pair bucket[pos], warp per row, with the pair's slot
// base and its query's score bound — the rest build the work units.
__global__ void qb_units_kernel(const uint4 *__restrict__ q16, int K8, int np, const int64_t *__restrict__ bucket,
                                const int64_t *__restrict__ boff, int nc, const int64_t *__restrict__ qslot,
                                const int64_t *__restrict__ slot_rel, uint4 *__restrict__ qb,
                                int64_t *__restrict__ aslot, const uint32_t *__restrict__ qbound,
                                uint32_t *__restrict__ abound, int64_t max_pairs, unsigned qb_blocks,
                                const int64_t *__restrict__ item_off, const int64_t *__restrict__ list_off,
                                const int64_t *__restrict__ xoff, int rc, int qch, int64_t max_units,
                                TcUnit *__restrict__ units, int64_t *__restrict__ n_units) {
    if (blockIdx.x < qb_blocks) {
        const int lane = threadIdx.x & 31;
        const int64_t pos = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
        if (pos >= max_pairs || pos >= boff[nc]) return;
        const int64_t pair = bucket[pos];
        const int64_t q = pair / np;
        for (int j = lane; j < K8; j += 32) qb[pos * K8 + j] = q16[q * K8 + j];
        if (lane == 0) {
            aslot[pos] = qslot[q] + slot_rel[pair];
            abound[pos] = qbound[q];
        }
        return;
    }
    const int64_t i = (int64_t)(blockIdx.x - qb_blocks) * blockDim.x + threadIdx.x;
    tc_units_body(i, item_off, nc, boff, list_off, xoff, rc, qch, max_units, units, n_units);
}


// Two-sum of a and b: s = fl(a + b) and its exact rounding error.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// Compensated accumulation of (a_i - b_i)^2 into (s, c): each square is split
// into its rounded product and the product's exact error (fma), the running
// sum keeps its rounding error (two-sum).
__device__ __forceinline__ void l2_acc4(const float4 a, const float4 b, int valid, float &s, float &c) {
    const float t[4] = {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __fsub_rn(a.w, b.w)};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        if (u < valid) {
            const float p = __fmul_rn(t[u], t[u]);
            const float e = __fmaf_rn(t[u], t[u], -p);
            float s2, err;
            two_sum(s, p, s2, err);
            s = s2;
            c = __fadd_rn(c, __fadd_rn(err, e));
        }
    }
}

// Combine the 32 lanes' (sum, error) pairs with two-sums; the result is
// within about one ulp of the exact sum.
__device__ __forceinline__ float l2_warp_total(float s, float c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float so = __shfl_xor_sync(0xffffffffu, s, o), co = __shfl_xor_sync(0xffffffffu, c, o);
        float s2, err;
        two_sum(s, so, s2, err);
        s = s2;
        c = __fadd_rn(c, __fadd_rn(co, err));
    }
    return __fadd_rn(s, c);
}

// Exact squared L2 (compensated FP32) of the query row q to rows[0..n) of X
// (n <= 2), by one warp: lane l takes columns 4l..4l+3 of every 128-column
// block (coalesced float4 loads, all of a 512-column block issued together).
__device__ __forceinline__ void l2sq_warp_rows(const float *__restrict__ q, const float *__restrict__ X, int dp,
                                               int d, const int64_t *rows, int n, float *out, int lane) {
    float s[2] = {0.f, 0.f}, c[2] = {0.f, 0.f};
    for (int base = 0; base < d; base += 512) {
        float4 qa[4], xa[2][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i0 = base + u * 128 + lane * 4;
            qa[u] = i0 < d ? *reinterpret_cast<const float4 *>(q + i0) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int r = 0; r < 2; ++r)
                xa[r][u] = (r < n && i0 < d) ? __ldg(reinterpret_cast<const float4 *>(X + rows[r] * dp + i0))
                                             : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i0 = base + u * 128 + lane * 4;
            const int valid = min(4, d - i0);
#pragma unroll
            for (int r = 0; r < 2; ++r)
                if (r < n) l2_acc4(qa[u], xa[r][u], valid, s[r], c[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < 2; ++r)
        if (r < n) out[r] = l2_warp_total(s[r], c[r]);
}

constexpr int SEL_PCH = 256;   // probes staged per pass
constexpr int SEL_WB = 512;    // candidate keys buffered per warp
constexpr int SEL_QCAP = 256;  // qualifying quarters listed from the threshold's staged minima

// Ascending bitonic sort of n (power of two, <= 512) keys in shared memory by
// one warp.
__device__ __forceinline__ void warp_bitonic_sort(uint64_t *a, int n, int lane) {
    for (int size = 2; size <= n; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = lane; i < (n >> 1); i += 32) {
                const int lo = 2 * i - (i & (stride - 1)), hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const uint64_t x = a[lo], y = a[hi];
                if ((x > y) == asc) {
                    a[lo] = y;
                    a[hi] = x;
                }
            }
            __syncwarp();
        }
}

// The S smallest of a key multiset held in shared memory, by the whole block
// (radix select on 8-bit digits from the top, stopping as soon as the
// boundary digit is taken whole).  The keys are keys[w * WB + i], i < cnt[w],
// one region per warp (warp w reads region w).  The S smallest (all, if
// fewer) go to out[], in no particular order; returns how many.  Keys are
// unique, so exactly min(S, total) are selected.
template <int NT>
__device__ int block_radix_select(const uint64_t *keys, int WB, const int *cnt, int S, uint64_t *out, int *hist,
                                  int *sh) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint64_t *mine = keys + (size_t)warp * WB;
    const int nmine = cnt[warp];
    uint64_t prefix = 0, mask = 0;
    int need = S;
    bool all = false;  // keys matching the prefix are all taken
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int i = t; i < 256; i += NT) hist[i] = 0;
        __syncthreads();
        for (int i = lane; i < nmine; i += 32) {
            const uint64_t k = mine[i];
            if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255], 1);
        }
        __syncthreads();
        if (warp == 0) {
            int h[8], sum = 0;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                h[e] = hist[lane * 8 + e];
                sum += h[e];
            }
            int inc = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            int before = inc - sum;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                if (before < need && need <= before + h[e]) {
                    sh[0] = lane * 8 + e;
                    sh[1] = before;
                }
                before += h[e];
            }
            if (lane == 31) sh[2] = inc;  // keys matching the prefix
        }
        __syncthreads();
        if (shift == 56 && sh[2] <= S) {  // no more keys than S: take them all
            all = true;
            break;
        }
        const int dg = sh[0];
        need -= sh[1];
        prefix |= (uint64_t)dg << shift;
        mask |= (uint64_t)0xff << shift;
        const bool whole = hist[dg] == need;
        __syncthreads();
        if (whole) {
            all = true;
            break;
        }
    }
    // take every key below the prefix and the keys equal to it (all of them,
    // or the single key left after all eight digits)
    if (t == 0) sh[3] = 0;
    __syncthreads();
    for (int i = lane; i < nmine; i += 32) {
        const uint64_t k = mine[i];
        const uint64_t km = k & mask;
        if (km < prefix || (km == prefix && (all || need > 0))) out[atomicAdd(&sh[3], 1)] = k;
    }
    __syncthreads();
    return sh[3];
}

// k-th smallest (1-based) of n unsigned values in shared memory, by the whole
// block (radix select on 8-bit digits); all ones if n < kth.
template <int NT>
__device__ uint32_t block_kth_u32(const uint32_t *v, int n, int kth, int *hist, int *sh) {
    if (n < kth) return 0xffffffffu;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t prefix = 0, mask = 0;
    int need = kth;
    for (int shift = 24; shift >= 0; shift -= 8) {
        for (int i = t; i < 256; i += NT) hist[i] = 0;
        __syncthreads();
        for (int i = t; i < n; i += NT) {
            const uint32_t x = v[i];
            if ((x & mask) == prefix) atomicAdd(&hist[(x >> shift) & 255], 1);
        }
        __syncthreads();
        if (warp == 0) {
            int h[8], sum = 0;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                h[e] = hist[lane * 8 + e];
                sum += h[e];
            }
            int inc = sum;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int x = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += x;
            }
            int before = inc - sum;
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                if (before < need && need <= before + h[e]) {
                    sh[0] = lane * 8 + e;
                    sh[1] = before;
                }
                before += h[e];
            }
        }
        __syncthreads();
        prefix |= (uint32_t)sh[0] << shift;
        mask |= 0xffu << shift;
        need -= sh[1];
        __syncthreads();
    }
    return prefix;
}

// Offer each lane's key (want: it is a real row) to the warp's shared-memory
// buffer W of SEL_WB keys (wn keys held, warp-uniform): keys below the warp
// threshold are appended; a full buffer is sorted and cut to its best S, its
// S-th key becoming the new threshold, and the keys that did not fit are
// offered again.
__device__ __forceinline__ void sel_buffer_offer(uint64_t key, bool want, uint64_t *W, int &wn, uint64_t &wthr,
                                                 int S, int lane) {
    bool w = want && key < wthr;
    while (true) {
        const unsigned b2 = __ballot_sync(0xffffffffu, w);
        if (!b2) break;
        const int pos = wn + __popc(b2 & ((1u << lane) - 1u));
        if (w && pos < SEL_WB) {
            W[pos] = key;
            w = false;
        }
        wn += __popc(b2);
        if (wn <= SEL_WB) break;
        __syncwarp();
        warp_bitonic_sort(W, SEL_WB, lane);
        wthr = W[S - 1];
        wn = S;
        w = w && key < wthr;
        __syncwarp();
    }
}

// Selection of one query by B blocks of NT threads (B = 1 for large batches;
// small batches split each query's range over up to 16 blocks, whose partial
// best-S lists the last block to finish merges).  The list scan leaves, per
// (query, list) pair, the scores of the list's rows in 128-row slots and the
// minimum score of every 32-row quarter of every slot.  Keys are (score, row),
// so ties go to the lower row.
//   threshold  tau = the S-th smallest quarter minimum of the block's slots
//              (radix select): S distinct rows score <= tau, so tau bounds the
//              query's S-th best score; tau is capped by the query's bound
//              from the probe stage, above which the scan stored no quarter;
//   sweep      the quarters whose minimum is <= tau, listed from the minima
//              staged for the threshold (typically a few dozen of the query's
//              hundreds of slots), are read four per warp at a time (one
//              coalesced 128-byte load each); slots beyond the staged ones are
//              swept 8 at a time (lane l: quarter l % 4 of slot l / 4);
//   buffer     scores <= tau become keys in the warp's shared-memory buffer
//              (512 keys); a full buffer is sorted and cut to its best S;
//   select     radix select of the S smallest keys of all warps' buffers;
//   re-rank    two rows per warp at a time: exact squared L2 in FP32
//              (compensated sum); warp 0 returns the k nearest, ties to the
//              lower original index.
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) ivf_tc_select_kernel(
    const float *__restrict__ scores, const uint4 *__restrict__ tmin4, const uint32_t *__restrict__ qbound,
    const int32_t *__restrict__ probes, int np,
    const int64_t *__restrict__ qseg, const int64_t *__restrict__ seg_rel, const int64_t *__restrict__ list_off,
    int S, const float *__restrict__ Q, const float *__restrict__ X, int d, int dp, const int32_t *__restrict__ ids,
    int64_t nq, int k, int B, uint64_t *__restrict__ part, int *__restrict__ done, int64_t *__restrict__ out_idx,
    float *__restrict__ out_dist, int64_t *__restrict__ out_cnt) {
    constexpr int NW = NT / 32;
    __shared__ uint64_t wreg[NW * SEL_WB];
    __shared__ int64_t p_slot[SEL_PCH], p_lb[SEL_PCH], p_len[SEL_PCH], p_tpre[SEL_PCH + 1];
    __shared__ int64_t w_sum[NW];
    __shared__ uint64_t sel[64], s_rk[64];
    __shared__ int hist[256], sh[4], s_wn[NW];
    __shared__ int s_last, s_qn;
    __shared__ int32_t qlist[SEL_QCAP];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int64_t q = blockIdx.x / B;
    const int bq = (int)(blockIdx.x % B);  // this block's share of the query's slots (B > 1 needs np <= SEL_PCH)
    uint64_t *W = wreg + warp * SEL_WB;
    int wn = 0;                 // keys in this warp's buffer (warp-uniform)
    uint64_t wthr = KEY_EMPTY;  // this warp's threshold (its S-th best key after a cut)
    uint32_t tau = 0xffffffffu;

    for (int p0 = 0; p0 < np; p0 += SEL_PCH) {
        int64_t sweep_lo;  // first slot of this pass the sweep reads minima for
        const int pc = min(SEL_PCH, np - p0);
        // per-probe metadata and the prefix sum of the slot counts
        int64_t nslot = 0;
        if (t < pc) {
            const int64_t pair = q * np + p0 + t;
            const int32_t l = probes[pair];
            p_lb[t] = 0;
            p_len[t] = 0;
            p_slot[t] = 0;
            if (l >= 0) {
                p_lb[t] = list_off[l];
                p_len[t] = list_off[l + 1] - p_lb[t];
                p_slot[t] = qseg[q] + seg_rel[pair];
                nslot = (p_len[t] + 127) >> 7;
            }
        }
        int64_t inc = nslot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) w_sum[warp] = inc;
        __syncthreads();
        int64_t before = 0;
        for (int w = 0; w < warp; ++w) before += w_sum[w];
        if (t < pc) p_tpre[t + 1] = before + inc;
        if (t == 0) p_tpre[0] = 0;
        __syncthreads();
        const int64_t all = p_tpre[pc];
        // parts actually used: at least 2S slots each, so that every part's
        // threshold comes from enough slot minima (idle parts publish nothing)
        const int bu = (int)max((int64_t)1, min((int64_t)B, all / (2 * S)));
        const int64_t lo = bq < bu ? all * bq / bu : all, hi = bq < bu ? all * (bq + 1) / bu : all;
        sweep_lo = lo;
        if (p0 == 0) {
            // threshold from the quarter minima of the block's first slots (any
            // S of them are S distinct rows' scores, so they bound it)
            uint32_t *tm = reinterpret_cast<uint32_t *>(wreg);
            const int ns = (int)min(hi - lo, (int64_t)NW * SEL_WB / 2);
            int p = 0;
            for (int i = t; i < ns; i += NT) {
                const int64_t f = lo + i;
                while (p_tpre[p + 1] <= f) ++p;
                const uint4 m = __ldg(tmin4 + p_slot[p] + (f - p_tpre[p]));
                tm[4 * i] = m.x;
                tm[4 * i + 1] = m.y;
                tm[4 * i + 2] = m.z;
                tm[4 * i + 3] = m.w;
            }
            __syncthreads();
            // and never above the query's bound: quarters above it were not stored
            tau = min(block_kth_u32<NT>(tm, 4 * ns, S, hist, sh), qbound[q]);
            wthr = tau == 0xffffffffu ? KEY_EMPTY : make_key(tau, 0xffffffffu);
            // the qualifying quarters among the staged minima, listed (any order)
            if (t == 0) s_qn = 0;
            __syncthreads();
            for (int i = t; i < 4 * ns; i += NT)
                if (tm[i] <= tau) {
                    const int pos = atomicAdd(&s_qn, 1);
                    if (pos < SEL_QCAP) qlist[pos] = i;
                }
            __syncthreads();
            // all of them listed: they are read straight from the list, four
            // quarters per warp at a time with their loads in flight together;
            // the sweep below covers the slots past the staged ones
            if (s_qn <= SEL_QCAP) {
                const int nl = s_qn;
                for (int e0 = warp * 4; e0 < nl; e0 += NW * 4) {
                    const int nb = min(4, nl - e0);
                    uint64_t key[4];
                    bool want[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int idx = u < nb ? qlist[e0 + u] : 0;
                        const int64_t f = lo + (idx >> 2);
                        int a = 0, b = pc;  // probe pp: p_tpre[pp] <= f < p_tpre[pp + 1]
                        while (b - a > 1) {
                            const int mid = (a + b) >> 1;
                            if (p_tpre[mid] <= f) a = mid;
                            else b = mid;
                        }
                        const int64_t slot = f - p_tpre[a];
                        const int i = (idx & 3) * 32 + lane;  // row within the slot
                        const int64_t r0 = slot * 128;
                        const bool ok = u < nb && r0 + i < p_len[a];
                        const uint32_t v = ok ? f2ord(__ldg(scores + (p_slot[a] + slot) * 128 + i)) : 0xffffffffu;
                        key[u] = make_key(v, (uint32_t)(p_lb[a] + r0 + i));
                        want[u] = ok;
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) sel_buffer_offer(key[u], want[u], W, wn, wthr, S, lane);
                }
                sweep_lo = lo + ns;
            }
            __syncthreads();  // the list and the staged minima are done with before the buffers fill
        }
        int p = 0;  // probe of this lane's slot (monotone over the sweep)
        // warp w takes 8 slots at a time: lane l looks at quarter l % 4 of slot g0 + l / 4
        for (int64_t g0 = sweep_lo + (int64_t)warp * 8; g0 < hi; g0 += (int64_t)NW * 8) {
            const int64_t f = g0 + (lane >> 2);
            const int qu = lane & 3;
            bool qual = false;
            if (f < hi) {
                while (p_tpre[p + 1] <= f) ++p;
                qual = __ldg(reinterpret_cast<const uint32_t *>(tmin4 + p_slot[p] + (f - p_tpre[p])) + qu) <= tau;
            }
            unsigned bal = __ballot_sync(0xffffffffu, qual);
            while (bal) {
                // up to four qualifying quarters at a time, their loads in flight together
                int src[4], nb = 0;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    src[u] = bal ? __ffs(bal) - 1 : -1;
                    if (bal) {
                        bal &= bal - 1;
                        ++nb;
                    }
                }
                uint32_t v[4];
                uint64_t key[4];
                bool want[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int sl = src[u] < 0 ? 0 : src[u];
                    const int pp = __shfl_sync(0xffffffffu, p, sl);
                    const int64_t slot = g0 + (sl >> 2) - p_tpre[pp];
                    const int i = (sl & 3) * 32 + lane;  // row within the slot
                    const int64_t r0 = slot * 128;
                    const bool ok = u < nb && r0 + i < p_len[pp];
                    v[u] = ok ? f2ord(__ldg(scores + (p_slot[pp] + slot) * 128 + i)) : 0xffffffffu;
                    key[u] = make_key(v[u], (uint32_t)(p_lb[pp] + r0 + i));
                    want[u] = ok;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) sel_buffer_offer(key[u], want[u], W, wn, wthr, S, lane);
            }
        }
        __syncthreads();
    }
    if (lane == 0) s_wn[warp] = wn;
    __syncthreads();
    int m = block_radix_select<NT>(wreg, SEL_WB, s_wn, S, sel, hist, sh);
    if (B > 1) {
        // publish this block's best S; the last block of the query merges all
        uint64_t *mine = part + ((size_t)q * B + bq) * S;
        for (int i = t; i < S; i += NT) mine[i] = i < m ? sel[i] : KEY_EMPTY;
        __threadfence();
        __syncthreads();
        if (t == 0) s_last = atomicAdd(done + q, 1) == B - 1;
        __syncthreads();
        if (!s_last) return;
        __threadfence();
        // block b's list goes to region b mod 8 (at offset (b / 8) * S)
        const uint64_t *all_q = part + (size_t)q * B * S;
        for (int i = t; i < B * S; i += NT) {
            const int b = i / S;
            wreg[(b % NW) * SEL_WB + (b / NW) * S + i % S] = __ldcg(all_q + i);
        }
        if (t < NW) s_wn[t] = ((B - t + NW - 1) / NW) * S;
        if (t == 0) done[q] = 0;  // ready for the next batch
        __syncthreads();
        m = block_radix_select<NT>(wreg, SEL_WB, s_wn, S, sel, hist, sh);
    }

    // exact re-rank of the candidates, two rows per warp at a time; first every
    // thread prefetches a share of all candidate rows' 128-byte lines into L2,
    // so that the warps' row loads do not each wait a full DRAM round trip
    const float *qrow = Q + q * dp;
    {
        const int lines = (d * 4 + 127) / 128, nc = min(m, S);
        for (int i = t; i < nc * lines; i += NT) {
            const uint64_t c = sel[i / lines];
            if (c != KEY_EMPTY)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(X + (int64_t)key_idx(c) * dp + (i % lines) * 32));
        }
    }
    for (int r = 2 * warp; r < S; r += 2 * NW) {
        int64_t rows[2];
        int n = 0;
        for (int u = 0; u < 2; ++u) {
            const uint64_t c = (r + u < S && r + u < m) ? sel[r + u] : KEY_EMPTY;
            rows[u] = c != KEY_EMPTY ? (int64_t)key_idx(c) : -1;
        }
        n = rows[0] < 0 ? 0 : (rows[1] < 0 ? 1 : 2);
        if (rows[0] < 0 && rows[1] >= 0) {  // keep the valid row first
            rows[0] = rows[1];
            rows[1] = -1;
            n = 1;
        }
        float dd[2];
        if (n) l2sq_warp_rows(qrow, X, dp, d, rows, n, dd, lane);
        if (lane == 0)
            for (int u = 0; u < 2 && r + u < S; ++u) s_rk[r + u] = KEY_EMPTY;
        __syncwarp();
        if (lane == 0)
            for (int u = 0; u < n; ++u) s_rk[r + u] = make_key(__float_as_uint(dd[u]), (uint32_t)ids[rows[u]]);
    }
    __syncthreads();
    if (warp != 0) return;
    WarpTopK<1> F;
    F.init();
    uint64_t fthr = KEY_EMPTY;
    for (int r0 = 0; r0 < S; r0 += 32) {
        const uint64_t key = (r0 + lane < S) ? s_rk[r0 + lane] : KEY_EMPTY;
        F.offer(key, fthr, k);
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

// Selection of one query per warp (no block barriers; an autotuner option): the
// same keys (score, row), the same S smallest, the same exact re-rank and
// output as ivf_tc_select_kernel.
//   threshold  tau = the S-th smallest quarter minimum of the query's first 64
//              slots (a bitwise select over the warp's 256 values): S distinct
//              rows score <= tau; capped by the query's bound;
//   sweep      the block kernel's warp loop over all the query's slots: 8
//              slots a step, only quarters whose minimum is <= tau are read,
//              their scores <= the warp threshold buffered as keys;
//   select     bitonic sort of the buffer (a full buffer is cut to its best S
//              on the way), the first S keys;
//   re-rank    two rows at a time (rows prefetched into L2 first), then the k
//              nearest, ties to the lower original index.
// Needs np <= 64 probes.
constexpr int SELW_WARPS = 4;

__global__ void __launch_bounds__(32 * SELW_WARPS) ivf_tc_select_warp_kernel(
    const float *__restrict__ scores, const uint4 *__restrict__ tmin4, const uint32_t *__restrict__ qbound,
    const int32_t *__restrict__ probes, int np,
    const int64_t *__restrict__ qseg, const int64_t *__restrict__ seg_rel, const int64_t *__restrict__ list_off,
    int S, const float *__restrict__ Q, const float *__restrict__ X, int d, int dp, const int32_t *__restrict__ ids,
    int64_t nq, int k, int64_t *__restrict__ out_idx, float *__restrict__ out_dist, int64_t *__restrict__ out_cnt) {
    __shared__ uint64_t wreg[SELW_WARPS * SEL_WB];
    __shared__ int64_t w_pre[SELW_WARPS][65], w_lb[SELW_WARPS][64], w_len[SELW_WARPS][64], w_sb[SELW_WARPS][64];
    __shared__ uint64_t w_rk[SELW_WARPS][64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t q = (int64_t)blockIdx.x * SELW_WARPS + warp;
    if (q >= nq) return;  // the whole warp; no block barrier below
    uint64_t *W = wreg + warp * SEL_WB;
    int64_t *pre = w_pre[warp], *plb = w_lb[warp], *plen = w_len[warp], *psb = w_sb[warp];
    // probes: lane l holds probes l and l + 32; the slot counts' prefix sum in probe order
    int64_t ns[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int p = h * 32 + lane;
        ns[h] = 0;
        plb[p] = 0;
        plen[p] = 0;
        psb[p] = 0;
        const int32_t l = p < np ? probes[q * np + p] : -1;
        if (l >= 0) {
            plb[p] = list_off[l];
            plen[p] = list_off[l + 1] - plb[p];
            psb[p] = qseg[q] + seg_rel[q * np + p];
            ns[h] = (plen[p] + 127) >> 7;
        }
    }
    int64_t inc0 = ns[0], inc1 = ns[1];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t a = __shfl_up_sync(0xffffffffu, inc0, o), b = __shfl_up_sync(0xffffffffu, inc1, o);
        if (lane >= o) {
            inc0 += a;
            inc1 += b;
        }
    }
    const int64_t tot0 = __shfl_sync(0xffffffffu, inc0, 31);
    inc1 += tot0;
    pre[lane + 1] = inc0;
    pre[lane + 33] = inc1;
    if (lane == 0) pre[0] = 0;
    __syncwarp();
    const int64_t all = pre[64];
    // threshold from the quarter minima of the first (up to) 64 slots
    uint32_t mv[8];
    const int64_t nfirst = min(all, (int64_t)64);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int64_t f = h * 32 + lane;
        uint4 m4 = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
        if (f < nfirst) {
            int lo = 0, hi = 64;  // the probe whose slots hold f: pre[p] <= f < pre[p + 1]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (pre[mid] <= f) lo = mid;
                else hi = mid;
            }
            m4 = __ldg(tmin4 + psb[lo] + (f - pre[lo]));
        }
        mv[4 * h] = m4.x;
        mv[4 * h + 1] = m4.y;
        mv[4 * h + 2] = m4.z;
        mv[4 * h + 3] = m4.w;
    }
    uint32_t tau = 0xffffffffu;
    if (4 * nfirst >= S) {
        tau = 0;
        for (int b = 31; b >= 0; --b) {
            const uint32_t t = tau | ((1u << b) - 1u);
            int cnt = 0;
#pragma unroll
            for (int u = 0; u < 8; ++u) cnt += __popc(__ballot_sync(0xffffffffu, mv[u] <= t));
            if (cnt < S) tau |= 1u << b;
        }
    }
    tau = min(tau, qbound[q]);  // quarters above the query's bound were not stored
    uint64_t wthr = tau == 0xffffffffu ? KEY_EMPTY : make_key(tau, 0xffffffffu);
    int wn = 0;
    int p = 0;  // probe of this lane's slot (monotone over the sweep)
    for (int64_t g0 = 0; g0 < all; g0 += 8) {
        const int64_t f = g0 + (lane >> 2);
        const int qu = lane & 3;
        bool qual = false;
        if (f < all) {
            while (pre[p + 1] <= f) ++p;
            qual = __ldg(reinterpret_cast<const uint32_t *>(tmin4 + psb[p] + (f - pre[p])) + qu) <= tau;
        }
        unsigned bal = __ballot_sync(0xffffffffu, qual);
        while (bal) {
            // up to four qualifying quarters at a time, their loads in flight together
            int src[4], nb = 0;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                src[u] = bal ? __ffs(bal) - 1 : -1;
                if (bal) {
                    bal &= bal - 1;
                    ++nb;
                }
            }
            uint64_t key[4];
            bool want[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int sl = src[u] < 0 ? 0 : src[u];
                const int pp = __shfl_sync(0xffffffffu, p, sl);
                const int64_t slot = g0 + (sl >> 2) - pre[pp];
                const int i = (sl & 3) * 32 + lane;  // row within the slot
                const int64_t r0 = slot * 128;
                const bool ok = u < nb && r0 + i < plen[pp];
                const uint32_t v = ok ? f2ord(__ldg(scores + (psb[pp] + slot) * 128 + i)) : 0xffffffffu;
                key[u] = make_key(v, (uint32_t)(plb[pp] + r0 + i));
                want[u] = ok;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                bool w = want[u] && key[u] < wthr;
                while (true) {
                    const unsigned b2 = __ballot_sync(0xffffffffu, w);
                    if (!b2) break;
                    const int pos = wn + __popc(b2 & ((1u << lane) - 1u));
                    if (w && pos < SEL_WB) {
                        W[pos] = key[u];
                        w = false;
                    }
                    wn += __popc(b2);
                    if (wn <= SEL_WB) break;
                    // full: keep the best S; keys that did not fit are offered again
                    __syncwarp();
                    warp_bitonic_sort(W, SEL_WB, lane);
                    wthr = W[S - 1];
                    wn = S;
                    w = w && key[u] < wthr;
                    __syncwarp();
                }
            }
        }
    }
    // the S best of the buffer: sort it (padded to a power of two)
    int P = 32;
    while (P < wn) P <<= 1;
    for (int i = wn + lane; i < P; i += 32) W[i] = KEY_EMPTY;
    __syncwarp();
    warp_bitonic_sort(W, P, lane);
    const int m = min(S, wn);
    // exact re-rank; every candidate row prefetched into L2 first
    const float *qrow = Q + q * dp;
    {
        const int lines = (d * 4 + 127) / 128;
        for (int i = lane; i < m * lines; i += 32)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(X + (int64_t)key_idx(W[i / lines]) * dp + (i % lines) * 32));
    }
    for (int r = 0; r < m; r += 2) {
        int64_t rows[2] = {(int64_t)key_idx(W[r]), r + 1 < m ? (int64_t)key_idx(W[r + 1]) : -1};
        const int n = r + 1 < m ? 2 : 1;
        float dd[2];
        l2sq_warp_rows(qrow, X, dp, d, rows, n, dd, lane);
        if (lane == 0)
            for (int u = 0; u < n; ++u) w_rk[warp][r + u] = make_key(__float_as_uint(dd[u]), (uint32_t)ids[rows[u]]);
    }
    __syncwarp();
    WarpTopK<1> F;
    F.init();
    uint64_t fthr = KEY_EMPTY;
    for (int r0 = 0; r0 < S; r0 += 32) {
        const uint64_t key = (r0 + lane < m) ? w_rk[warp][r0 + lane] : KEY_EMPTY;
        F.offer(key, fthr, k);
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
    const int64_t nqc = (nq + TC_QCHUNK - 1) / TC_QCHUNK, ncc = (nc + 127) / 128;
    if (t == 0) *n_units = nqc * ncc;
    if (t < nq) aslot[t] = t * nc;
    if (t >= nqc * ncc) return;
    const int64_t qc = t / ncc, cc = t % ncc;
    TcUnit u;
    u.a0 = qc * TC_QCHUNK;
    u.na = (int32_t)min((int64_t)TC_QCHUNK, nq - u.a0);
    u.r0 = cc * 128;
    u.r1 = min((int64_t)nc, u.r0 + 128);
    u.rbase = 0;
    u.xrow = u.r0;
    u.rch = 0;
    units[t] = u;
}

constexpr int PROBE_MAX_D = 2048;  // query row staged in shared memory

// The query's score bound for the list scan, from b = this thread's probed
// candidate list's distance bound (+inf for threads without one): with D the
// smallest b, at least `shortlist` scored rows x have |q - x|^2 <= D, so the
// shortlist-th smallest exact score |x|^2 - 2 q.x is at most D - |q|^2.  The
// scan's BF16 score differs from the exact one by at most
// 2 |q.x - acc| + rounding <= 2 (2^-7 + 2^-16 + 2^-9 (1 + 2^-8)^2) |q| |x| + ...
// (both operands rounded to 8 significant bits; 2^-9 of sum |q_i x_i| allowed
// for the tensor core's accumulation, far above FP32's), so the bound adds
// 0.03 |q| xmax + 2^-12 (xmax + |q|)^2 and rounds every other term outwards.
// Block-wide (all threads call it); thread 0 writes the ordered bound, or all
// ones when there is none.
__device__ __forceinline__ uint32_t probe_bound_key(float D, float qn, float xmax) {
    const float qa = sqrtf(qn);
    const float B = D * (1.f + 1.f / 1024.f) - qn * (1.f - 1.f / 1024.f) + 0.03f * qa * xmax +
                    (xmax + qa) * (xmax + qa) * (1.f / 4096.f);
    return (B < INFINITY && B == B) ? f2ord(B) : 0xffffffffu;
}

__device__ __forceinline__ void write_probe_bound(float b, const float *sqr, int d, float xmax,
                                                  uint32_t *__restrict__ qbound, int64_t q, float *red) {
    const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = fminf(b, __shfl_xor_sync(0xffffffffu, b, o));
    if (warp == 2) {
        float s = 0.f;
        for (int t = lane; t < d; t += 32) s = fmaf(sqr[t], sqr[t], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) red[2] = s;
    }
    if (lane == 0 && warp < 2) red[warp] = b;
    __syncthreads();
    if (j == 0) qbound[q] = probe_bound_key(fminf(red[0], red[1]), red[2], xmax);
}

// Per query (block of 256 threads): the 64 best centroids by BF16 score, their
// exact squared distances (FP32), sorted nearest first; then either the first
// np of them (fixed probing) or the learned prober's choice (MLP fused here).
template <bool MLP>
__global__ void __launch_bounds__(256) coarse_probe_kernel(const float *__restrict__ scores, int nc, int ncp2,
                                                           const float *__restrict__ Q, int d, int dp,
                                                           const float *__restrict__ C, int64_t nq, int np,
                                                           ProberWeights w, float logit_tau,
                                                           int32_t *__restrict__ probes,
                                                           int32_t *__restrict__ nprobed,
                                                           const float *__restrict__ rho, int shortlist, float xmax,
                                                           uint32_t *__restrict__ qbound, float *__restrict__ h1_out,
                                                           int32_t *__restrict__ cand_out,
                                                           float *__restrict__ cb_out, float *__restrict__ qn_out) {
    constexpr int NC = PROBER_CAND, H = PROBER_HIDDEN;
    static_assert(H == 256 && NC == 64, "warp-per-row MLP layout: 32 lanes x 8 weights, 8 warps x 8 candidates");
    __shared__ int32_t sc[NC];
    __shared__ float sd[NC], sf[NC], sz[NC], sb[NC], sred[4];
    __shared__ __align__(16) float sh1[H], sh2[H];
    __shared__ int s_cnt0;
    __shared__ __align__(16) float sqr[PROBE_MAX_D];
    __shared__ int hist[256], rsh[4], rcnt[8];
    __shared__ uint64_t top[NC];
    extern __shared__ uint64_t skeys[];  // next_pow2(nc) keys, 8 regions of next_pow2(nc) / 8
    const int64_t q = blockIdx.x;
    const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
    const float *sq = scores + q * nc;
    for (int t = j; t < d; t += 256) sqr[t] = Q[q * dp + t];
    // the 64 smallest keys (BF16 score, centroid) are the candidates: radix
    // select over the 8 warps' regions
    const int wb = ncp2 >> 3;
    for (int c = j; c < nc; c += 256) skeys[c] = make_key(f2ord(sq[c]), (uint32_t)c);
    if (j < 8) rcnt[j] = max(0, min(wb, nc - j * wb));
    __syncthreads();
    const int ntop = block_radix_select<256>(skeys, wb, rcnt, NC, top, hist, rsh);
    if (j < NC) sc[j] = j < ntop ? (int32_t)key_idx(top[j]) : -1;
    __syncthreads();
    {   // exact squared distances: one warp per candidate (eight per warp), so
        // that each load instruction reads 512 contiguous bytes of a centroid row
        const float4 *qr = reinterpret_cast<const float4 *>(sqr);
        const int n4 = d >> 2;
#pragma unroll 2
        for (int i = warp; i < NC; i += 8) {
            const int c = sc[i];  // warp-uniform
            float s0 = 0.f, s1 = 0.f;
            if (c >= 0) {
                const float4 *cr = reinterpret_cast<const float4 *>(C + (int64_t)c * dp);
                for (int t = lane; t < n4; t += 32) {
                    const float4 a = __ldg(cr + t), b = qr[t];
                    const float e0 = b.x - a.x, e1 = b.y - a.y, e2 = b.z - a.z, e3 = b.w - a.w;
                    s0 = fmaf(e0, e0, s0);
                    s1 = fmaf(e1, e1, s1);
                    s0 = fmaf(e2, e2, s0);
                    s1 = fmaf(e3, e3, s1);
                }
                for (int t = (n4 << 2) + lane; t < d; t += 32) {  // d % 4 tail
                    const float e = sqr[t] - C[(int64_t)c * dp + t];
                    s0 = fmaf(e, e, s0);
                }
            }
            float sum = s0 + s1;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            if (lane == 0) sd[i] = sum;
        }
    }
    __syncthreads();
    if (warp == 0) {
        // sort the 64 (exact distance, centroid) keys in registers: lane l
        // holds positions l and l + 32 (bitonic network, shuffles only)
        uint64_t r2[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = h * 32 + lane;
            r2[h] = sc[i] >= 0 ? make_key(__float_as_uint(sd[i]), (uint32_t)sc[i]) : KEY_EMPTY;
        }
#pragma unroll
        for (int size = 2; size <= NC; size <<= 1)
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                if (stride == 32) {
                    const uint64_t a = r2[0], b = r2[1];
                    r2[0] = a < b ? a : b;
                    r2[1] = a < b ? b : a;
                } else {
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int i = h * 32 + lane;
                        const uint64_t y = __shfl_xor_sync(0xffffffffu, r2[h], stride);
                        const bool lower = (i & stride) == 0, asc = (i & size) == 0;
                        const bool take_min = lower == asc;
                        r2[h] = take_min ? (r2[h] < y ? r2[h] : y) : (r2[h] < y ? y : r2[h]);
                    }
                }
            }
        skeys[lane] = r2[0];
        skeys[lane + 32] = r2[1];
    }
    __syncthreads();
    if (j < NC) {
        const uint64_t k = skeys[j];
        const bool e = k == KEY_EMPTY;
        const float d1 = __uint_as_float(key_dist(skeys[0]));
        sc[j] = e ? -1 : (int32_t)key_idx(k);
        sf[j] = e ? 0.f : fmaxf(0.f, 1.f - (__uint_as_float(key_dist(k)) - d1) / fmaxf(d1, 1e-12f));
        // bound on the squared distance of the query's shortlist-th nearest row if
        // this list is probed: its `shortlist` rows nearest the centroid lie within
        // rho of it, hence within |q - c| + rho of the query
        float b = INFINITY;
        if (qbound && !e) {
            const float r = rho[(size_t)key_idx(k) * IVF_RHO + shortlist - 1];
            if (r < INFINITY) {
                const float t = sqrtf(__uint_as_float(key_dist(k)) * (1.f + 1.f / 1024.f)) + r;
                b = t * t;
            }
        }
        sb[j] = b;
    }
    __syncthreads();
    if (!MLP) {
        if (j < np) probes[q * np + j] = sc[j];
        if (qbound) write_probe_bound(j < np ? sb[j] : INFINITY, sqr, d, xmax, qbound, q, sred);
        return;
    }
    const __nv_bfloat16 *W1 = reinterpret_cast<const __nv_bfloat16 *>(w.W1);
    const __nv_bfloat16 *W2 = reinterpret_cast<const __nv_bfloat16 *>(w.W2);
    const __nv_bfloat16 *W3 = reinterpret_cast<const __nv_bfloat16 *>(w.W3);
    // layer 1: thread j = hidden unit j, gathered rows of W1 (loads issued ahead)
    float a = w.b1[j];
#pragma unroll 32
    for (int i = 0; i < NC; ++i) {
        const int c = sc[i];
        const float wv = c >= 0 ? __bfloat162float(W1[(size_t)c * H + j]) : 0.f;
        a = fmaf(sf[i], wv, a);
    }
    sh1[j] = fmaxf(a, 0.f);
    if (h1_out) {
        // batched MLP: hand the first layer, the candidates, their bounds and
        // |q|^2 to mlp_probe_kernel, which runs layers 2 and 3 for 8 queries
        // per block (W2 read once per 8 queries instead of once per query)
        h1_out[q * H + j] = sh1[j];
        if (j < NC) {
            cand_out[q * NC + j] = sc[j];
            cb_out[q * NC + j] = sb[j];
        }
        if (warp == 2) {
            float qs = 0.f;
            for (int t = lane; t < d; t += 32) qs = fmaf(sqr[t], sqr[t], qs);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) qs += __shfl_xor_sync(0xffffffffu, qs, o);
            if (lane == 0) qn_out[q] = qs;
        }
        return;
    }
    __syncthreads();
    // layer 2: warp w computes outputs 32w .. 32w + 31, one W2 row (512 bytes,
    // lane l its 16 bytes) per load instruction, four rows in flight; lane l
    // holds h1[8l .. 8l + 7]
    {
        const float4 *h4 = reinterpret_cast<const float4 *>(sh1);
        const float4 x0 = h4[2 * lane], x1 = h4[2 * lane + 1];
        const float xs[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll 1
        for (int r0 = warp * 32; r0 < warp * 32 + 32; r0 += 4) {
            uint4 u[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) u[k] = __ldg(reinterpret_cast<const uint4 *>(W2 + (size_t)(r0 + k) * H) + lane);
            float acc[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u[k]);
                float t = 0.f;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float2 f = __bfloat1622float2(h[e]);
                    t = fmaf(f.x, xs[2 * e], t);
                    t = fmaf(f.y, xs[2 * e + 1], t);
                }
                acc[k] = t;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int k = 0; k < 4; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (lane == k) sh2[r0 + k] = fmaxf(acc[k] + w.b2[r0 + k], 0.f);
        }
    }
    __syncthreads();
    // layer 3: one warp per candidate (eight per warp, four in flight), its W3
    // row in one load instruction
    {
        const float4 *h4 = reinterpret_cast<const float4 *>(sh2);
        const float4 x0 = h4[2 * lane], x1 = h4[2 * lane + 1];
        const float xs[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
#pragma unroll 1
        for (int k0 = 0; k0 < 8; k0 += 4) {
            uint4 u[4];
            int cs[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                cs[k] = sc[warp + 8 * (k0 + k)];
                u[k] = cs[k] >= 0 ? __ldg(reinterpret_cast<const uint4 *>(W3 + (size_t)cs[k] * H) + lane)
                                  : make_uint4(0u, 0u, 0u, 0u);
            }
            float acc[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u[k]);
                float t = 0.f;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const float2 f = __bfloat1622float2(h[e]);
                    t = fmaf(f.x, xs[2 * e], t);
                    t = fmaf(f.y, xs[2 * e + 1], t);
                }
                acc[k] = t;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int k = 0; k < 4; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < 4; ++k) sz[warp + 8 * (k0 + k)] = cs[k] >= 0 ? acc[k] + w.b3[cs[k]] : -INFINITY;
        }
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
    if (qbound) write_probe_bound(keep ? sb[i] : INFINITY, sqr, d, xmax, qbound, q, sred);
}

// Layers 2 and 3 of the prober and the probe choice for MLP_QB queries per
// block (large batches; the first layer ran in coarse_probe_kernel):
//   layer 2  thread j = hidden unit j for the block's queries, its W2 row
//            read once (16-byte loads), the queries' first-layer outputs from
//            shared memory;
//   layer 3  warp w = query w: its 64 candidate lists' W3 rows (one 512-byte
//            row per load instruction, four in flight) against the query's
//            second-layer output;
//   choice   the nearest candidate always, the others whose logit is at
//            least the threshold, in distance order; the list scan's score
//            bound from the chosen lists.
// The arithmetic (FP32 accumulation of BF16 weights, same order per dot
// product within a lane) matches the fused kernel's up to summation order.
constexpr int MLP_QB = 8;
constexpr int64_t MLP_BATCH_MIN = 1024;  // smaller batches keep the MLP fused in coarse_probe_kernel
__global__ void __launch_bounds__(256) mlp_probe_kernel(const float *__restrict__ H1,
                                                        const int32_t *__restrict__ cand,
                                                        const float *__restrict__ cb, const float *__restrict__ qnv,
                                                        int64_t nq, ProberWeights w, float logit_tau, float xmax,
                                                        int32_t *__restrict__ probes, int32_t *__restrict__ nprobed,
                                                        uint32_t *__restrict__ qbound) {
    constexpr int NC = PROBER_CAND, H = PROBER_HIDDEN;
    __shared__ __align__(16) float h1s[MLP_QB][H], h2s[MLP_QB][H];
    const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
    const int64_t q0 = (int64_t)blockIdx.x * MLP_QB;
    const int nqb = (int)min((int64_t)MLP_QB, nq - q0);
    for (int i = j; i < MLP_QB * H; i += 256) {
        const int qq = i / H;
        h1s[qq][i % H] = qq < nqb ? H1[(q0 + qq) * H + i % H] : 0.f;
    }
    __syncthreads();
    {   // layer 2
        const __nv_bfloat16 *W2 = reinterpret_cast<const __nv_bfloat16 *>(w.W2);
        const uint4 *row = reinterpret_cast<const uint4 *>(W2 + (size_t)j * H);
        float acc[MLP_QB];
#pragma unroll
        for (int qq = 0; qq < MLP_QB; ++qq) acc[qq] = 0.f;
#pragma unroll 4
        for (int i8 = 0; i8 < H / 8; ++i8) {
            const uint4 u = __ldg(row + i8);
            const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
            float wv[8];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float2 f = __bfloat1622float2(h[e]);
                wv[2 * e] = f.x;
                wv[2 * e + 1] = f.y;
            }
#pragma unroll
            for (int qq = 0; qq < MLP_QB; ++qq) {
                const float4 x0 = *reinterpret_cast<const float4 *>(&h1s[qq][8 * i8]);
                const float4 x1 = *reinterpret_cast<const float4 *>(&h1s[qq][8 * i8 + 4]);
                acc[qq] = fmaf(wv[0], x0.x, acc[qq]);
                acc[qq] = fmaf(wv[1], x0.y, acc[qq]);
                acc[qq] = fmaf(wv[2], x0.z, acc[qq]);
                acc[qq] = fmaf(wv[3], x0.w, acc[qq]);
                acc[qq] = fmaf(wv[4], x1.x, acc[qq]);
                acc[qq] = fmaf(wv[5], x1.y, acc[qq]);
                acc[qq] = fmaf(wv[6], x1.z, acc[qq]);
                acc[qq] = fmaf(wv[7], x1.w, acc[qq]);
            }
        }
        const float b2 = w.b2[j];
#pragma unroll
        for (int qq = 0; qq < MLP_QB; ++qq) h2s[qq][j] = fmaxf(acc[qq] + b2, 0.f);
    }
    __syncthreads();
    if (warp >= nqb) return;
    const int64_t q = q0 + warp;
    // layer 3 for this warp's query: lane l holds h2[8l .. 8l + 7]
    const __nv_bfloat16 *W3 = reinterpret_cast<const __nv_bfloat16 *>(w.W3);
    const float4 x0 = *reinterpret_cast<const float4 *>(&h2s[warp][8 * lane]);
    const float4 x1 = *reinterpret_cast<const float4 *>(&h2s[warp][8 * lane + 4]);
    const float xs[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
    const int32_t c_lo = cand[q * NC + lane], c_hi = cand[q * NC + 32 + lane];
    float z_lo = -INFINITY, z_hi = -INFINITY;
#pragma unroll 1
    for (int i0 = 0; i0 < NC; i0 += 4) {
        uint4 u[4];
        int cs[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            cs[k] = __shfl_sync(0xffffffffu, (i0 + k) < 32 ? c_lo : c_hi, (i0 + k) & 31);
            u[k] = cs[k] >= 0 ? __ldg(reinterpret_cast<const uint4 *>(W3 + (size_t)cs[k] * H) + lane)
                              : make_uint4(0u, 0u, 0u, 0u);
        }
        float acc[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u[k]);
            float t = 0.f;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float2 f = __bfloat1622float2(h[e]);
                t = fmaf(f.x, xs[2 * e], t);
                t = fmaf(f.y, xs[2 * e + 1], t);
            }
            acc[k] = t;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < 4; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = i0 + k;
            const float z = cs[k] >= 0 ? acc[k] + w.b3[cs[k]] : -INFINITY;
            if (i < 32 && lane == i) z_lo = z;
            if (i >= 32 && lane == i - 32) z_hi = z;
        }
    }
    // the choice: candidate 0 always, the others at or above the threshold
    const bool k_lo = c_lo >= 0 && (lane == 0 || z_lo >= logit_tau);
    const bool k_hi = c_hi >= 0 && z_hi >= logit_tau;
    const unsigned m_lo = __ballot_sync(0xffffffffu, k_lo), m_hi = __ballot_sync(0xffffffffu, k_hi);
    const int n_lo = __popc(m_lo);
    if (k_lo) probes[q * NC + __popc(m_lo & ((1u << lane) - 1u))] = c_lo;
    if (k_hi) probes[q * NC + n_lo + __popc(m_hi & ((1u << lane) - 1u))] = c_hi;
    const int total = n_lo + __popc(m_hi);
    for (int t = total + lane; t < NC; t += 32) probes[q * NC + t] = -1;
    if (lane == 0 && nprobed) nprobed[q] = total;
    if (qbound) {
        float b = fminf(k_lo ? cb[q * NC + lane] : INFINITY, k_hi ? cb[q * NC + 32 + lane] : INFINITY);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) b = fminf(b, __shfl_xor_sync(0xffffffffu, b, o));
        if (lane == 0) qbound[q] = probe_bound_key(b, qnv[q], xmax);
    }
}

// Probes of the tensor-core engine: BF16 centroid scores on the tensor cores,
// exact re-rank of the 64 best, then fixed n_probe or the learned prober.
static int ivfl2_probes_tc(gn_index *ix, const float *dQ, int64_t nq, int *np_out, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    IvfScratch &T = S.s;
    // per query: the list scan's score bound (all ones: none, every score kept)
    GN_TRY(T.qbound.ensure((size_t)std::max<int64_t>(nq, 1) * 4));
    if (S.nc < PROBER_CAND || S.d > PROBE_MAX_D || S.nc > 8192) {  // outside the 64-candidate stage's limits
        if (S.prober) return fail(GN_ERR_INVALID, "learned probing needs at least 64 lists");
        int np = std::min<int32_t>(S.nprobe, S.nc);
        *np_out = np;
        GN_CUDA_TRY(cudaMemsetAsync(T.qbound.p, 0xff, (size_t)nq * 4, st));
        return ivfl2_coarse(ix, dQ, nq, np, st);
    }
    const bool mlp = S.prober != nullptr;
    const int np = mlp ? PROBER_CAND : std::min<int32_t>(std::min<int32_t>(S.nprobe, S.nc), PROBER_CAND);
    if (!mlp && S.nprobe > PROBER_CAND) {  // wider fixed probing: the FP32 coarse stage
        *np_out = std::min<int32_t>(S.nprobe, S.nc);
        GN_CUDA_TRY(cudaMemsetAsync(T.qbound.p, 0xff, (size_t)nq * 4, st));
        return ivfl2_coarse(ix, dQ, nq, *np_out, st);
    }
    *np_out = np;
    const int64_t units = ceil_div(nq, TC_QCHUNK) * ceil_div(S.nc, 128);
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
    a.next_unit = S.sched.as<unsigned long long>() + 0;
    a.grid = (int)std::min<int64_t>(dev_info().num_sms, units);
    GN_TRY(tc_ivf_launch(a, st));
    const int ncp2 = (int)next_pow2(S.nc);
    const size_t ksm = (size_t)ncp2 * 8;
    if (ksm > 48 * 1024) {
        GN_CUDA_TRY(cudaFuncSetAttribute(coarse_probe_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ksm));
        GN_CUDA_TRY(cudaFuncSetAttribute(coarse_probe_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ksm));
    }
    ProberWeights w;
    float *h1 = nullptr, *cbnd = nullptr, *qnv = nullptr;
    int32_t *cand = nullptr;
    if (mlp) {
        GN_TRY(prober_weights(S.prober, &w));
        GN_TRY(T.nprobed.ensure((size_t)nq * 4));
        if (nq >= MLP_BATCH_MIN) {  // layers 2 and 3 batched over 8 queries per block
            GN_TRY(T.mh1.ensure((size_t)nq * PROBER_HIDDEN * 4));
            GN_TRY(T.mcand.ensure((size_t)nq * PROBER_CAND * 4));
            GN_TRY(T.mcb.ensure((size_t)nq * PROBER_CAND * 4));
            GN_TRY(T.mqn.ensure((size_t)nq * 4));
            h1 = T.mh1.as<float>();
            cand = T.mcand.as<int32_t>();
            cbnd = T.mcb.as<float>();
            qnv = T.mqn.as<float>();
        }
        coarse_probe_kernel<true><<<(unsigned)nq, 256, ksm, st>>>(S.cscores.as<float>(), S.nc, ncp2, dQ, S.d, S.dp,
                                                               S.cent.as<float>(), nq, np, w, S.prober_tau,
                                                               T.probes.as<int32_t>(), T.nprobed.as<int32_t>(),
                                                               S.rho.as<float>(), S.shortlist, S.xmax,
                                                               T.qbound.as<uint32_t>(), h1, cand, cbnd, qnv);
        if (h1)
            mlp_probe_kernel<<<(unsigned)ceil_div(nq, MLP_QB), 256, 0, st>>>(
                h1, cand, cbnd, qnv, nq, w, S.prober_tau, S.xmax, T.probes.as<int32_t>(), T.nprobed.as<int32_t>(),
                T.qbound.as<uint32_t>());
    } else {
        coarse_probe_kernel<false><<<(unsigned)nq, 256, ksm, st>>>(S.cscores.as<float>(), S.nc, ncp2, dQ, S.d, S.dp,
                                                                S.cent.as<float>(), nq, np, w, 0.f,
                                                                T.probes.as<int32_t>(), nullptr,
                                                                S.rho.as<float>(), S.shortlist, S.xmax,
                                                                T.qbound.as<uint32_t>(), nullptr, nullptr, nullptr,
                                                                nullptr);
    }
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

// FP32 list rows (dp floats) -> the tiled BF16 layout of IvfL2State::x16:
// thread per (row, 8 values); row r of list l goes to padded row
// p = xoff[l] + (r - list_off[l]), tile p / 128, and its K slice kb to the
// 16 KB block (tile * K/64 + kb); values past d are zero.
__global__ void x16_tiled_kernel(const float *__restrict__ X, int64_t n, int d, int dp,
                                 const int64_t *__restrict__ list_off, int nc, const int64_t *__restrict__ xoff,
                                 int K, uint4 *__restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int g8 = K / 8;
    const int64_t r = t / g8;
    if (r >= n) return;
    const int g = (int)(t % g8);
    int lo = 0, hi = nc;  // list l: list_off[l] <= r < list_off[l + 1]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (list_off[mid] <= r) lo = mid;
        else hi = mid;
    }
    const int64_t p = xoff[lo] + (r - list_off[lo]);
    const int kb = g >> 3, e0 = (g & 7) * 8, c0 = kb * 64 + e0;
    __align__(16) __nv_bfloat16 v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) v[e] = __float2bfloat16_rn(c0 + e < d ? X[r * dp + c0 + e] : 0.f);
    out[((((p >> 7) * (K / 64) + kb) * 128 + (p & 127)) * 64 + e0) / 8] = *reinterpret_cast<const uint4 *>(v);
}

// Squared distance (FP32) of every list row to its list's centroid, warp per row.
__global__ void row_centroid_dist_kernel(const float *__restrict__ X, int64_t n, int d, int dp,
                                         const int64_t *__restrict__ list_off, int nc, const float *__restrict__ C,
                                         float *__restrict__ out) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= n) return;
    int lo = 0, hi = nc;  // list l: list_off[l] <= r < list_off[l + 1]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (list_off[mid] <= r) lo = mid;
        else hi = mid;
    }
    float s = 0.f;
    for (int t = lane; t < d; t += 32) {
        const float e = X[r * dp + t] - C[(int64_t)lo * dp + t];
        s = fmaf(e, e, s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[r] = s;
}

// Inputs of the list scan's score bound (the probe stage turns them into a
// per-query bound): per list, the distances to its centroid of the 64 rows
// nearest it, ascending, each rounded up by a relative 2^-10 (covering the
// FP32 sum's rounding); +inf past the list's size.  And the largest row norm.
static int ivfl2_list_radii(IvfL2State &S, cudaStream_t st) {
    std::vector<float> dist((size_t)S.n), nrm((size_t)S.n);
    if (S.n > 0) {
        DBuf tmp;
        GN_TRY(tmp.ensure((size_t)S.n * 4));
        row_centroid_dist_kernel<<<(unsigned)ceil_div(S.n * 32, 256), 256, 0, st>>>(
            S.vecs.as<float>(), S.n, S.d, S.dp, S.list_off.as<int64_t>(), S.nc, S.cent.as<float>(), tmp.as<float>());
        GN_CUDA_TRY(cudaGetLastError());
        GN_CUDA_TRY(cudaMemcpyAsync(dist.data(), tmp.p, (size_t)S.n * 4, cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaMemcpyAsync(nrm.data(), S.vnorm.p, (size_t)S.n * 4, cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
    }
    std::vector<float> rho((size_t)S.nc * IVF_RHO, INFINITY);
    for (int32_t l = 0; l < S.nc; ++l) {
        float *b = dist.data() + S.h_off[(size_t)l], *e = dist.data() + S.h_off[(size_t)l + 1];
        const int64_t m = std::min<int64_t>(IVF_RHO, e - b);
        std::partial_sort(b, b + m, e);
        for (int64_t j = 0; j < m; ++j)
            rho[(size_t)l * IVF_RHO + j] = std::sqrt(std::max(0.f, b[j]) * (1.f + 1.f / 1024.f));
    }
    float x2 = 0.f;
    for (float v : nrm) x2 = std::max(x2, v);
    S.xmax = std::sqrt(x2 * (1.f + 1.f / 1024.f));
    GN_TRY(S.rho.ensure(rho.size() * 4));
    GN_CUDA_TRY(cudaMemcpyAsync(S.rho.p, rho.data(), rho.size() * 4, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));  // rho goes out of scope
    return GN_OK;
}

int ivfl2_prepare_tc(gn_index *ix, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    GN_TRY(ivfl2_list_radii(S, st));
    S.K = (int)round_up(S.d, 64);
    // BF16 list rows, tiled (see IvfL2State::x16): padded list starts
    std::vector<int64_t> xo((size_t)S.nc + 1, 0);
    for (int32_t l = 0; l < S.nc; ++l)
        xo[(size_t)l + 1] = xo[(size_t)l] + round_up(S.h_off[(size_t)l + 1] - S.h_off[(size_t)l], 128);
    S.x16_rows = std::max<int64_t>(xo[(size_t)S.nc], 128);
    if (S.x16_rows * (S.K / 64) >= ((int64_t)1 << 31))
        return fail(GN_ERR_UNSUPPORTED, "tensor-core IVF: too many rows x dimensions for the tiled layout");
    GN_TRY(S.xoff.ensure(xo.size() * 8));
    GN_CUDA_TRY(cudaMemcpyAsync(S.xoff.p, xo.data(), xo.size() * 8, cudaMemcpyHostToDevice, st));
    GN_TRY(S.x16.ensure((size_t)S.x16_rows * S.K * 2));
    GN_CUDA_TRY(cudaMemsetAsync(S.x16.p, 0, (size_t)S.x16_rows * S.K * 2, st));
    if (S.n > 0)
        x16_tiled_kernel<<<(unsigned)ceil_div(S.n * (S.K / 8), 256), 256, 0, st>>>(
            S.vecs.as<float>(), S.n, S.d, S.dp, S.list_off.as<int64_t>(), S.nc, S.xoff.as<int64_t>(), S.K,
            S.x16.as<uint4>());
    GN_CUDA_TRY(cudaStreamSynchronize(st));  // xo goes out of scope
    const int64_t crows = std::max<int64_t>(S.nc, 128);  // at least one 128-row TMA box
    GN_TRY(S.c16.ensure((size_t)crows * S.K * 2));
    GN_CUDA_TRY(cudaMemsetAsync(S.c16.p, 0, (size_t)crows * S.K * 2, st));
    to_bf16_rows(S.cent.as<float>(), S.nc, S.d, S.dp, S.c16.p, S.K, st);
    GN_TRY(S.err.ensure(4));
    GN_CUDA_TRY(cudaMemsetAsync(S.err.p, 0, 4, st));
    GN_TRY(S.sched.ensure(2 * sizeof(unsigned long long)));
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
    const IvfL2State::TcTune &tn = S.tune[tune_bucket(nq)];
    const int rc = tn.rc ? tn.rc : (nq >= 64 ? 1024 : 256);
    // score segments in 128-row slots: slot_rel / qslot count slots, and a
    // pair's tile t has its minima at tmin4[(slot base + t) * 4 ...]
    // queries per work unit (the MMA's N side): 128, or fewer to cut a mid-size
    // batch's lists into more units
    const int qch = tn.qc ? tn.qc : TC_QCHUNK;
    GN_TRY(ivf_plan(T, nq, np, S.nc, S.list_off.as<int64_t>(), rc, qch, st, 128));
    const int64_t npairs = nq * np;
    const int64_t qb_rows = std::max<int64_t>(npairs, 256);  // >= one 256-row TMA box
    GN_TRY(S.qb.ensure((size_t)qb_rows * S.K * 2));
    GN_TRY(S.aslot.ensure((size_t)npairs * 8));
    GN_TRY(S.abound.ensure((size_t)std::max<int64_t>(npairs, 1) * 4));
    const int64_t maxlen = S.top_rows.size() > 1 ? S.top_rows[1] : 0;
    // sized for the shortest row chunk (256) so that a smaller batch never needs more
    const int64_t max_units = (ceil_div(npairs, qch) + S.nc) * (ceil_div(maxlen, 256) + 1);
    GN_TRY(S.units.ensure((size_t)max_units * sizeof(TcUnit)));
    GN_TRY(S.nunits.ensure(8));
    const unsigned qb_blocks = (unsigned)ceil_div(npairs, 8);
    qb_units_kernel<<<qb_blocks + (unsigned)ceil_div(max_units, 256), 256, 0, st>>>(
        S.q16.as<uint4>(), S.K / 8, np, T.bucket.as<int64_t>(), T.boff.as<int64_t>(), S.nc, T.qslot.as<int64_t>(),
        T.slot_rel.as<int64_t>(), S.qb.as<uint4>(), S.aslot.as<int64_t>(), T.qbound.as<uint32_t>(),
        S.abound.as<uint32_t>(), npairs, qb_blocks,
        T.item_off.as<int64_t>(), S.list_off.as<int64_t>(), S.xoff.as<int64_t>(), rc, qch, max_units, S.units.as<TcUnit>(),
        S.nunits.as<int64_t>());
    // score slots: at most the rows of the np largest lists per query, plus one
    // partial slot per probe
    const int64_t np_eff = std::min<int64_t>(np, (int64_t)S.top_rows.size() - 1);
    const int64_t slots_total = nq * (ceil_div(S.top_rows[(size_t)np_eff], 128) + np);
    GN_TRY(S.scores.ensure((size_t)std::max<int64_t>(slots_total, 1) * 128 * 4));
    GN_TRY(S.tmin.ensure((size_t)std::max<int64_t>(slots_total, 1) * 4 * 4));
    TcIvfLaunch a;
    a.X = S.x16.p;
    a.x_rows = S.x16_rows;
    a.tiled = 1;
    a.Q = S.qb.p;
    a.q_rows = qb_rows;
    a.K = S.K;
    a.units = S.units.as<TcUnit>();
    a.n_units = S.nunits.as<int64_t>();
    a.xnorm = S.vnorm.as<float>();
    a.aslot = S.aslot.as<int64_t>();
    a.seg_mul = 128;
    a.scores = S.scores.as<float>();
    a.tmin4 = S.tmin.as<uint32_t>();
    a.abound = S.abound.as<uint32_t>();
    a.err = S.err.as<int>();
    a.next_unit = S.sched.as<unsigned long long>() + 1;
    if (S.drill) {  // armed failure drill: this launch's waits run out after ~0.1 ms
        a.drill = 1;
        a.wait_limit = 200000;
        S.drill = 0;
        S.cfg++;
    }
    a.grid = dev_info().num_sms;
    timing_begin(st, "tc_ivf_kernel");
    GN_TRY(tc_ivf_launch(a, st));
    timing_end(st);
    // selector: a warp per query when the autotuner chose it (nt = 32; it
    // measured slower than the block selectors on the 1M x 512 mixture, whose
    // queries probe ~300 slots each: one warp sweeps them one dependent load
    // after another), else blocks of nt threads per query
    const int nsm = dev_info().num_sms;
    if (np <= 64 && tn.nt == 32) {
        ivf_tc_select_warp_kernel<<<(unsigned)ceil_div(nq, SELW_WARPS), 32 * SELW_WARPS, 0, st>>>(
            S.scores.as<float>(), S.tmin.as<uint4>(), T.qbound.as<uint32_t>(), T.probes.as<int32_t>(), np,
            T.qslot.as<int64_t>(), T.slot_rel.as<int64_t>(), S.list_off.as<int64_t>(), S.shortlist, dQ,
            S.vecs.as<float>(), S.d, S.dp, S.ids.as<int32_t>(), nq, k, d_idx, d_dist, d_cnt);
        GN_CUDA_TRY(cudaGetLastError());
        return GN_OK;
    }
    // B blocks per query: split small batches so that they still fill the GPU
    int B = 1;
    const int bmax = tn.bmax ? tn.bmax : 16;
    if (np <= SEL_PCH)
        while (B < bmax && nq * B * 2 <= (int64_t)nsm * 4) B *= 2;
    if (B > 1) {
        // nq * B <= 4 * SMs here: one size for every small batch
        GN_TRY(S.sel_part.ensure((size_t)std::max<int64_t>(nq * B, (int64_t)nsm * 4) * S.shortlist * 8));
        const size_t cap0 = S.sel_done.cap;
        GN_TRY(S.sel_done.ensure((size_t)std::max<int64_t>(nq, 1024) * 4));
        if (S.sel_done.cap != cap0) GN_CUDA_TRY(cudaMemsetAsync(S.sel_done.p, 0, S.sel_done.cap, st));
    }
    const unsigned blocks = (unsigned)(nq * B);
    // small batches: 8 warps per query part; large: 4 warps, more queries in flight
    auto sel = [&](auto NTC) -> int {
        constexpr int NT = decltype(NTC)::value;
        static bool carve = false;  // shared memory over L1: the scores are streamed once
        if (!carve) {
            GN_CUDA_TRY(cudaFuncSetAttribute(ivf_tc_select_kernel<NT>,
                                             cudaFuncAttributePreferredSharedMemoryCarveout, 100));
            carve = true;
        }
        ivf_tc_select_kernel<NT><<<blocks, NT, 0, st>>>(
            S.scores.as<float>(), S.tmin.as<uint4>(), T.qbound.as<uint32_t>(), T.probes.as<int32_t>(), np,
            T.qslot.as<int64_t>(), T.slot_rel.as<int64_t>(),
            S.list_off.as<int64_t>(), S.shortlist, dQ, S.vecs.as<float>(), S.d, S.dp, S.ids.as<int32_t>(), nq, k, B,
            S.sel_part.as<uint64_t>(), S.sel_done.as<int>(), d_idx, d_dist, d_cnt);
        return GN_OK;
    };
    if (tn.nt == 128 || (tn.nt != 256 && nq * B >= (int64_t)nsm * 8)) GN_TRY(sel(std::integral_constant<int, 128>()));
    else GN_TRY(sel(std::integral_constant<int, 256>()));
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
    std::lock_guard<std::mutex> lk(ix->mu);
    int herr = 0;
    if (ix->ivfl2->err.p) {
        if (ix->stream) GN_CUDA_TRY(cudaStreamSynchronize(ix->stream));
        GN_CUDA_TRY(cudaDeviceSynchronize());
        GN_CUDA_TRY(cudaMemcpy(&herr, ix->ivfl2->err.p, 4, cudaMemcpyDeviceToHost));
        if (herr) GN_CUDA_TRY(cudaMemset(ix->ivfl2->err.p, 0, 4));  // read and cleared
    }
    if (err_out) *err_out = herr;
    return GN_OK;
}

// Failure drill (tests): the next tensor-core list scan of this index issues
// no tile copies and bounds its pipeline waits to 200,000 cycles, so they run
// out: the launch ends early with the error word set and its TMEM freed.
extern "C" int gn_ivfl2_failure_drill(gn_index *ix) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    std::lock_guard<std::mutex> lk(ix->mu);
    ix->ivfl2->drill = 1;
    ix->ivfl2->cfg++;
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
