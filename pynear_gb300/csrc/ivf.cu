// ivf.cu — IVF-flat indexes: CSR build, coarse probing, bucketed list scans.
//
// Search of a query batch runs entirely on the device, with no host round
// trip between its kernels:
//   1. coarse   the nprobe nearest centroids of every query (fused GEMM +
//               warp top-k for L2; the exact Hamming flat scan for binary);
//   2. buckets  (query, probe) pairs grouped by list: counts, offsets, fill;
//   3. plan     work items = (list, chunk of queries probing it, chunk of list
//               rows); every (query, probe, row chunk) owns one partial slot;
//   4. scan     a persistent kernel pulls items from an atomic counter, scores
//               the chunk (FP32 tile GEMM for L2, popcount for Hamming) and
//               writes each query's partial top-k to its slot;
//   5. merge    one warp per query reduces its slots to the final top-k.
// Lists are stored as a CSR (offsets, rows in list order, original ids).  The
// float index orders its lists by descending size so the persistent scan
// starts with the longest items.
//
// Reference: IVFFlatL2Index (pynear/forest.py:36-111,189-204) and
// IVFFlatBinaryIndex (pynear/include/BinaryIVF.hpp:65-111).  Result order is
// the lexicographic (distance, original index) order; a query gets fewer than k
// results when its probed lists hold fewer rows.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "distance.cuh"
#include "flat_scan.cuh"
#include "gemm_topk.cuh"
#include "ivf.cuh"
#include "kmeans.cuh"
#include "prober.cuh"
#include "timing.cuh"
#include "topk.cuh"

namespace gn {

constexpr int IVF_QCHUNK_L2 = GT_BM;  // queries per float work item
constexpr int IVF_QCHUNK_BIN = 32;    // queries per binary work item (4 warps x 8)

// ── coarse probing (float): GEMM + per-query top-nprobe ───────────────────
// blockIdx.y selects a slice of cps centroids (one slice when the batch alone
// fills the GPU); with several slices each writes its sorted partial top-np
// keys to part[(q * gridDim.y + slice) * np ...] for coarse_merge_kernel.
template <int R>
__global__ void __launch_bounds__(GT_THREADS) ivf_coarse_kernel(const float *__restrict__ Q,
                                                                const float *__restrict__ qn, int64_t nq, int dp,
                                                                const float *__restrict__ C,
                                                                const float *__restrict__ cn, int nc, int np,
                                                                int cps, int32_t *__restrict__ probes,
                                                                uint64_t *__restrict__ part) {
    __shared__ GemmTileSmem s;
    __shared__ int64_t arow[GT_BM];
    const int64_t q0 = (int64_t)blockIdx.x * GT_BM;
    const int cb = blockIdx.y * cps, ce = min(nc, cb + cps);
    if (threadIdx.x < GT_BM) arow[threadIdx.x] = (q0 + threadIdx.x < nq) ? q0 + threadIdx.x : -1;
    __syncthreads();
    const int tm = threadIdx.x >> 5, tn = threadIdx.x & 31;
    WarpTopK<R> L[8];
    uint64_t thr[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) { L[i].init(); thr[i] = KEY_EMPTY; }
    float acc[8][4];
    for (int c0 = cb; c0 < ce; c0 += GT_BN) {
        gt_tile(s, acc, Q, arow, dp, C, c0, ce, dp, dp);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t q = arow[tm * 8 + i];
            const float qv = q >= 0 ? qn[q] : 0.f;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = c0 + tn * 4 + j;
                uint64_t key = KEY_EMPTY;
                if (c < ce && q >= 0) {
                    const float v = fmaxf(0.f, fmaf(-2.f, acc[i][j], qv + cn[c]));
                    key = make_key(__float_as_uint(v), (uint32_t)c);
                }
                L[i].offer(key, thr[i], np);
            }
        }
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int64_t q = arow[tm * 8 + i];
        if (q < 0) continue;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int p = r * 32 + lane;
            if (p >= np) continue;
            if (part) part[((size_t)q * gridDim.y + blockIdx.y) * np + p] = L[i].v[r];
            else probes[q * np + p] = (L[i].v[r] == KEY_EMPTY) ? -1 : (int32_t)key_idx(L[i].v[r]);
        }
    }
}

template <int R>
__global__ void coarse_merge_kernel(const uint64_t *__restrict__ part, int nsplit, int np, int64_t nq,
                                    int32_t *__restrict__ probes, uint64_t *__restrict__ keys_out) {
    const int lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= nq) return;
    WarpTopK<R> L;
    L.init();
    uint64_t thr = KEY_EMPTY;
    for (int sp = 0; sp < nsplit; ++sp)
        for (int j0 = 0; j0 < np; j0 += 32) {
            const int j = j0 + lane;
            L.offer(j < np ? part[((size_t)q * nsplit + sp) * np + j] : KEY_EMPTY, thr, np);
        }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int p = r * 32 + lane;
        if (p >= np) continue;
        if (keys_out) keys_out[q * np + p] = L.v[r];
        else probes[q * np + p] = (L.v[r] == KEY_EMPTY) ? -1 : (int32_t)key_idx(L.v[r]);
    }
}

// ── bucketing and planning ────────────────────────────────────────────────
__global__ void ivf_bucket_count_kernel(const int32_t *__restrict__ probes, int64_t npairs, int32_t *__restrict__ bcnt) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npairs) return;
    const int32_t l = probes[t];
    if (l >= 0) atomicAdd(bcnt + l, 1);
}

// Exclusive block-wide scan of per-thread totals (one block of 1024 threads).
__device__ int64_t block_exclusive_scan(int64_t v, int64_t *total) {
    __shared__ int64_t warp_tot[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const int64_t excl = x - v + (w > 0 ? warp_tot[w - 1] : 0);
    if (total) *total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

// boff = exclusive scan of bucket counts; item_off = exclusive scan of the
// per-list item counts ceil(count / qchunk) * ceil(len / rc).
__global__ void __launch_bounds__(1024) ivf_plan_kernel(const int32_t *__restrict__ bcnt,
                                                        const int64_t *__restrict__ list_off, int nc, int rc,
                                                        int qchunk, int64_t *__restrict__ boff,
                                                        int64_t *__restrict__ item_off) {
    const int per = (nc + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(nc, b + per);
    int64_t sb = 0, si = 0;
    for (int l = b; l < e; ++l) {
        const int64_t cnt = bcnt[l], len = list_off[l + 1] - list_off[l];
        sb += cnt;
        si += (cnt > 0 && len > 0) ? ((cnt + qchunk - 1) / qchunk) * ((len + rc - 1) / rc) : 0;
    }
    int64_t tb = 0, ti = 0;
    int64_t xb = block_exclusive_scan(sb, &tb);
    int64_t xi = block_exclusive_scan(si, &ti);
    for (int l = b; l < e; ++l) {
        const int64_t cnt = bcnt[l], len = list_off[l + 1] - list_off[l];
        boff[l] = xb;
        item_off[l] = xi;
        xb += cnt;
        xi += (cnt > 0 && len > 0) ? ((cnt + qchunk - 1) / qchunk) * ((len + rc - 1) / rc) : 0;
    }
    if (threadIdx.x == 0) {
        boff[nc] = tb;
        item_off[nc] = ti;
    }
}

__global__ void ivf_bucket_fill_kernel(const int32_t *__restrict__ probes, int64_t npairs,
                                       const int64_t *__restrict__ boff, int32_t *__restrict__ fill,
                                       int64_t *__restrict__ bucket) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= npairs) return;
    const int32_t l = probes[t];
    if (l >= 0) bucket[boff[l] + atomicAdd(fill + l, 1)] = t;
}

// per query (one warp): slot offset of each probe (relative, exclusive scan
// of the probes' slot counts) and the query's slot count
__global__ void ivf_slots_kernel(const int32_t *__restrict__ probes, int64_t nq, int np,
                                 const int64_t *__restrict__ list_off, int rc, int64_t *__restrict__ slot_rel,
                                 int64_t *__restrict__ qcount) {
    const int lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= nq) return;
    int64_t s = 0;
    for (int p0 = 0; p0 < np; p0 += 32) {
        const int p = p0 + lane;
        int64_t c = 0;
        if (p < np) {
            const int32_t l = probes[q * np + p];
            if (l >= 0) c = (list_off[l + 1] - list_off[l] + rc - 1) / rc;
        }
        int64_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (p < np) slot_rel[q * np + p] = s + inc - c;
        s += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) qcount[q] = s;
}

// qslot[0..nq] = exclusive scan of qcount (one block)
__global__ void __launch_bounds__(1024) ivf_qscan_kernel(const int64_t *__restrict__ qcount, int64_t nq,
                                                         int64_t *__restrict__ qslot) {
    const int64_t per = (nq + blockDim.x - 1) / blockDim.x;
    const int64_t b = threadIdx.x * per, e = min(nq, b + per);
    int64_t s = 0;
    for (int64_t i = b; i < e; ++i) s += qcount[i];
    int64_t tot = 0;
    int64_t x = block_exclusive_scan(s, &tot);
    for (int64_t i = b; i < e; ++i) {
        qslot[i] = x;
        x += qcount[i];
    }
    if (threadIdx.x == 0) qslot[nq] = tot;
}

// The whole plan of a small batch in one block (replaces the count, plan,
// fill, slots and scan kernels and their memsets): bucket counts in shared
// memory, list offsets and work items, bucket fill, per-query slots and their
// scan.  Same outputs as the multi-kernel plan.
__global__ void __launch_bounds__(1024) ivf_plan_small_kernel(
    const int32_t *__restrict__ probes, int64_t nq, int np, int nc, const int64_t *__restrict__ list_off, int rc,
    int qchunk, int slot_rc, int32_t *__restrict__ bcnt, int64_t *__restrict__ boff, int64_t *__restrict__ item_off,
    int64_t *__restrict__ bucket, int64_t *__restrict__ slot_rel, int64_t *__restrict__ qcount,
    int64_t *__restrict__ qslot, int64_t *__restrict__ counter) {
    extern __shared__ int32_t plan_sm[];  // [nc] counts, [nc] fill cursors
    int32_t *s_cnt = plan_sm, *s_fill = plan_sm + nc;
    const int t = threadIdx.x, nt = blockDim.x;
    const int64_t npairs = nq * np;
    for (int l = t; l < nc; l += nt) s_cnt[l] = s_fill[l] = 0;
    if (t == 0) *counter = 0;
    __syncthreads();
    for (int64_t i = t; i < npairs; i += nt) {
        const int32_t l = probes[i];
        if (l >= 0) atomicAdd(&s_cnt[l], 1);
    }
    __syncthreads();
    {
        const int per = (nc + nt - 1) / nt;
        const int b = t * per, e = min(nc, b + per);
        int64_t sb = 0, si = 0;
        for (int l = b; l < e; ++l) {
            const int64_t cnt = s_cnt[l], len = list_off[l + 1] - list_off[l];
            sb += cnt;
            si += (cnt > 0 && len > 0) ? ((cnt + qchunk - 1) / qchunk) * ((len + rc - 1) / rc) : 0;
        }
        int64_t tb = 0, ti = 0;
        int64_t xb = block_exclusive_scan(sb, &tb);
        int64_t xi = block_exclusive_scan(si, &ti);
        for (int l = b; l < e; ++l) {
            const int64_t cnt = s_cnt[l], len = list_off[l + 1] - list_off[l];
            bcnt[l] = (int32_t)cnt;
            boff[l] = xb;
            item_off[l] = xi;
            xb += cnt;
            xi += (cnt > 0 && len > 0) ? ((cnt + qchunk - 1) / qchunk) * ((len + rc - 1) / rc) : 0;
        }
        if (t == 0) {
            boff[nc] = tb;
            item_off[nc] = ti;
        }
    }
    __syncthreads();
    for (int64_t i = t; i < npairs; i += nt) {
        const int32_t l = probes[i];
        if (l >= 0) bucket[boff[l] + atomicAdd(&s_fill[l], 1)] = i;
    }
    // slots: warp per query
    const int lane = t & 31;
    for (int64_t q = t >> 5; q < nq; q += nt >> 5) {
        int64_t s = 0;
        for (int p0 = 0; p0 < np; p0 += 32) {
            const int p = p0 + lane;
            int64_t c = 0;
            if (p < np) {
                const int32_t l = probes[q * np + p];
                if (l >= 0) c = (list_off[l + 1] - list_off[l] + slot_rc - 1) / slot_rc;
            }
            int64_t inc = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            if (p < np) slot_rel[q * np + p] = s + inc - c;
            s += __shfl_sync(0xffffffffu, inc, 31);
        }
        if (lane == 0) qcount[q] = s;
    }
    __syncthreads();
    {
        const int64_t per = (nq + nt - 1) / nt;
        const int64_t b = t * per, e = min(nq, b + per);
        int64_t s = 0;
        for (int64_t i = b; i < e; ++i) s += qcount[i];
        int64_t tot = 0;
        int64_t x = block_exclusive_scan(s, &tot);
        for (int64_t i = b; i < e; ++i) {
            qslot[i] = x;
            x += qcount[i];
        }
        if (t == 0) qslot[nq] = tot;
    }
}

__device__ __forceinline__ int find_list(const int64_t *item_off, int nc, int64_t item) {
    int lo = 0, hi = nc;  // item_off[lo] <= item < item_off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (item_off[mid] <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ── float list scan (persistent) ──────────────────────────────────────────
template <int R>
__global__ void __launch_bounds__(GT_THREADS) ivf_scan_kernel(
    const float *__restrict__ Q, const float *__restrict__ qn, int np, int dp, const float *__restrict__ V,
    const float *__restrict__ vn, const int32_t *__restrict__ ids, const int64_t *__restrict__ list_off, int nc,
    const int64_t *__restrict__ boff, const int64_t *__restrict__ bucket, const int64_t *__restrict__ item_off,
    int rc, const int64_t *__restrict__ qslot, const int64_t *__restrict__ slot_rel, int k,
    int *__restrict__ counter, uint64_t *__restrict__ part) {
    __shared__ GemmTileSmem s;
    __shared__ int64_t arow[GT_BM], apair[GT_BM];
    __shared__ int64_t s_item;
    __shared__ int s_list;
    const int64_t total = item_off[nc];
    const int tm = threadIdx.x >> 5, tn = threadIdx.x & 31;
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = atomicAdd(counter, 1);
            s_list = s_item < total ? find_list(item_off, nc, s_item) : 0;
        }
        __syncthreads();
        const int64_t item = s_item;
        if (item >= total) break;
        const int l = s_list;
        const int64_t lb = list_off[l], le = list_off[l + 1];
        const int64_t nrc = (le - lb + rc - 1) / rc;
        const int64_t local = item - item_off[l];
        const int64_t qc = local / nrc, rch = local % nrc;
        const int64_t b0 = boff[l] + qc * GT_BM, b1 = min(boff[l + 1], b0 + GT_BM);
        if (threadIdx.x < GT_BM) {
            const int64_t pr = (b0 + threadIdx.x < b1) ? bucket[b0 + threadIdx.x] : -1;
            apair[threadIdx.x] = pr;
            arow[threadIdx.x] = pr >= 0 ? pr / np : -1;
        }
        __syncthreads();
        const int64_t r0 = lb + rch * rc, r1 = min(le, r0 + rc);
        WarpTopK<R> L[8];
        uint64_t thr[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) { L[i].init(); thr[i] = KEY_EMPTY; }
        float qv[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t q = arow[tm * 8 + i];
            qv[i] = q >= 0 ? qn[q] : 0.f;
        }
        float acc[8][4];
        for (int64_t rb = r0; rb < r1; rb += GT_BN) {
            gt_tile(s, acc, Q, arow, dp, V, rb, r1, dp, dp);
            float xn[4];
            uint32_t xid[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t row = rb + tn * 4 + j;
                xn[j] = row < r1 ? vn[row] : 0.f;
                xid[j] = row < r1 ? (uint32_t)ids[row] : 0u;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const bool qok = arow[tm * 8 + i] >= 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int64_t row = rb + tn * 4 + j;
                    uint64_t key = KEY_EMPTY;
                    if (qok && row < r1) {
                        const float v = fmaxf(0.f, fmaf(-2.f, acc[i][j], qv[i] + xn[j]));
                        key = make_key(__float_as_uint(v), xid[j]);
                    }
                    L[i].offer(key, thr[i], k);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t pr = apair[tm * 8 + i];
            if (pr >= 0) {
                const int64_t slot = qslot[pr / np] + slot_rel[pr] + rch;
                L[i].store(part + slot * k, k);
            }
        }
        __syncthreads();
    }
}

// ── binary list scan (persistent) ─────────────────────────────────────────
template <int R>
__global__ void __launch_bounds__(128) ivfbin_scan_kernel(
    const uint4 *__restrict__ Q, int w4, int np, const uint4 *__restrict__ V, const int32_t *__restrict__ ids,
    const int64_t *__restrict__ list_off, int nc, const int64_t *__restrict__ boff,
    const int64_t *__restrict__ bucket, const int64_t *__restrict__ item_off, int rc,
    const int64_t *__restrict__ qslot, const int64_t *__restrict__ slot_rel, int k, int *__restrict__ counter,
    uint64_t *__restrict__ part) {
    extern __shared__ uint4 sq[];  // [32][w4]
    __shared__ int64_t apair[IVF_QCHUNK_BIN];
    __shared__ int64_t s_item;
    __shared__ int s_list;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = item_off[nc];
    for (;;) {
        if (threadIdx.x == 0) {
            s_item = atomicAdd(counter, 1);
            s_list = s_item < total ? find_list(item_off, nc, s_item) : 0;
        }
        __syncthreads();
        const int64_t item = s_item;
        if (item >= total) break;
        const int l = s_list;
        const int64_t lb = list_off[l], le = list_off[l + 1];
        const int64_t nrc = (le - lb + rc - 1) / rc;
        const int64_t local = item - item_off[l];
        const int64_t qc = local / nrc, rch = local % nrc;
        const int64_t b0 = boff[l] + qc * IVF_QCHUNK_BIN, b1 = min(boff[l + 1], b0 + IVF_QCHUNK_BIN);
        if (threadIdx.x < IVF_QCHUNK_BIN)
            apair[threadIdx.x] = (b0 + threadIdx.x < b1) ? bucket[b0 + threadIdx.x] : -1;
        __syncthreads();
        for (int i = threadIdx.x; i < IVF_QCHUNK_BIN * w4; i += blockDim.x) {
            const int64_t pr = apair[i / w4];
            sq[i] = pr >= 0 ? Q[(pr / np) * w4 + (i % w4)] : make_uint4(0, 0, 0, 0);
        }
        __syncthreads();
        const int64_t r0 = lb + rch * rc, r1 = min(le, r0 + rc);
        const uint4 *myq = sq + warp * 8 * w4;
        WarpTopK<R> L[8];
        uint64_t thr[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) { L[j].init(); thr[j] = KEY_EMPTY; }
        for (int64_t base = r0; base < r1; base += 32) {
            const int64_t row = base + lane;
            const bool valid = row < r1;
            uint32_t dist[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) dist[j] = 0;
            const uint4 *rp = V + (valid ? row : r0) * w4;
#pragma unroll 4
            for (int c = 0; c < w4; ++c) {
                const uint4 x = ldg_nc_u4(rp + c);
#pragma unroll
                for (int j = 0; j < 8; ++j) dist[j] += popc4(x, myq[j * w4 + c]);
            }
            const uint32_t oid = valid ? (uint32_t)ids[row] : 0u;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const bool ok = valid && apair[warp * 8 + j] >= 0;
                L[j].offer(ok ? make_key(dist[j], oid) : KEY_EMPTY, thr[j], k);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t pr = apair[warp * 8 + j];
            if (pr >= 0) L[j].store(part + (qslot[pr / np] + slot_rel[pr] + rch) * k, k);
        }
        __syncthreads();
    }
}

// ── merge of a query's slots ──────────────────────────────────────────────
template <int R>
__global__ void ivf_merge_kernel(const uint64_t *__restrict__ part, const int64_t *__restrict__ qslot, int64_t nq,
                                 int k, int is_hamming, int64_t *__restrict__ out_idx, void *__restrict__ out_dist,
                                 int64_t *__restrict__ out_cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= nq) return;
    WarpTopK<R> L;
    L.init();
    uint64_t thr = KEY_EMPTY;
    for (int64_t sl = qslot[q]; sl < qslot[q + 1]; ++sl) {
        const uint64_t *p = part + sl * k;
        for (int j0 = 0; j0 < k; j0 += 32) {
            const int j = j0 + lane;
            const uint64_t key = (j < k) ? p[j] : KEY_EMPTY;
            if (__all_sync(0xffffffffu, key >= thr)) break;
            L.offer(key, thr, k);
        }
    }
    int cnt = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int pos = r * 32 + lane;
        const bool e = L.v[r] == KEY_EMPTY;
        cnt += __popc(__ballot_sync(0xffffffffu, pos < k && !e));
        if (pos < k) {
            out_idx[q * k + pos] = e ? -1 : (int64_t)key_idx(L.v[r]);
            if (is_hamming) reinterpret_cast<int64_t *>(out_dist)[q * k + pos] = e ? 0 : (int64_t)key_dist(L.v[r]);
            else reinterpret_cast<float *>(out_dist)[q * k + pos] = e ? 0.f : __uint_as_float(key_dist(L.v[r]));
        }
    }
    if (lane == 0 && out_cnt) out_cnt[q] = cnt;
}

__global__ void gather_rows_kernel(const float *__restrict__ X, int dp, const int32_t *__restrict__ perm, int64_t n,
                                   float *__restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int dp4 = dp >> 2;
    if (t >= n * dp4) return;
    const int64_t i = t / dp4;
    const int j = (int)(t % dp4);
    reinterpret_cast<float4 *>(out)[t] = reinterpret_cast<const float4 *>(X)[(int64_t)perm[i] * dp4 + j];
}

__global__ void gather_rows_u4_kernel(const uint4 *__restrict__ X, int w4, const int32_t *__restrict__ perm, int64_t n,
                                      uint4 *__restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * w4) return;
    const int64_t i = t / w4;
    out[t] = X[(int64_t)perm[i] * w4 + (t % w4)];
}

__global__ void i64_to_i32_kernel(const int64_t *__restrict__ a, int64_t n, int32_t *__restrict__ b) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) b[t] = (int32_t)a[t];
}

// ── shared host helpers ───────────────────────────────────────────────────
static int g_scan_blocks_l2 = 0, g_scan_blocks_bin = 0;

template <typename F>
static int dispatch_r(int k, F &&f) {
    if (k <= 32) return f(std::integral_constant<int, 1>());
    if (k <= 64) return f(std::integral_constant<int, 2>());
    if (k <= 128) return f(std::integral_constant<int, 4>());
    if (k <= 256) return f(std::integral_constant<int, 8>());
    return fail(GN_ERR_UNSUPPORTED, "IVF search supports k <= 256");
}

// Build the CSR permutation on the host: lists in `order`, rows of each list in
// ascending original index.  Returns perm (list order -> original row).
static void csr_from_labels(const std::vector<int32_t> &labels, int32_t nlab, const std::vector<int32_t> &order,
                            std::vector<int32_t> &perm, std::vector<int64_t> &off) {
    std::vector<int64_t> cnt((size_t)nlab, 0);
    for (int32_t l : labels) cnt[(size_t)l]++;
    std::vector<int64_t> start((size_t)nlab, 0);
    off.assign(order.size() + 1, 0);
    for (size_t i = 0; i < order.size(); ++i) {
        start[(size_t)order[i]] = off[i];
        off[i + 1] = off[i] + cnt[(size_t)order[i]];
    }
    perm.assign(labels.size(), 0);
    std::vector<int64_t> fillp = start;
    for (size_t i = 0; i < labels.size(); ++i) perm[(size_t)fillp[(size_t)labels[i]]++] = (int32_t)i;
}

static void top_rows_from_off(const std::vector<int64_t> &off, std::vector<int64_t> &top) {
    std::vector<int64_t> len(off.size() - 1);
    for (size_t i = 0; i + 1 < off.size(); ++i) len[i] = off[i + 1] - off[i];
    std::sort(len.begin(), len.end(), std::greater<int64_t>());
    top.assign(len.size() + 1, 0);
    for (size_t i = 0; i < len.size(); ++i) top[i + 1] = top[i] + len[i];
}

// Upper bound of the partial slots one query can own.
static int64_t max_slots_per_query(const std::vector<int64_t> &top, int np, int rc) {
    const int64_t p = std::min<int64_t>(np, (int64_t)top.size() - 1);
    return p + (top[(size_t)p] + rc - 1) / rc;
}

constexpr int64_t PLAN_SMALL_PAIRS = 16384;  // batches planned by one block
constexpr int PLAN_SMALL_LISTS = 8192;

// Bucket the (query, probe) pairs by list and plan the work items; probes
// (int32, nq*np) must be filled.  Produces boff, bucket, item_off, slot_rel,
// qslot in S.  All on the device, no host synchronisation.
int ivf_plan(IvfScratch &S, int64_t nq, int np, int nc, const int64_t *d_list_off, int rc, int qchunk,
             cudaStream_t st, int slot_rc) {
    if (slot_rc <= 0) slot_rc = rc;
    const int64_t npairs = nq * np;
    GN_TRY(S.bcnt.ensure((size_t)nc * 4));
    GN_TRY(S.fill.ensure((size_t)nc * 4));
    GN_TRY(S.boff.ensure((size_t)(nc + 1) * 8));
    GN_TRY(S.item_off.ensure((size_t)(nc + 1) * 8));
    GN_TRY(S.bucket.ensure((size_t)npairs * 8));
    GN_TRY(S.slot_rel.ensure((size_t)npairs * 8));
    GN_TRY(S.qcount.ensure((size_t)nq * 8));
    GN_TRY(S.qslot.ensure((size_t)(nq + 1) * 8));
    GN_TRY(S.counter.ensure(8));
    if (npairs <= PLAN_SMALL_PAIRS && nc <= PLAN_SMALL_LISTS) {  // one block does it all
        const size_t smem = (size_t)nc * 2 * sizeof(int32_t);
        static bool attr = false;
        if (!attr) {
            GN_CUDA_TRY(cudaFuncSetAttribute(ivf_plan_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)(PLAN_SMALL_LISTS * 2 * sizeof(int32_t))));
            attr = true;
        }
        ivf_plan_small_kernel<<<1, 1024, smem, st>>>(S.probes.as<int32_t>(), nq, np, nc, d_list_off, rc, qchunk,
                                                     slot_rc, S.bcnt.as<int32_t>(), S.boff.as<int64_t>(),
                                                     S.item_off.as<int64_t>(), S.bucket.as<int64_t>(),
                                                     S.slot_rel.as<int64_t>(), S.qcount.as<int64_t>(),
                                                     S.qslot.as<int64_t>(), S.counter.as<int64_t>());
        GN_CUDA_TRY(cudaGetLastError());
        return GN_OK;
    }
    GN_CUDA_TRY(cudaMemsetAsync(S.bcnt.p, 0, (size_t)nc * 4, st));
    GN_CUDA_TRY(cudaMemsetAsync(S.fill.p, 0, (size_t)nc * 4, st));
    GN_CUDA_TRY(cudaMemsetAsync(S.counter.p, 0, 8, st));
    const unsigned pb = (unsigned)ceil_div(npairs, 256);
    ivf_bucket_count_kernel<<<pb, 256, 0, st>>>(S.probes.as<int32_t>(), npairs, S.bcnt.as<int32_t>());
    ivf_plan_kernel<<<1, 1024, 0, st>>>(S.bcnt.as<int32_t>(), d_list_off, nc, rc, qchunk, S.boff.as<int64_t>(),
                                        S.item_off.as<int64_t>());
    ivf_bucket_fill_kernel<<<pb, 256, 0, st>>>(S.probes.as<int32_t>(), npairs, S.boff.as<int64_t>(),
                                               S.fill.as<int32_t>(), S.bucket.as<int64_t>());
    ivf_slots_kernel<<<(unsigned)ceil_div(nq, 4), 128, 0, st>>>(S.probes.as<int32_t>(), nq, np, d_list_off,
                                                                  slot_rc, S.slot_rel.as<int64_t>(),
                                                                  S.qcount.as<int64_t>());
    ivf_qscan_kernel<<<1, 1024, 0, st>>>(S.qcount.as<int64_t>(), nq, S.qslot.as<int64_t>());
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

// Plan, run the metric's scan kernel (scan_launch(grid)), merge the slots.
template <typename ScanLaunch>
static int ivf_run_lists(IvfScratch &S, int64_t nq, int np, int nc, const int64_t *d_list_off, int rc, int qchunk,
                         int k, int is_hamming, int64_t *d_idx, void *d_dist, int64_t *d_cnt, int grid,
                         ScanLaunch &&scan_launch, cudaStream_t st) {
    GN_TRY(ivf_plan(S, nq, np, nc, d_list_off, rc, qchunk, st));
    timing_begin(st, is_hamming ? "ivfbin_scan_kernel" : "ivf_scan_kernel");
    GN_TRY(scan_launch(grid));
    timing_end(st);
    return dispatch_r(k, [&](auto RC) {
        constexpr int R = decltype(RC)::value;
        ivf_merge_kernel<R><<<(unsigned)ceil_div(nq, 4), 128, 0, st>>>(S.part.as<uint64_t>(), S.qslot.as<int64_t>(),
                                                                       nq, k, is_hamming, d_idx, d_dist, d_cnt);
        return GN_OK;
    });
}

int64_t ivf_max_slots_per_query(const std::vector<int64_t> &top, int np, int rc) {
    return max_slots_per_query(top, np, rc);
}

// ── float IVF: build ──────────────────────────────────────────────────────
static int ivfl2_build_from_labels(gn_index *ix, const float *dX, int64_t n, int d, int dp,
                                   const std::vector<float> &hcent, int32_t ncent, const std::vector<int32_t> &labels,
                                   cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    // live clusters ordered by descending size, ties by cluster id
    std::vector<int64_t> cnt((size_t)ncent, 0);
    for (int32_t l : labels) {
        if (l < 0 || l >= ncent) return fail(GN_ERR_INVALID, "label out of range");
        cnt[(size_t)l]++;
    }
    std::vector<int32_t> order;
    for (int32_t c = 0; c < ncent; ++c)
        if (cnt[(size_t)c] > 0) order.push_back(c);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return cnt[(size_t)a] > cnt[(size_t)b]; });
    std::vector<int32_t> perm;
    csr_from_labels(labels, ncent, order, perm, S.h_off);
    S.nc = (int32_t)order.size();
    S.K = 0;  // BF16 copy for the tensor-core engine is rebuilt on first use
    S.cfg++;
    S.n = n;
    S.d = d;
    S.dp = dp;
    std::vector<float> cent((size_t)S.nc * dp, 0.f);
    for (int32_t i = 0; i < S.nc; ++i)
        std::memcpy(cent.data() + (size_t)i * dp, hcent.data() + (size_t)order[(size_t)i] * dp, (size_t)dp * 4);
    GN_TRY(S.cent.ensure(cent.size() * 4));
    GN_TRY(S.cnorm.ensure((size_t)S.nc * 4));
    GN_TRY(S.list_off.ensure(S.h_off.size() * 8));
    GN_TRY(S.vecs.ensure((size_t)n * dp * 4));
    GN_TRY(S.vnorm.ensure((size_t)n * 4));
    GN_TRY(S.ids.ensure((size_t)n * 4));
    GN_CUDA_TRY(cudaMemcpyAsync(S.cent.p, cent.data(), cent.size() * 4, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.list_off.p, S.h_off.data(), S.h_off.size() * 8, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.ids.p, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
    gather_rows_kernel<<<(unsigned)ceil_div(n * (dp / 4), 256), 256, 0, st>>>(dX, dp, S.ids.as<int32_t>(), n,
                                                                             S.vecs.as<float>());
    row_norms(S.vecs.as<float>(), n, dp, S.vnorm.as<float>(), st);
    row_norms(S.cent.as<float>(), S.nc, dp, S.cnorm.as<float>(), st);
    top_rows_from_off(S.h_off, S.top_rows);
    S.rc = (int)std::max<int64_t>(GT_BN, std::min<int64_t>(8192, round_up((512 * 1024) / dp, GT_BN)));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

// Coarse probing of a float IVF: qn = |q|^2 and the np nearest lists of each
// query.  Small batches split the centroids over more CTAs.  With keep_keys
// the sorted partial key lists stay in T.cpart (nsplit of them per query) and
// probes are not written; otherwise probes get the merged list ids.
int ivfl2_coarse_run(gn_index *ix, const float *dQ, int64_t nq, int np, bool keep_keys, int *nsplit_out,
                     cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    IvfScratch &T = S.s;
    GN_TRY(T.qn.ensure((size_t)nq * 4));
    GN_TRY(T.probes.ensure((size_t)nq * np * 4));
    row_norms(dQ, nq, S.dp, T.qn.as<float>(), st);
    const int64_t qblocks = ceil_div(nq, GT_BM);
    int nsplit = 1;
    while (qblocks * nsplit * 2 <= dev_info().num_sms && (int64_t)GT_BN * nsplit * 2 <= S.nc) nsplit *= 2;
    const int cps = (int)round_up(ceil_div(S.nc, nsplit), GT_BN);
    nsplit = (int)ceil_div(S.nc, cps);
    const bool use_part = keep_keys || nsplit > 1;
    if (use_part) GN_TRY(T.cpart.ensure((size_t)nq * nsplit * np * 8));
    if (nsplit_out) *nsplit_out = nsplit;
    return dispatch_r(np, [&](auto RC) {
        constexpr int R = decltype(RC)::value;
        ivf_coarse_kernel<R><<<dim3((unsigned)qblocks, (unsigned)nsplit), GT_THREADS, 0, st>>>(
            dQ, T.qn.as<float>(), nq, S.dp, S.cent.as<float>(), S.cnorm.as<float>(), S.nc, np, cps,
            T.probes.as<int32_t>(), use_part ? T.cpart.as<uint64_t>() : nullptr);
        if (use_part && !keep_keys)
            coarse_merge_kernel<R><<<(unsigned)ceil_div(nq, 4), 128, 0, st>>>(T.cpart.as<uint64_t>(), nsplit, np, nq,
                                                                              T.probes.as<int32_t>(), nullptr);
        return GN_OK;
    });
}

int ivfl2_coarse(gn_index *ix, const float *dQ, int64_t nq, int np, cudaStream_t st) {
    return ivfl2_coarse_run(ix, dQ, nq, np, false, nullptr, st);
}

// The np nearest lists of each query as sorted keys (squared distance, list).
int ivfl2_coarse_sorted_keys(gn_index *ix, const float *dQ, int64_t nq, int np, uint64_t *keys, cudaStream_t st) {
    int nsplit = 1;
    GN_TRY(ivfl2_coarse_run(ix, dQ, nq, np, true, &nsplit, st));
    IvfScratch &T = ix->ivfl2->s;
    return dispatch_r(np, [&](auto RC) {
        constexpr int R = decltype(RC)::value;
        coarse_merge_kernel<R><<<(unsigned)ceil_div(nq, 4), 128, 0, st>>>(T.cpart.as<uint64_t>(), nsplit, np, nq,
                                                                          nullptr, keys);
        return GN_OK;
    });
}

// Probes of a batch: the learned prober when one is attached (up to 64 lists,
// -1 padded), else the fixed n_probe nearest lists.  Returns the probe width.
int ivfl2_probes(gn_index *ix, const float *dQ, int64_t nq, int *np_out, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    if (S.prober) {
        if (S.nc < PROBER_CAND) return fail(GN_ERR_INVALID, "learned probing needs at least 64 lists");
        GN_TRY(S.s.nprobed.ensure((size_t)nq * 4));
        GN_TRY(prober_apply(S.prober, ix, dQ, nq, S.prober_tau, S.s.probes.as<int32_t>(), S.s.nprobed.as<int32_t>(),
                            st));
        *np_out = PROBER_CAND;
        return GN_OK;
    }
    const int np = std::min<int32_t>(S.nprobe, S.nc);
    *np_out = np;
    return ivfl2_coarse(ix, dQ, nq, np, st);
}

// ── float IVF: search on device buffers ───────────────────────────────────
static int ivfl2_scan_fp32(gn_index *ix, const float *dQ, int64_t nq, int np, int k, int64_t *d_idx, float *d_dist,
                           int64_t *d_cnt, cudaStream_t st);

int ivfl2_search_core(gn_index *ix, const float *dQ, int64_t nq, int k, int64_t *d_idx, float *d_dist,
                      int64_t *d_cnt, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    IvfScratch &T = S.s;
    const int np = std::min<int32_t>(S.nprobe, S.nc);
    if (np <= 0) return fail(GN_ERR_INVALID, "n_probe must be positive");
    if (np > 256) return fail(GN_ERR_UNSUPPORTED, "n_probe > 256 is not supported");
    if (nq == 0) return GN_OK;
    if (S.mode == 1) return ivfl2_search_tc(ix, dQ, nq, k, d_idx, d_dist, d_cnt, st);
    int npw = np;
    GN_TRY(ivfl2_probes(ix, dQ, nq, &npw, st));
    return ivfl2_scan_fp32(ix, dQ, nq, npw, k, d_idx, d_dist, d_cnt, st);
}

static int ivfl2_scan_fp32(gn_index *ix, const float *dQ, int64_t nq, int np, int k, int64_t *d_idx, float *d_dist,
                           int64_t *d_cnt, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    IvfScratch &T = S.s;
    const int64_t slots = nq * max_slots_per_query(S.top_rows, np, S.rc);
    GN_TRY(T.part.ensure((size_t)slots * k * 8));
    if (!g_scan_blocks_l2) {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ivf_scan_kernel<1>, GT_THREADS, 0);
        g_scan_blocks_l2 = std::max(1, per) * dev_info().num_sms;
    }
    return ivf_run_lists(
        T, nq, np, S.nc, S.list_off.as<int64_t>(), S.rc, IVF_QCHUNK_L2, k, 0, d_idx, d_dist, d_cnt,
        g_scan_blocks_l2,
        [&](int grid) {
            return dispatch_r(k, [&](auto RC) {
                constexpr int R = decltype(RC)::value;
                ivf_scan_kernel<R><<<grid, GT_THREADS, 0, st>>>(
                    dQ, T.qn.as<float>(), np, S.dp, S.vecs.as<float>(), S.vnorm.as<float>(), S.ids.as<int32_t>(),
                    S.list_off.as<int64_t>(), S.nc, T.boff.as<int64_t>(), T.bucket.as<int64_t>(),
                    T.item_off.as<int64_t>(), S.rc, T.qslot.as<int64_t>(), T.slot_rel.as<int64_t>(), k,
                    T.counter.as<int>(), T.part.as<uint64_t>());
                return GN_OK;
            });
        },
        st);
}

// ── binary IVF ────────────────────────────────────────────────────────────
static int ivfbin_search_dev(gn_index *ix, const uint8_t *dQ, int64_t nq, int k, int64_t *d_idx, int64_t *d_dist,
                             int64_t *d_cnt, cudaStream_t st) {
    IvfBinState &S = *ix->ivfbin;
    IvfScratch &T = S.s;
    const int np = std::min<int32_t>(S.nprobe, S.kc);
    if (nq == 0) return GN_OK;
    if (np <= 0) {  // nothing probed: empty results
        GN_CUDA_TRY(cudaMemsetAsync(d_cnt, 0, (size_t)nq * 8, st));
        GN_CUDA_TRY(cudaMemsetAsync(d_idx, 0xff, (size_t)nq * k * 8, st));
        GN_CUDA_TRY(cudaMemsetAsync(d_dist, 0, (size_t)nq * k * 8, st));
        return GN_OK;
    }
    if (np > FLAT_MAX_K_WARP) return fail(GN_ERR_UNSUPPORTED, "nprobe > 256 is not supported");
    // coarse: exact Hamming scan over the centroids, nearest (distance, id) first
    FlatScanArgs a;
    a.metric = M_HAMMING;
    a.db = S.cent.p;
    a.n = S.kc;
    a.d = S.nbytes;
    a.stride4 = S.w4;
    a.q = dQ;
    a.nq = nq;
    a.k = np;
    GN_TRY(T.probes64.ensure((size_t)nq * np * 8));
    GN_TRY(T.pdist.ensure((size_t)nq * np * 8));
    GN_TRY(T.probes.ensure((size_t)nq * np * 4));
    a.out_idx = T.probes64.as<int64_t>();
    a.out_dist = T.pdist.p;
    flat_plan(a);
    GN_TRY(T.cpart.ensure(flat_part_bytes(a)));
    GN_TRY(flat_launch(a, T.cpart.as<uint64_t>(), st));
    i64_to_i32_kernel<<<(unsigned)ceil_div(nq * np, 256), 256, 0, st>>>(T.probes64.as<int64_t>(), nq * np,
                                                                      T.probes.as<int32_t>());
    const int64_t slots = nq * max_slots_per_query(S.top_rows, np, S.rc);
    GN_TRY(T.part.ensure((size_t)slots * k * 8));
    const size_t smem = (size_t)IVF_QCHUNK_BIN * S.w4 * 16;
    if (!g_scan_blocks_bin) {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ivfbin_scan_kernel<1>, 128, 4096);
        g_scan_blocks_bin = std::max(1, per) * dev_info().num_sms;
    }
    return ivf_run_lists(
        T, nq, np, S.kc, S.list_off.as<int64_t>(), S.rc, IVF_QCHUNK_BIN, k, 1, d_idx, d_dist, d_cnt,
        g_scan_blocks_bin,
        [&](int grid) {
            return dispatch_r(k, [&](auto RC) {
                constexpr int R = decltype(RC)::value;
                if (smem > 48 * 1024)
                    cudaFuncSetAttribute(ivfbin_scan_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                ivfbin_scan_kernel<R><<<grid, 128, smem, st>>>(
                    reinterpret_cast<const uint4 *>(dQ), S.w4, np, S.vecs.as<uint4>(), S.ids.as<int32_t>(),
                    S.list_off.as<int64_t>(), S.kc, T.boff.as<int64_t>(), T.bucket.as<int64_t>(),
                    T.item_off.as<int64_t>(), S.rc, T.qslot.as<int64_t>(), T.slot_rel.as<int64_t>(), k,
                    T.counter.as<int>(), T.part.as<uint64_t>());
                return GN_OK;
            });
        },
        st);
}

void ivf_free(gn_index *ix) {
    if (ix->ivfl2) delete ix->ivfl2->graphs;
    delete ix->ivfl2;
    delete ix->ivfbin;
    ix->ivfl2 = nullptr;
    ix->ivfbin = nullptr;
}

}  // namespace gn

using namespace gn;

// After a synchronised search: a tensor-core pipeline wait that ran out set
// the index's error word; report it (and clear it, so the next search runs).
// End of a blocking search: one stream synchronisation for the results and the
// tensor-core engine's error word.
static int ivfl2_finish(gn_index *ix, cudaStream_t st) {
    IvfL2State &S = *ix->ivfl2;
    return finish_blocking(ix, (S.mode == 1 && S.err.p) ? S.err.as<int>() : nullptr, st,
                           "tensor-core IVF search: a pipeline wait timed out; results are invalid");
}

extern "C" {

int gn_kmeans_l2(const float *data, int64_t n, int64_t d, int64_t k, int64_t max_iter, uint32_t seed,
                 int32_t *labels, float *centroids, int64_t *iters_out) {
    if (!data || !labels || !centroids) return fail(GN_ERR_INVALID, "kmeans_l2: NULL pointer");
    if (n <= 0 || d <= 0) return fail(GN_ERR_INVALID, "kmeans_l2: data must be a non-empty (N, D) array");
    if (k <= 0 || k > n) return fail(GN_ERR_INVALID, "kmeans_l2: k must be between 1 and N");
    if (n >= 0x7fffffffLL) return fail(GN_ERR_UNSUPPORTED, "kmeans_l2: at most 2^31-2 rows");
    cudaStream_t st;
    GN_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct Guard {
        cudaStream_t s;
        ~Guard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
    } g{st};
    const int dp = (int)round_up(d, 16);
    DBuf X, C, cn, L;
    GN_TRY(upload_rows(X, data, n, d * 4, dp / 4, st));
    GN_TRY(C.ensure((size_t)k * dp * 4));
    GN_TRY(cn.ensure((size_t)k * 4));
    GN_TRY(L.ensure((size_t)n * 4));
    GN_TRY(kmeans_l2_device(X.as<float>(), n, (int)d, dp, k, max_iter, seed, C.as<float>(), cn.as<float>(),
                            L.as<int32_t>(), iters_out, st));
    GN_CUDA_TRY(cudaMemcpyAsync(labels, L.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaMemcpy2DAsync(centroids, (size_t)d * 4, C.p, (size_t)dp * 4, (size_t)d * 4, (size_t)k,
                                  cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    return GN_OK;
}

int gn_ivfl2_create(int32_t n_clusters, int32_t n_probe, gn_index **out) {
    if (!out) return fail(GN_ERR_INVALID, "out is NULL");
    if (n_clusters <= 0) return fail(GN_ERR_INVALID, "n_clusters must be positive");
    if (n_probe <= 0) return fail(GN_ERR_INVALID, "n_probe must be positive");
    gn_index *ix = new gn_index();
    ix->kind = K_IVFL2;
    ix->metric = GN_METRIC_L2;
    ix->ivfl2 = new IvfL2State();
    ix->ivfl2->nlist_req = n_clusters;
    ix->ivfl2->nprobe = std::min(n_probe, n_clusters);
    *out = ix;
    return GN_OK;
}

static int ivfl2_check(gn_index *ix) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    return GN_OK;
}

// The lists of an index with live forks, or of a fork, stay as they are.
static int ivfl2_check_rebuild(gn_index *ix) {
    if (ix->fork_parent) return fail(GN_ERR_INVALID, "a fork shares its parent's lists: call set() on a new index");
    if (has_forks(ix)) return fail(GN_ERR_INVALID, "the index has live forks that share its lists: destroy them first");
    return GN_OK;
}

int gn_ivfl2_set(gn_index *ix, const float *data, int64_t n, int64_t d) {
    GN_TRY(ivfl2_check(ix));
    GN_TRY(ivfl2_check_rebuild(ix));
    if (n <= 0 || d <= 0 || !data) return fail(GN_ERR_INVALID, "data must be a 2-D array of shape (N, D)");
    if (n >= 0x7fffffffLL) return fail(GN_ERR_UNSUPPORTED, "at most 2^31-2 rows");
    std::lock_guard<std::mutex> lk(ix->mu);
    GN_TRY(make_stream(ix));
    cudaStream_t st = ix->stream;
    IvfL2State &S = *ix->ivfl2;
    S.nc = 0;
    const int dp = (int)round_up(d, 16);
    const int64_t k = std::min<int64_t>(S.nlist_req, n);
    DBuf X, C, cn, L;
    GN_TRY(upload_rows(X, data, n, d * 4, dp / 4, st));
    GN_TRY(C.ensure((size_t)k * dp * 4));
    GN_TRY(cn.ensure((size_t)k * 4));
    GN_TRY(L.ensure((size_t)n * 4));
    GN_TRY(kmeans_l2_device(X.as<float>(), n, (int)d, dp, k, 100, 42, C.as<float>(), cn.as<float>(), L.as<int32_t>(),
                            nullptr, st));
    std::vector<int32_t> labels((size_t)n);
    std::vector<float> hc((size_t)k * dp);
    GN_CUDA_TRY(cudaMemcpyAsync(labels.data(), L.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaMemcpyAsync(hc.data(), C.p, hc.size() * 4, cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    ix->n = n;
    ix->dim = d;
    return ivfl2_build_from_labels(ix, X.as<float>(), n, (int)d, dp, hc, (int32_t)k, labels, st);
}

int gn_ivfl2_set_assigned(gn_index *ix, const float *data, int64_t n, int64_t d, const float *centroids,
                          int32_t n_centroids, const int32_t *labels) {
    GN_TRY(ivfl2_check(ix));
    GN_TRY(ivfl2_check_rebuild(ix));
    if (n <= 0 || d <= 0 || !data || !centroids || !labels || n_centroids <= 0)
        return fail(GN_ERR_INVALID, "set_assigned: bad arguments");
    std::lock_guard<std::mutex> lk(ix->mu);
    GN_TRY(make_stream(ix));
    cudaStream_t st = ix->stream;
    const int dp = (int)round_up(d, 16);
    DBuf X;
    GN_TRY(upload_rows(X, data, n, d * 4, dp / 4, st));
    std::vector<float> hc((size_t)n_centroids * dp, 0.f);
    for (int32_t c = 0; c < n_centroids; ++c) std::memcpy(hc.data() + (size_t)c * dp, centroids + (size_t)c * d, (size_t)d * 4);
    std::vector<int32_t> lab(labels, labels + n);
    ix->n = n;
    ix->dim = d;
    return ivfl2_build_from_labels(ix, X.as<float>(), n, (int)d, dp, hc, n_centroids, lab, st);
}

// A fork: a second search context over the parent's lists.  It views the
// parent's read-only data (centroids, CSR offsets, FP32 and tiled BF16 rows,
// ids) and owns everything a search writes (scratch, error word, unit
// counters, stream, captured graphs), so searches on the parent and its forks
// run concurrently on different streams.  Settings (n_probe, engine,
// shortlist, prober, tuning table) start as copies of the parent's and are
// the fork's own from then on.
int gn_ivfl2_fork(gn_index *parent, gn_index **out) {
    GN_TRY(ivfl2_check(parent));
    if (!out) return fail(GN_ERR_INVALID, "out is NULL");
    if (parent->fork_parent) return fail(GN_ERR_INVALID, "fork the parent index, not a fork");
    std::lock_guard<std::mutex> lk(parent->mu);
    IvfL2State &P = *parent->ivfl2;
    if (P.nc == 0) return fail(GN_ERR_EMPTY, "Index is empty — call set() first");
    GN_TRY(make_stream(parent));
    if (P.K == 0) GN_TRY(ivfl2_prepare_tc(parent, parent->stream));  // tiled BF16 rows, shared from here on
    GN_CUDA_TRY(cudaStreamSynchronize(parent->stream));
    gn_index *ix = new gn_index();
    ix->kind = K_IVFL2;
    ix->metric = parent->metric;
    ix->n = parent->n;
    ix->dim = parent->dim;
    ix->ivfl2 = new IvfL2State();
    IvfL2State &S = *ix->ivfl2;
    S.nlist_req = P.nlist_req;
    S.nprobe = P.nprobe;
    S.d = P.d;
    S.dp = P.dp;
    S.nc = P.nc;
    S.n = P.n;
    S.h_off = P.h_off;
    S.top_rows = P.top_rows;
    S.rc = P.rc;
    S.mode = P.mode;
    S.shortlist = P.shortlist;
    S.K = P.K;
    S.x16_rows = P.x16_rows;
    S.prober = P.prober;
    S.prober_tau = P.prober_tau;
    for (int b = 0; b < 7; ++b) S.tune[b] = P.tune[b];
    S.cent.view(P.cent);
    S.cnorm.view(P.cnorm);
    S.list_off.view(P.list_off);
    S.vecs.view(P.vecs);
    S.vnorm.view(P.vnorm);
    S.ids.view(P.ids);
    S.x16.view(P.x16);
    S.xoff.view(P.xoff);
    S.c16.view(P.c16);
    S.rho.view(P.rho);
    S.xmax = P.xmax;
    // the fork's own error word and unit counters
    int rc = S.err.ensure(4);
    if (rc == GN_OK) rc = S.sched.ensure(2 * sizeof(unsigned long long));
    if (rc == GN_OK && cudaMemset(S.err.p, 0, 4) != cudaSuccess) rc = fail(GN_ERR_CUDA, "fork: clearing the error word");
    if (rc != GN_OK) {
        delete ix;
        return rc;
    }
    fork_attach(ix, parent);
    *out = ix;
    return GN_OK;
}

int gn_ivfl2_search_knn_device(gn_index *ix, const float *d_queries, int64_t nq, int64_t k, int64_t *d_idx,
                               float *d_dist, int64_t *d_cnt, void *stream) {
    GN_TRY(ivfl2_check(ix));
    if (ix->ivfl2->nc == 0) return fail(GN_ERR_EMPTY, "Index is empty — call set() first");
    if (k <= 0) return fail(GN_ERR_INVALID, "k must be positive");
    std::lock_guard<std::mutex> lk(ix->mu);
    IvfL2State &S = *ix->ivfl2;
    if (S.graphs && nq > 0 && nq <= S.graphs->max_batch && k == S.graphs->k && !timing_on())
        return ivfl2_search_graph(ix, d_queries, false, nq, (int)k, d_idx, d_dist, d_cnt, false, (cudaStream_t)stream);
    const cudaStream_t st = (cudaStream_t)stream;
    const float *dQ = d_queries;
    if (S.d != S.dp || ((uintptr_t)d_queries & 15)) {  // kernels read 16-byte aligned rows at the padded pitch
        GN_TRY(upload_rows(S.s.q, d_queries, nq, S.d * 4, S.dp / 4, st, true));
        dQ = S.s.q.as<float>();
    }
    GN_TRY(ivfl2_search_core(ix, dQ, nq, (int)k, d_idx, d_dist, d_cnt, st));
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

int gn_ivfl2_search_knn(gn_index *ix, const float *queries, int64_t nq, int64_t k, int64_t *out_idx, float *out_dist,
                        int64_t *out_cnt) {
    GN_TRY(ivfl2_check(ix));
    IvfL2State &S = *ix->ivfl2;
    if (S.nc == 0) return fail(GN_ERR_EMPTY, "Index is empty — call set() first");
    if (k <= 0) return fail(GN_ERR_INVALID, "k must be positive");
    if (nq < 0 || (nq > 0 && (!queries || !out_idx || !out_dist || !out_cnt)))
        return fail(GN_ERR_INVALID, "bad query arguments");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (nq == 0) return GN_OK;
    begin_blocking(ix);
    if (S.graphs && nq <= S.graphs->max_batch && k == S.graphs->k && !timing_on() && !S.drill) {
        GN_TRY(ivfl2_search_graph(ix, queries, true, nq, (int)k, out_idx, out_dist, out_cnt, true, ix->stream));
        return ivfl2_finish(ix, ix->stream);
    }
    cudaStream_t st = ix->stream;
    GN_TRY(upload_queries(ix, S.s.q, queries, nq, S.d * 4, S.dp / 4, st));
    GN_TRY(ix->out_idx.ensure((size_t)nq * k * 8));
    GN_TRY(ix->out_dist.ensure((size_t)nq * k * 4));
    GN_TRY(ix->part.ensure((size_t)nq * 8));
    GN_TRY(ivfl2_search_core(ix, S.s.q.as<float>(), nq, (int)k, ix->out_idx.as<int64_t>(), ix->out_dist.as<float>(),
                            ix->part.as<int64_t>(), st));
    GN_TRY(download_result(ix, out_idx, ix->out_idx.p, (size_t)nq * k * 8, st));
    GN_TRY(download_result(ix, out_dist, ix->out_dist.p, (size_t)nq * k * 4, st));
    GN_TRY(download_result(ix, out_cnt, ix->part.p, (size_t)nq * 8, st));
    GN_CUDA_TRY(cudaGetLastError());
    return ivfl2_finish(ix, st);
}

int gn_ivfl2_set_n_probe(gn_index *ix, int32_t n_probe) {
    GN_TRY(ivfl2_check(ix));
    if (n_probe <= 0) return fail(GN_ERR_INVALID, "n_probe must be positive");
    std::lock_guard<std::mutex> lk(ix->mu);
    ix->ivfl2->nprobe = n_probe;
    ix->ivfl2->cfg++;
    return GN_OK;
}

int gn_ivfl2_info(gn_index *ix, int32_t *n_clusters_built, int32_t *n_probe, int64_t *n, int64_t *d) {
    GN_TRY(ivfl2_check(ix));
    if (n_clusters_built) *n_clusters_built = ix->ivfl2->nc;
    if (n_probe) *n_probe = ix->ivfl2->nprobe;
    if (n) *n = ix->ivfl2->n;
    if (d) *d = ix->ivfl2->d;
    return GN_OK;
}

int gn_ivfl2_export(gn_index *ix, float *centroids, int64_t *offsets, int64_t *ids) {
    GN_TRY(ivfl2_check(ix));
    IvfL2State &S = *ix->ivfl2;
    std::lock_guard<std::mutex> lk(ix->mu);
    if (S.nc == 0) return fail(GN_ERR_EMPTY, "index is empty");
    cudaStream_t st = ix->stream;
    if (centroids)
        GN_CUDA_TRY(cudaMemcpy2DAsync(centroids, (size_t)S.d * 4, S.cent.p, (size_t)S.dp * 4, (size_t)S.d * 4,
                                      (size_t)S.nc, cudaMemcpyDeviceToHost, st));
    if (offsets) std::memcpy(offsets, S.h_off.data(), S.h_off.size() * 8);
    if (ids) {
        std::vector<int32_t> h((size_t)S.n);
        GN_CUDA_TRY(cudaMemcpyAsync(h.data(), S.ids.p, (size_t)S.n * 4, cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        for (int64_t i = 0; i < S.n; ++i) ids[i] = h[(size_t)i];
    }
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    return GN_OK;
}

// ── binary IVF C ABI ──────────────────────────────────────────────────────
int gn_ivfbin_create(int32_t nlist, int32_t nprobe, int32_t max_iter, uint32_t seed, gn_index **out) {
    if (!out) return fail(GN_ERR_INVALID, "out is NULL");
    if (nlist <= 0) return fail(GN_ERR_INVALID, "nlist must be positive");
    gn_index *ix = new gn_index();
    ix->kind = K_IVFBIN;
    ix->metric = GN_METRIC_HAMMING;
    ix->ivfbin = new IvfBinState();
    ix->ivfbin->nlist = nlist;
    ix->ivfbin->nprobe = nprobe;
    ix->ivfbin->max_iter = max_iter;
    ix->ivfbin->seed = seed;
    *out = ix;
    return GN_OK;
}

static int ivfbin_check(gn_index *ix) {
    if (!ix || ix->kind != K_IVFBIN || !ix->ivfbin) return fail(GN_ERR_INVALID, "not an IVFFlatBinary index");
    return GN_OK;
}

int gn_ivfbin_set(gn_index *ix, const uint8_t *data, int64_t n, int64_t nbytes) {
    GN_TRY(ivfbin_check(ix));
    IvfBinState &S = *ix->ivfbin;
    if (n < 0 || (n > 0 && (!data || nbytes <= 0))) return fail(GN_ERR_INVALID, "bad data shape");
    if (n >= 0x7fffffffLL) return fail(GN_ERR_UNSUPPORTED, "at most 2^31-2 rows");
    std::lock_guard<std::mutex> lk(ix->mu);
    GN_TRY(make_stream(ix));
    cudaStream_t st = ix->stream;
    S.n = 0;
    S.kc = 0;
    ix->n = 0;
    if (n == 0) return GN_OK;  // the reference clears the index on an empty set
    S.nbytes = (int)nbytes;
    S.w4 = (int)ceil_div(nbytes, 16);
    const size_t row = (size_t)S.w4 * 16;
    S.kc = (int32_t)std::min<int64_t>(S.nlist, n);
    DBuf X, L;
    GN_TRY(upload_rows(X, data, n, nbytes, S.w4, st));
    GN_TRY(S.cent.ensure((size_t)S.kc * row));
    GN_TRY(L.ensure((size_t)n * 4));
    GN_TRY(kmeans_bin_device(X.as<uint8_t>(), n, (int)nbytes, S.w4, S.kc, S.max_iter, S.seed, S.cent.as<uint8_t>(),
                             L.as<int32_t>(), st));
    S.h_labels.resize((size_t)n);
    GN_CUDA_TRY(cudaMemcpyAsync(S.h_labels.data(), L.p, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<int32_t> order((size_t)S.kc);
    std::iota(order.begin(), order.end(), 0);
    std::vector<int32_t> perm;
    csr_from_labels(S.h_labels, S.kc, order, perm, S.h_off);
    GN_TRY(S.vecs.ensure((size_t)n * row));
    GN_TRY(S.ids.ensure((size_t)n * 4));
    GN_TRY(S.list_off.ensure(S.h_off.size() * 8));
    GN_CUDA_TRY(cudaMemcpyAsync(S.ids.p, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.list_off.p, S.h_off.data(), S.h_off.size() * 8, cudaMemcpyHostToDevice, st));
    gather_rows_u4_kernel<<<(unsigned)ceil_div(n * S.w4, 256), 256, 0, st>>>(X.as<uint4>(), S.w4, S.ids.as<int32_t>(),
                                                                             n, S.vecs.as<uint4>());
    top_rows_from_off(S.h_off, S.top_rows);
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    GN_CUDA_TRY(cudaGetLastError());
    S.n = n;
    ix->n = n;
    ix->dim = nbytes;
    return GN_OK;
}

int gn_ivfbin_search_knn(gn_index *ix, const uint8_t *queries, int64_t nq, int64_t k, int64_t *out_idx,
                         int64_t *out_dist, int64_t *out_cnt) {
    GN_TRY(ivfbin_check(ix));
    IvfBinState &S = *ix->ivfbin;
    if (k <= 0) return fail(GN_ERR_INVALID, "k must be positive");
    if (nq < 0 || (nq > 0 && (!queries || !out_idx || !out_dist || !out_cnt)))
        return fail(GN_ERR_INVALID, "bad query arguments");
    std::lock_guard<std::mutex> lk(ix->mu);
    if (nq == 0) return GN_OK;
    if (S.n == 0) {  // searching an empty index yields empty rows
        for (int64_t i = 0; i < nq; ++i) out_cnt[i] = 0;
        return GN_OK;
    }
    cudaStream_t st = ix->stream;
    begin_blocking(ix);
    GN_TRY(upload_queries(ix, S.s.q, queries, nq, S.nbytes, S.w4, st));
    GN_TRY(ix->out_idx.ensure((size_t)nq * k * 8));
    GN_TRY(ix->out_dist.ensure((size_t)nq * k * 8));
    GN_TRY(ix->part.ensure((size_t)nq * 8));
    GN_TRY(ivfbin_search_dev(ix, S.s.q.as<uint8_t>(), nq, (int)k, ix->out_idx.as<int64_t>(),
                             ix->out_dist.as<int64_t>(), ix->part.as<int64_t>(), st));
    GN_TRY(download_result(ix, out_idx, ix->out_idx.p, (size_t)nq * k * 8, st));
    GN_TRY(download_result(ix, out_dist, ix->out_dist.p, (size_t)nq * k * 8, st));
    GN_TRY(download_result(ix, out_cnt, ix->part.p, (size_t)nq * 8, st));
    GN_TRY(finish_blocking(ix, nullptr, st, ""));
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

int gn_ivfbin_get_params(gn_index *ix, int32_t *nlist, int32_t *nprobe) {
    GN_TRY(ivfbin_check(ix));
    if (nlist) *nlist = ix->ivfbin->nlist;
    if (nprobe) *nprobe = ix->ivfbin->nprobe;
    return GN_OK;
}

int gn_ivfbin_set_nprobe(gn_index *ix, int32_t nprobe) {
    GN_TRY(ivfbin_check(ix));
    ix->ivfbin->nprobe = nprobe;
    return GN_OK;
}

int gn_ivfbin_export(gn_index *ix, uint8_t *centroids, int32_t *labels, int32_t *k_out) {
    GN_TRY(ivfbin_check(ix));
    IvfBinState &S = *ix->ivfbin;
    std::lock_guard<std::mutex> lk(ix->mu);
    if (k_out) *k_out = S.kc;
    if (S.n == 0) return GN_OK;
    if (centroids)
        GN_CUDA_TRY(cudaMemcpy2DAsync(centroids, (size_t)S.nbytes, S.cent.p, (size_t)S.w4 * 16, (size_t)S.nbytes,
                                      (size_t)S.kc, cudaMemcpyDeviceToHost, ix->stream));
    if (labels) std::memcpy(labels, S.h_labels.data(), (size_t)S.n * 4);
    GN_CUDA_TRY(cudaStreamSynchronize(ix->stream));
    return GN_OK;
}

}  // extern "C"
