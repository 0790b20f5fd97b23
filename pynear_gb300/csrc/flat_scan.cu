// flat_scan.cu — exact exhaustive k-NN scans (Hamming and float metrics).
//
// Work decomposition: the query set is cut into groups of WARPS*QW queries and
// the database into n_slices row slices; one CTA handles one (slice, group)
// unit.  Units are numbered slice-major so that the CTAs resident at the same
// time read the same slice and share it through L2.  Each warp owns QW queries;
// lane l scores row base+l against all of them (the row stays in registers,
// query words come from shared memory as broadcasts), then offers the keys to
// the warp's register top-k lists.  Each (query, slice) writes its sorted k
// keys to a partial buffer; flat_merge_kernel (flat_merge_split_kernel for
// small batches) reduces the slices.
//
// Reference semantics (pynear/include/VPTree.hpp:143-191): exact k nearest rows
// per query; here ties go to the lower row index.
#include "distance.cuh"
#include "flat_scan.cuh"
#include "tc_sm100.cuh"
#include "timing.cuh"
#include "tmap.cuh"
#include "topk.cuh"

namespace gn {

// ── Hamming scan ───────────────────────────────────────────────────────────
// db: n rows of w4 uint4 words.  q: nq rows, same layout.
template <int QW, int R>
__global__ void __launch_bounds__(128) hamming_scan_kernel(const uint4 *__restrict__ db, int64_t n, int w4,
                                                           const uint4 *__restrict__ q, int64_t nq, int k,
                                                           int n_slices, int64_t slice_rows, int n_groups,
                                                           uint64_t *__restrict__ part) {
    extern __shared__ uint4 sq[];  // [WARPS*QW][w4]
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int unit = blockIdx.x;
    const int slice = unit / n_groups, group = unit % n_groups;
    const int64_t q0 = (int64_t)group * warps * QW;

    for (int i = threadIdx.x; i < warps * QW * w4; i += blockDim.x) {
        int64_t qi = q0 + i / w4;
        sq[i] = (qi < nq) ? q[qi * w4 + (i % w4)] : make_uint4(0, 0, 0, 0);
    }
    __syncthreads();

    const int64_t r0 = (int64_t)slice * slice_rows;
    const int64_t r1 = min(n, r0 + slice_rows);
    const uint4 *myq = sq + warp * QW * w4;

    WarpTopK<R> lists[QW];
    uint64_t thr[QW];
#pragma unroll
    for (int j = 0; j < QW; ++j) { lists[j].init(); thr[j] = KEY_EMPTY; }

    for (int64_t base = r0; base < r1; base += 32) {
        const int64_t row = base + lane;
        const bool valid = row < r1;
        uint32_t dist[QW];
#pragma unroll
        for (int j = 0; j < QW; ++j) dist[j] = 0;
        const uint4 *rp = db + (valid ? row : r0) * w4;
#pragma unroll 4
        for (int c = 0; c < w4; ++c) {
            uint4 x = ldg_nc_u4(rp + c);
#pragma unroll
            for (int j = 0; j < QW; ++j) dist[j] += popc4(x, myq[j * w4 + c]);
        }
#pragma unroll
        for (int j = 0; j < QW; ++j) {
            uint64_t key = valid ? make_key(dist[j], (uint32_t)row) : KEY_EMPTY;
            lists[j].offer(key, thr[j], k);
        }
    }
#pragma unroll
    for (int j = 0; j < QW; ++j) {
        int64_t qi = q0 + warp * QW + j;
        if (qi < nq) lists[j].store(part + ((size_t)qi * n_slices + slice) * k, k);
    }
}

// ── float scan (L2 / L1 / Linf in the reference's arithmetic order) ───────
// db: n rows of dp floats (dp % 4 == 0, zero padded past d).
//
// Lane l of every warp scores row base + l, the whole row in one thread (the
// reference's eight-accumulator order needs it).  The rows reach shared memory
// by TMA (cp.async.bulk.tensor) in boxes of 32 floats (128 bytes) x the
// stage's rows with the 128-byte swizzle, so the 16-byte chunk c of row r sits
// at chunk c ^ (r & 7) of the row's 128 bytes and the eight lanes of each
// quarter-warp phase of a 16-byte shared load (eight consecutive rows, same
// logical chunk) hit eight different bank groups.  Thread 0 keeps FS_STAGES - 1
// stages in flight ahead of the one consumed (one mbarrier per stage, bounded
// waits); the warps (16 queries) share each staged row block.
constexpr int FS_ROWS = 128;  // slices are whole multiples of the short-row stage
constexpr int FS_BOX = 32;    // floats per box row (128 bytes)
constexpr int FS_STAGES = 3;

// Stage shape: rows of at most 64 floats go 128 rows at a time (four 32-row
// blocks, the whole row in one stage); longer rows 32 rows at a time, up to
// 256 floats (8 boxes) per stage and in column chunks beyond that, so that a
// thread's accumulators (its one row) carry across the chunks of its row.
// Rows narrower than 32 floats are one box exactly the row's width, without
// swizzle (16-byte chunk c of row r at r * dp * 4 + 16 c).
struct FsGeom {
    int nbx;     // boxes of 32 floats per row
    int rows;    // rows per stage (128 or 32)
    int cb;      // boxes per stage
    int nchunk;  // column chunks per row
    int bw;      // floats per box row: 32 (swizzled) or the row width (narrow rows)
};
__host__ __device__ inline FsGeom fs_geom(int dp4) {
    FsGeom g;
    g.nbx = (dp4 * 4 + FS_BOX - 1) / FS_BOX;
    g.bw = dp4 * 4 < FS_BOX ? dp4 * 4 : FS_BOX;
    if (g.nbx <= 2) {
        g.rows = 128;
        g.cb = g.nbx;
    } else {
        g.rows = 32;
        g.cb = g.nbx < 8 ? g.nbx : 8;
    }
    g.nchunk = (g.nbx + g.cb - 1) / g.cb;
    return g;
}
inline size_t fs_stage_bytes(int dp4) {
    const FsGeom g = fs_geom(dp4);
    return (size_t)g.cb * g.rows * g.bw * 4;
}
// queries, then 1024-byte aligned stages, then the stage barriers
inline size_t fs_smem_bytes(int warps, int qw, int dp4) {
    return (size_t)warps * qw * dp4 * 16 + 1024 + FS_STAGES * fs_stage_bytes(dp4) + FS_STAGES * 8;
}

// DW: the row width when known at compile time (32, 64 or 128 floats, no
// padding): every shared-memory address and loop bound becomes a constant, so
// the inner loop is the arithmetic and the loads alone; 0 = any width.
template <int METRIC, int QW, int R, int DW = 0>
__global__ void __launch_bounds__(128) float_scan_kernel(const __grid_constant__ CUtensorMap tm, int64_t n,
                                                         int d_arg, int dp, const float *__restrict__ q, int64_t nq,
                                                         int k, int n_slices, int64_t slice_rows, int n_groups,
                                                         uint64_t *__restrict__ part, int *__restrict__ err) {
    const int d = DW ? DW : d_arg;
    extern __shared__ float4 sqf[];  // [WARPS*QW][dp/4] queries, then the stage ring
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int unit = blockIdx.x;
    const int slice = unit / n_groups, group = unit % n_groups;
    const int64_t q0 = (int64_t)group * warps * QW;
    const int dp4 = DW ? DW / 4 : dp >> 2;
    const FsGeom g = fs_geom(dp4);
    const uint32_t box_bytes = (uint32_t)g.rows * g.bw * 4;
    const uint32_t stage_bytes = (uint32_t)g.cb * box_bytes;
    uint8_t *ring = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(sqf + warps * QW * dp4) + 1023) & ~(uintptr_t)1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(ring + FS_STAGES * stage_bytes);
    volatile int *verr = err;

    const float4 *q4 = reinterpret_cast<const float4 *>(q);
    for (int i = threadIdx.x; i < warps * QW * dp4; i += blockDim.x) {
        int64_t qi = q0 + i / dp4;
        sqf[i] = (qi < nq) ? q4[qi * dp4 + (i % dp4)] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < FS_STAGES; ++s) mbar_init(full + s, 1);
        mbar_fence_init();
    }

    const int64_t r0 = (int64_t)slice * slice_rows;
    const int64_t r1 = min(n, r0 + slice_rows);
    const float4 *myq = sqf + warp * QW * dp4;
    const int nb = d >> 3, rem = d & 7;
    const int tail4 = 2 * nb;  // float4 index of the remainder pair (when rem > 0)
    const int64_t nrb = (r1 - r0 + g.rows - 1) / g.rows;
    const int64_t nstage = nrb * g.nchunk;

    // stage si = (row group si / nchunk, column chunk si % nchunk) into ring slot si % FS_STAGES
    auto issue = [&](int64_t si) {
        const int slot = (int)(si % FS_STAGES);
        const int y = (int)(r0 + (si / g.nchunk) * g.rows);
        const int b0 = (int)(si % g.nchunk) * g.cb;
        const int nbox = min(g.cb, g.nbx - b0);
        uint8_t *dst = ring + (size_t)slot * stage_bytes;
        mbar_expect_tx(full + slot, (uint32_t)nbox * box_bytes);
        for (int bi = 0; bi < nbox; ++bi) tma_load_2d(dst + bi * box_bytes, &tm, (b0 + bi) * g.bw, y, full + slot);
    };

    WarpTopK<R> lists[QW];
    uint64_t thr[QW];
#pragma unroll
    for (int j = 0; j < QW; ++j) { lists[j].init(); thr[j] = KEY_EMPTY; }

    __syncthreads();  // queries and barriers ready
    if (threadIdx.x == 0)
        for (int64_t si = 0; si < min((int64_t)FS_STAGES - 1, nstage); ++si) issue(si);
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    FAcc<METRIC> acc[QW];
    float4 x0t = zero4, x1t = zero4;  // the row's remainder pair
    bool ok = true;
    int64_t si = 0;
    for (; si < nstage; ++si) {
        // keep FS_STAGES - 1 stages in flight: slot (si - 1) % FS_STAGES was
        // released by every thread at the end of the previous iteration
        if (threadIdx.x == 0 && si + FS_STAGES - 1 < nstage) issue(si + FS_STAGES - 1);
        const int slot = (int)(si % FS_STAGES);
        if (!mbar_wait(full + slot, (uint32_t)((si / FS_STAGES) & 1), verr)) ok = false;
        if (__syncthreads_or(!ok)) break;  // a wait ran out: every thread leaves together
        const int kc = (int)(si % g.nchunk);
        const int c0 = kc * g.cb * 8;                      // first float4 of this column chunk
        const int c1 = min(dp4, c0 + g.cb * 8);
        const int cb0 = c0 >> 1, cb1 = min(nb, c1 >> 1);  // full blocks of eight in this chunk
        const uint8_t *st = ring + (size_t)slot * stage_bytes;
        for (int rb = 0; rb < g.rows / 32; ++rb) {
            const int rl = rb * 32 + lane;  // row within the stage
            const int sw = rl & 7;
            // float4 c of this lane's row (c in [c0, c1)): box (c - c0) / 8, swizzled chunk
            auto rowf4 = [&](int c) -> float4 {
                const int cc = c - c0;
                if (g.bw < FS_BOX) return *reinterpret_cast<const float4 *>(st + rl * (g.bw * 4) + cc * 16);
                return *reinterpret_cast<const float4 *>(st + (cc >> 3) * box_bytes + rl * 128 +
                                                         (((cc & 7) ^ sw) << 4));
            };
            if (kc == 0) {
#pragma unroll
                for (int j = 0; j < QW; ++j) acc[j].zero();
            }
#pragma unroll 2
            for (int c = cb0; c < cb1; ++c) {
                const float4 x0 = rowf4(2 * c), x1 = rowf4(2 * c + 1);
#pragma unroll
                for (int j = 0; j < QW; ++j) acc[j].block8(myq[j * dp4 + 2 * c], myq[j * dp4 + 2 * c + 1], x0, x1);
            }
            if (rem > 0 && tail4 >= c0 && tail4 < c1) {
                x0t = rowf4(tail4);
                if (rem > 4) x1t = rowf4(tail4 + 1);
            }
            if (kc == g.nchunk - 1) {
                const int64_t row = r0 + (si / g.nchunk) * g.rows + rl;
                const bool valid = row < r1;
#pragma unroll
                for (int j = 0; j < QW; ++j) {
                    float4 qa = zero4, qb = zero4;
                    if (rem > 0) qa = myq[j * dp4 + tail4];
                    if (rem > 4) qb = myq[j * dp4 + tail4 + 1];
                    float dist = acc[j].finish(rem, qa, qb, x0t, x1t);
                    uint64_t key = valid ? make_key(__float_as_uint(dist), (uint32_t)row) : KEY_EMPTY;
                    lists[j].offer(key, thr[j], k);
                }
            }
        }
        __syncthreads();  // slot si % FS_STAGES is free for the next issue
    }
    if (!ok) {
        // a wait ran out in stage si: let the copies issued for stages si ..
        // si + FS_STAGES - 1 land (each wait bounded) before the CTA leaves
        if (threadIdx.x == 0)
            for (int64_t x = si; x < min(nstage, si + FS_STAGES); ++x) {
                const int slot = (int)(x % FS_STAGES);
                const long long t0 = clock64();
                while (!mbar_try_wait(full + slot, (uint32_t)((x / FS_STAGES) & 1)) && clock64() - t0 < 400000) {
                }
            }
        return;
    }
#pragma unroll
    for (int j = 0; j < QW; ++j) {
        int64_t qi = q0 + warp * QW + j;
        if (qi < nq) lists[j].store(part + ((size_t)qi * n_slices + slice) * k, k);
    }
}

// ── merge of per-slice partial lists → final output ───────────────────────
// Offer a query's sorted per-slice lists s_begin, s_begin + s_step, ... (k <=
// 32: one 32-key chunk per slice) to a warp's list: the chunks of MERGE_AHEAD
// slices are loaded together, so that a small batch's hundreds of slices cost
// hundreds / MERGE_AHEAD load latencies instead of one each.
constexpr int MERGE_AHEAD = 16;
template <int R>
__device__ __forceinline__ void merge_slices_ahead(const uint64_t *__restrict__ p, int s_begin, int n_slices,
                                                   int s_step, int k, int lane, WarpTopK<R> &L, uint64_t &thr) {
    for (int s0 = s_begin; s0 < n_slices; s0 += MERGE_AHEAD * s_step) {
        uint64_t kk[MERGE_AHEAD];
#pragma unroll
        for (int u = 0; u < MERGE_AHEAD; ++u) {
            const int s = s0 + u * s_step;
            kk[u] = (s < n_slices && lane < k) ? p[(size_t)s * k + lane] : KEY_EMPTY;
        }
#pragma unroll
        for (int u = 0; u < MERGE_AHEAD; ++u)
            if (!__all_sync(0xffffffffu, kk[u] >= thr)) L.offer(kk[u], thr, k);
    }
}

// Write a query's k nearest: idx (int64, -1 for empty), dist as float32
// (float metrics) or int64 (Hamming).
template <int R>
__device__ __forceinline__ void merge_store(const WarpTopK<R> &L, int64_t qi, int k, int is_hamming, int lane,
                                            int64_t *__restrict__ out_idx, void *__restrict__ out_dist) {
#pragma unroll
    for (int r = 0; r < R; ++r) {
        int pos = r * 32 + lane;
        if (pos < k) {
            uint64_t key = L.v[r];
            bool e = key == KEY_EMPTY;
            out_idx[qi * k + pos] = e ? -1 : (int64_t)key_idx(key);
            if (is_hamming) reinterpret_cast<int64_t *>(out_dist)[qi * k + pos] = e ? 0 : (int64_t)key_dist(key);
            else reinterpret_cast<float *>(out_dist)[qi * k + pos] = e ? 0.f : __uint_as_float(key_dist(key));
        }
    }
}

// One warp per query.
template <int R>
__global__ void flat_merge_kernel(const uint64_t *__restrict__ part, int n_slices, int k, int64_t nq, int is_hamming,
                                  int64_t *__restrict__ out_idx, void *__restrict__ out_dist) {
    const int lane = threadIdx.x & 31;
    const int64_t qi = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (qi >= nq) return;
    WarpTopK<R> L;
    L.init();
    uint64_t thr = KEY_EMPTY;
    const uint64_t *p = part + (size_t)qi * n_slices * k;
    if (k <= 32) merge_slices_ahead(p, 0, n_slices, 1, k, lane, L, thr);
    else for (int s = 0; s < n_slices; ++s) {
        for (int j0 = 0; j0 < k; j0 += 32) {
            int j = j0 + lane;
            uint64_t key = (j < k) ? p[(size_t)s * k + j] : KEY_EMPTY;
            // partial lists are sorted: once the smallest unseen key of this
            // chunk is above the threshold the rest of the list is too
            if (__all_sync(0xffffffffu, key >= thr)) break;
            L.offer(key, thr, k);
        }
    }
    merge_store(L, qi, k, is_hamming, lane, out_idx, out_dist);
}

// Small batches (k <= 32): one block of MERGE_WARPS warps per query, so that
// a batch too small to fill the GPU with one warp per query still merges its
// hundreds of slices quickly: warp w takes slices w, w + MERGE_WARPS, ...,
// then warp 0 offers the other warps' first k keys (disjoint rows) to its own
// list.  The k nearest are the same keys in the same order as flat_merge_kernel's.
constexpr int MERGE_WARPS = 8;
__global__ void __launch_bounds__(MERGE_WARPS * 32)
    flat_merge_split_kernel(const uint64_t *__restrict__ part, int n_slices, int k, int is_hamming,
                            int64_t *__restrict__ out_idx, void *__restrict__ out_dist) {
    __shared__ uint64_t wl[MERGE_WARPS][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t qi = blockIdx.x;
    WarpTopK<1> L;
    L.init();
    uint64_t thr = KEY_EMPTY;
    merge_slices_ahead(part + (size_t)qi * n_slices * k, warp, n_slices, MERGE_WARPS, k, lane, L, thr);
    wl[warp][lane] = lane < k ? L.v[0] : KEY_EMPTY;
    __syncthreads();
    if (warp != 0) return;
#pragma unroll 1
    for (int w = 1; w < MERGE_WARPS; ++w) {
        const uint64_t key = wl[w][lane];
        if (!__all_sync(0xffffffffu, key >= thr)) L.offer(key, thr, k);
    }
    merge_store(L, qi, k, is_hamming, lane, out_idx, out_dist);
}

// ── large-k path: materialised keys + radix select + bitonic sort ────────
template <int METRIC>
__global__ void flat_keys_kernel(const void *__restrict__ db, int64_t n, int d, int stride4,
                                 const void *__restrict__ q, int64_t q_begin, int64_t qc,
                                 uint64_t *__restrict__ keys) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t qq = t / n, row = t % n;
    if (qq >= qc) return;
    const int64_t qi = q_begin + qq;
    uint32_t bits;
    if (METRIC == M_HAMMING) {
        bits = hdist(reinterpret_cast<const uint4 *>(q) + qi * stride4, reinterpret_cast<const uint4 *>(db) + row * stride4,
                     stride4);
    } else {
        bits = __float_as_uint(fdist<METRIC>(reinterpret_cast<const float *>(q) + qi * stride4 * 4,
                                             reinterpret_cast<const float *>(db) + row * stride4 * 4, d));
    }
    keys[qq * n + row] = make_key(bits, (uint32_t)row);
}

// One CTA per query: exact k-th smallest key by MSD radix select (8-bit
// digits), gather the k keys at or below it, bitonic-sort them in place.
__global__ void __launch_bounds__(1024) radix_select_sort_kernel(const uint64_t *__restrict__ keys, int64_t n,
                                                                 int64_t k, int64_t pow2,
                                                                 uint64_t *__restrict__ sorted) {
    __shared__ uint32_t hist[256];
    __shared__ uint64_t s_prefix, s_mask;
    __shared__ int64_t s_krem;
    __shared__ unsigned long long s_count;
    const uint64_t *kq = keys + (int64_t)blockIdx.x * n;
    uint64_t *out = sorted + (int64_t)blockIdx.x * pow2;
    if (threadIdx.x == 0) { s_prefix = 0; s_mask = 0; s_krem = k; }
    __syncthreads();
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        const uint64_t prefix = s_prefix, mask = s_mask;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
            uint64_t v = kq[i];
            if ((v & mask) == prefix) atomicAdd(&hist[(v >> shift) & 0xff], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int64_t krem = s_krem, acc = 0;
            int dgt = 0;
            for (; dgt < 256; ++dgt) {
                if (acc + (int64_t)hist[dgt] >= krem) break;
                acc += hist[dgt];
            }
            s_krem = krem - acc;
            s_prefix = prefix | ((uint64_t)dgt << shift);
            s_mask = mask | (0xffull << shift);
        }
        __syncthreads();
    }
    const uint64_t kth = s_prefix;  // exact k-th smallest key (keys are unique)
    if (threadIdx.x == 0) s_count = 0;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        uint64_t v = kq[i];
        if (v <= kth) out[atomicAdd(&s_count, 1ull)] = v;
    }
    for (int64_t i = k + threadIdx.x; i < pow2; i += blockDim.x) out[i] = KEY_EMPTY;
    __syncthreads();
    for (int64_t size = 2; size <= pow2; size <<= 1) {
        for (int64_t stride = size >> 1; stride > 0; stride >>= 1) {
            for (int64_t i = threadIdx.x; i < pow2 / 2; i += blockDim.x) {
                int64_t lo = (i / stride) * stride * 2 + (i % stride);
                int64_t hi = lo + stride;
                bool up = ((lo & size) == 0);
                uint64_t a = out[lo], b = out[hi];
                if ((a > b) == up) { out[lo] = b; out[hi] = a; }
            }
            __syncthreads();
        }
    }
}

__global__ void keys_to_output_kernel(const uint64_t *__restrict__ sorted, int64_t pow2, int64_t qc, int64_t k,
                                      int64_t q_begin, int is_hamming, int64_t *__restrict__ out_idx,
                                      void *__restrict__ out_dist) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= qc * k) return;
    const int64_t qq = t / k, j = t % k;
    uint64_t key = sorted[qq * pow2 + j];
    bool e = key == KEY_EMPTY;
    const int64_t o = (q_begin + qq) * k + j;
    out_idx[o] = e ? -1 : (int64_t)key_idx(key);
    if (is_hamming) reinterpret_cast<int64_t *>(out_dist)[o] = e ? 0 : (int64_t)key_dist(key);
    else reinterpret_cast<float *>(out_dist)[o] = e ? 0.f : __uint_as_float(key_dist(key));
}

// ── host-side launchers ───────────────────────────────────────────────────
template <int R>
static int launch_scan(const FlatScanArgs &a, int n_groups, int threads, size_t smem, uint64_t *part,
                       cudaStream_t st) {
    const int units = n_groups * a.n_slices;
    if (a.metric == M_HAMMING) {
        timing_begin(st, "hamming_scan_kernel");
        auto kern = hamming_scan_kernel<8, R>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<units, threads, smem, st>>>(reinterpret_cast<const uint4 *>(a.db), a.n, a.stride4,
                                           reinterpret_cast<const uint4 *>(a.q), a.nq, a.k, a.n_slices, a.slice_rows,
                                           n_groups, part);
        timing_end(st);
    } else {
        if (!a.err) return fail(GN_ERR_INVALID, "float scan: no error word");
        // the rows as a TMA tensor: n rows x dp floats, boxes of 32 floats x the stage's rows, 128-byte swizzle
        CUtensorMap tm;
        const FsGeom fg = fs_geom(a.stride4);
        GN_TRY(tmap_encode_2d(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, a.db, (uint64_t)a.stride4 * 4, (uint64_t)a.n,
                              (uint64_t)a.stride4 * 16, (uint32_t)fg.bw, (uint32_t)fg.rows,
                              fg.bw == FS_BOX ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE));
        timing_begin(st, "float_scan_kernel");
        // rows of exactly 32, 64 or 128 floats with k <= 32: the width as a compile-time constant
        const int dw = (R == 1 && a.d == a.stride4 * 4 && (a.d == 32 || a.d == 64 || a.d == 128)) ? a.d : 0;
        auto go = [&](auto MC, auto QC) {
            constexpr int Mv = decltype(MC)::value, Qv = decltype(QC)::value;
            auto launch = [&](auto kern) {
                if (smem > 48 * 1024)
                    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                kern<<<units, threads, smem, st>>>(tm, a.n, a.d, a.stride4 * 4, reinterpret_cast<const float *>(a.q),
                                                   a.nq, a.k, a.n_slices, a.slice_rows, n_groups, part, a.err);
            };
            if (R == 1 && dw == 32) launch(float_scan_kernel<Mv, Qv, 1, 32>);
            else if (R == 1 && dw == 64) launch(float_scan_kernel<Mv, Qv, 1, 64>);
            else if (R == 1 && dw == 128) launch(float_scan_kernel<Mv, Qv, 1, 128>);
            else launch(float_scan_kernel<Mv, Qv, (Qv == 4 ? R : 1)>);
        };
        auto by_qw = [&](auto MC) {
            // fewer queries per warp only for small batches with k <= 32 (R == 1)
            if (a.qw == 1 && R == 1) go(MC, std::integral_constant<int, 1>());
            else if (a.qw == 2 && R == 1) go(MC, std::integral_constant<int, 2>());
            else go(MC, std::integral_constant<int, 4>());
        };
        if (a.metric == M_L2) by_qw(std::integral_constant<int, M_L2>());
        else if (a.metric == M_L1) by_qw(std::integral_constant<int, M_L1>());
        else by_qw(std::integral_constant<int, M_LINF>());
        timing_end(st);
    }
    // a batch of up to two queries per SM over many slices: a block per query
    if (R == 1 && a.nq > 0 && a.nq <= 2 * dev_info().num_sms && a.n_slices >= 2 * MERGE_WARPS) {
        flat_merge_split_kernel<<<(unsigned)a.nq, MERGE_WARPS * 32, 0, st>>>(
            part, a.n_slices, a.k, a.metric == M_HAMMING, a.out_idx, a.out_dist);
        return GN_OK;
    }
    const int qpb = 4;  // queries (warps) per merge block
    flat_merge_kernel<R><<<(unsigned)ceil_div(a.nq, qpb), qpb * 32, 0, st>>>(
        part, a.n_slices, a.k, a.nq, a.metric == M_HAMMING, a.out_idx, a.out_dist);
    return GN_OK;
}

// CTAs of the float scan resident per SM for this metric and list size.
template <int M, int R, int QW = 4>
static int float_scan_occupancy1(int threads, size_t smem) {
    int nb = 0;
    auto kern = float_scan_kernel<M, QW, R>;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem);
    if (e != cudaSuccess) {  // a refused query reads as 0
        cudaGetLastError();
        nb = 0;
    }
    return nb;
}
template <int R>
static int float_scan_occupancy(int metric, int qw, int threads, size_t smem) {
    if (R == 1 && qw == 1)
        return metric == M_L2 ? float_scan_occupancy1<M_L2, 1, 1>(threads, smem)
               : metric == M_L1 ? float_scan_occupancy1<M_L1, 1, 1>(threads, smem)
                                : float_scan_occupancy1<M_LINF, 1, 1>(threads, smem);
    if (R == 1 && qw == 2)
        return metric == M_L2 ? float_scan_occupancy1<M_L2, 1, 2>(threads, smem)
               : metric == M_L1 ? float_scan_occupancy1<M_L1, 1, 2>(threads, smem)
                                : float_scan_occupancy1<M_LINF, 1, 2>(threads, smem);
    if (metric == M_L2) return float_scan_occupancy1<M_L2, R>(threads, smem);
    if (metric == M_L1) return float_scan_occupancy1<M_L1, R>(threads, smem);
    return float_scan_occupancy1<M_LINF, R>(threads, smem);
}

void flat_plan(FlatScanArgs &a) {
    const DevInfo &di = dev_info();
    // float metrics: four queries per warp, fewer for a small batch with
    // k <= 32 so that every warp scores real queries; and no more warps than
    // the batch fills (every warp of a CTA reads each staged row block from
    // shared memory, so a warp of padding queries takes shared-memory
    // bandwidth from the scan: one query over 1M x 128 rows 0.131 -> 0.092 ms).
    // More warps with fewer queries each beat fewer warps with more (4 queries:
    // 4 warps of one 0.133 ms, 1 warp of four 0.167 ms).
    const int qw = (a.metric == M_HAMMING) ? 8 : (a.k <= 32 && a.nq <= 4) ? 1 : (a.k <= 32 && a.nq <= 8) ? 2 : 4;
    const size_t per_warp = (size_t)qw * a.stride4 * 16;
    int warps = a.metric == M_HAMMING ? 4 : (int)std::min<int64_t>(4, std::max<int64_t>(1, ceil_div(a.nq, (int64_t)qw)));
    while (warps > 1 && per_warp * warps > 200 * 1024) warps >>= 1;
    a.warps = warps;
    a.qw = qw;
    const int64_t n_groups = ceil_div(a.nq, (int64_t)warps * qw);
    // slices of at least 128 rows (one float stage): a small database spreads
    // over more SMs instead of running a few CTAs through many stages
    const int64_t max_slices = std::max<int64_t>(1, a.n / 128);
    int64_t slices;
    if (a.metric == M_HAMMING) {
        // aim for ~16 CTAs per SM over the launch
        slices = std::min<int64_t>(std::max<int64_t>(1, ceil_div(16LL * di.num_sms, n_groups)), max_slices);
    } else {
        // units of equal cost: pick the slice count (up to about four waves of
        // resident CTAs) whose last wave is fullest, the fewest slices on a tie
        const int threads = warps * 32;
        const size_t smem = fs_smem_bytes(warps, qw, a.stride4);
        int occ = a.k <= 32 ? float_scan_occupancy<1>(a.metric, qw, threads, smem)
                  : a.k <= 64 ? float_scan_occupancy<2>(a.metric, qw, threads, smem)
                  : a.k <= 128 ? float_scan_occupancy<4>(a.metric, qw, threads, smem)
                               : float_scan_occupancy<8>(a.metric, qw, threads, smem);
        const int64_t slots = (int64_t)std::max(occ, 1) * di.num_sms;
        const int64_t hi = std::min<int64_t>(max_slices, std::max<int64_t>(1, ceil_div(4 * slots, n_groups)));
        slices = 1;
        double best = -1.0;
        for (int64_t s = 1; s <= hi; ++s) {
            const int64_t units = n_groups * s;
            const double eff = (double)units / (double)(ceil_div(units, slots) * slots);
            if (eff > best + 1e-9) {
                best = eff;
                slices = s;
            }
        }
    }
    // float scans stage up to 128 rows at a time: whole stages per slice
    a.slice_rows = round_up(ceil_div(a.n, slices), a.metric == M_HAMMING ? 32 : FS_ROWS);
    a.n_slices = (int)ceil_div(a.n, a.slice_rows);
    a.n_groups = (int)n_groups;
}

size_t flat_part_bytes(const FlatScanArgs &a) { return (size_t)a.nq * a.n_slices * a.k * sizeof(uint64_t); }

static size_t flat_smem_bytes(const FlatScanArgs &a) {
    return a.metric == M_HAMMING ? (size_t)a.warps * a.qw * a.stride4 * 16 : fs_smem_bytes(a.warps, a.qw, a.stride4);
}

int flat_smem_ok(const FlatScanArgs &a) {
    return flat_smem_bytes(a) <= (size_t)dev_info().max_smem_optin;
}

// Launch the warp-select path (k <= 256).  part: flat_part_bytes(a) scratch.
int flat_launch(const FlatScanArgs &a, uint64_t *part, cudaStream_t st) {
    const int threads = a.warps * 32;
    const size_t smem = flat_smem_bytes(a);
    if (a.k <= 32) return launch_scan<1>(a, a.n_groups, threads, smem, part, st);
    if (a.k <= 64) return launch_scan<2>(a, a.n_groups, threads, smem, part, st);
    if (a.k <= 128) return launch_scan<4>(a, a.n_groups, threads, smem, part, st);
    return launch_scan<8>(a, a.n_groups, threads, smem, part, st);
}

int64_t next_pow2(int64_t v) {
    int64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

// Large-k path for one chunk of queries [q_begin, q_begin + qc).
// keys: qc*n scratch; sorted: qc*next_pow2(k) scratch.
void flat_large_k_launch(const FlatScanArgs &a, int64_t q_begin, int64_t qc, uint64_t *keys, uint64_t *sorted,
                         cudaStream_t st) {
    const int64_t total = qc * a.n;
    const unsigned blocks = (unsigned)ceil_div(total, 256);
    switch (a.metric) {
    case M_HAMMING: flat_keys_kernel<M_HAMMING><<<blocks, 256, 0, st>>>(a.db, a.n, a.d, a.stride4, a.q, q_begin, qc, keys); break;
    case M_L2: flat_keys_kernel<M_L2><<<blocks, 256, 0, st>>>(a.db, a.n, a.d, a.stride4, a.q, q_begin, qc, keys); break;
    case M_L1: flat_keys_kernel<M_L1><<<blocks, 256, 0, st>>>(a.db, a.n, a.d, a.stride4, a.q, q_begin, qc, keys); break;
    default: flat_keys_kernel<M_LINF><<<blocks, 256, 0, st>>>(a.db, a.n, a.d, a.stride4, a.q, q_begin, qc, keys); break;
    }
    const int64_t kk = std::min<int64_t>(a.k, a.n);
    const int64_t p2 = next_pow2(a.k);
    radix_select_sort_kernel<<<(unsigned)qc, 1024, 0, st>>>(keys, a.n, kk, p2, sorted);
    keys_to_output_kernel<<<(unsigned)ceil_div(qc * a.k, 256), 256, 0, st>>>(sorted, p2, qc, a.k, q_begin,
                                                                              a.metric == M_HAMMING, a.out_idx,
                                                                              a.out_dist);
}

}  // namespace gn

namespace gn {

// Loads every kernel the Hamming warp-select path can launch (the scan and
// the merge, for each list width).  With lazy module loading (the default
// since CUDA 12.2) a kernel's module is loaded, and its device memory
// allocated, at its first launch; querying the kernel's attributes loads it
// ahead of that.  Cheap once loaded.
int flat_preload_hamming() {
    cudaFuncAttributes fa;
    const void *fns[] = {(const void *)hamming_scan_kernel<8, 1>, (const void *)hamming_scan_kernel<8, 2>,
                         (const void *)hamming_scan_kernel<8, 4>, (const void *)hamming_scan_kernel<8, 8>,
                         (const void *)flat_merge_kernel<1>,      (const void *)flat_merge_kernel<2>,
                         (const void *)flat_merge_kernel<4>,      (const void *)flat_merge_kernel<8>,
                         (const void *)flat_merge_split_kernel};
    for (const void *f : fns) GN_CUDA_TRY(cudaFuncGetAttributes(&fa, f));
    return GN_OK;
}

}  // namespace gn
