// tc_scan.cu — tensor-core L2 candidate stage: BF16 GEMM on tcgen05 with a
// fused per-query top-S epilogue, and the exact FP32 re-rank that follows it.
//
// One persistent CTA per SM walks a list of work units.  A unit is a tile of up
// to 128 "A" rows (queries) against a range [r0, r1) of "B" rows (database
// rows), both K-major, in one of two precisions:
//   BF16       K padded to a multiple of 64 elements;
//   FP8 E4M3   with one FP32 scale per row (row = scale x E4M3 values, the
//              row's largest magnitude mapped to 448), K padded to 128;
// either way a pipeline stage holds 128 bytes of K per row.
//   warp 0     TMA producer: 128-byte K slices of A (128 rows) and B (256 rows)
//              into a 2- or 3-stage shared-memory ring (128-byte swizzle);
//   warp 1     allocates 512 TMEM columns, one thread issues tcgen05.mma
//              (M=128, N=256, K=16 BF16 or K=32 FP8) into one of two
//              256-column accumulators;
//   warps 2-9  epilogue: tcgen05.ld of the accumulator rows of their TMEM lane
//              quadrant, half of the columns each; score = |x|^2 - 2 q.x
//              (exact FP32 |x|^2; FP8: q.x = scale_q scale_x acc); each thread
//              owns one query row and keeps the S best (score, row) keys of its
//              columns in a shared-memory max-heap.  A block of 32 scores is
//              first reduced to its minimum, which is compared with the
//              threshold (the heap's root, and the other half's root): most
//              blocks end there, the rest are filtered score by score.
// At the end of a unit each query's S keys go to its partial slot.  A full
// list's S-th best score is published as the query's bound (atomicMin) every
// tile, and every tile reads it back, so the units of a query that run at the
// same time (its other database chunks) and later ones filter below it; the re-rank kernel
// merges a query's slots, keeps the S best by BF16 score, recomputes their
// distances exactly in FP32 and returns the k nearest.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "distance.cuh"
#include "gemm_topk.cuh"
#include "index.cuh"
#include "kmeans.cuh"
#include "tc_scan.cuh"
#include "tc_sm100.cuh"
#include "tmap.cuh"
#include "timing.cuh"
#include "topk.cuh"

namespace gn {

constexpr int TC_M = 128, TC_N = 256, TC_BK = 64;  // TC_BK: BF16 elements per 128-byte K slice
constexpr int TC_BK8 = 128;                          // FP8 elements per 128-byte K slice
constexpr int TC_A_BYTES = TC_M * TC_BK * 2;   // 16 KB
constexpr int TC_B_BYTES = TC_N * TC_BK * 2;   // 32 KB
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
// Epilogue warps: 8, two per TMEM lane quadrant, each covering half of the
// accumulator's columns (top-S mode: each thread keeps a query row's list for
// its half; the halves merge at the end of a unit).
__host__ __device__ constexpr int tc_nepi(int S) { return 8; }
__host__ __device__ constexpr int tc_threads(int S) { return 64 + 32 * tc_nepi(S); }
// pipeline depth: three stages, two where the lists need the room (S above
// 40; S = 40 with FP8's column scales)
__host__ __device__ constexpr int tc_stages(int S, bool f8 = false) { return S > 40 || (S > 32 && f8) ? 2 : 3; }

__host__ __device__ constexpr size_t tc_smem_bytes(int S, bool f8 = false) {
    // S == 0 is the store mode: a 32x33 transpose tile per epilogue warp;
    // top-S mode: two lists (one per column half) of S keys per query row;
    // per epilogue warp 32 column norms (and, FP8, 32 column scales)
    return 1024 /*alignment slack*/ + (size_t)tc_stages(S, f8) * TC_STAGE_BYTES +
           (S ? (size_t)2 * TC_M * S * 8 : (size_t)tc_nepi(S) * 32 * 33 * 4) +
           (size_t)tc_nepi(S) * 32 * 4 * (f8 ? 2 : 1) + 256;
}

// Max-heap of S keys in a thread's strided shared-memory list (element i at
// L[i * TC_M]): replace the root (the largest) by a smaller key and sift down.
__device__ __noinline__ void tc_heap_replace_top(uint64_t *L, int S, uint64_t key) {
    int i = 0;
    while (true) {
        const int c = 2 * i + 1;
        if (c >= S) break;
        uint64_t cv = L[c * TC_M];
        int cm = c;
        if (c + 1 < S) {
            const uint64_t c2 = L[(c + 1) * TC_M];
            if (c2 > cv) {
                cv = c2;
                cm = c + 1;
            }
        }
        if (cv <= key) break;
        L[i * TC_M] = cv;
        i = cm;
    }
    L[i * TC_M] = key;
}

template <int S, bool F8>
__global__ void __launch_bounds__(tc_threads(S), 1)
    tc_topk_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const TcUnit *__restrict__ units, const int64_t *__restrict__ n_units_ptr,
                   const int64_t *__restrict__ cta_off, int K, int kblk,
                   const float *__restrict__ bnorm, const float *__restrict__ ascale,
                   const float *__restrict__ bscale, const int64_t *__restrict__ arow_slot,
                   uint64_t *__restrict__ part, float *__restrict__ scores, uint32_t *__restrict__ qbound,
                   int *__restrict__ err) {
    constexpr bool STORE = (S == 0);
    static_assert(!(STORE && F8), "the store mode is BF16 only");
    constexpr int SL = STORE ? 1 : 2 * S;  // list keys per query row (two column halves)
    constexpr int NEPI = tc_nepi(S);
    constexpr int TC_STAGES = tc_stages(S, F8);
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint8_t *stage_base = smem;
    uint64_t *lists = reinterpret_cast<uint64_t *>(smem + TC_STAGES * TC_STAGE_BYTES);  // [2][S][TC_M]
    float *xpose = reinterpret_cast<float *>(smem + TC_STAGES * TC_STAGE_BYTES);  // store mode: [NEPI][32][33]
    float *snorm = STORE ? xpose + NEPI * 32 * 33 : reinterpret_cast<float *>(lists + TC_M * SL);
    float *sscale = snorm + NEPI * 32;  // FP8: per-warp column scales
    uint64_t *bars = reinterpret_cast<uint64_t *>(snorm + NEPI * 32 * (F8 ? 2 : 1));
    uint64_t *full = bars, *empty = bars + TC_STAGES, *accfull = bars + 2 * TC_STAGES,
             *accempty = bars + 2 * TC_STAGES + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * TC_STAGES + 4);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int *verr = err;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(accfull + b, 1);
            mbar_init(accempty + b, NEPI);
        }
        mbar_fence_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // this CTA's units: [u_begin, u_end) with stride u_step
    const int64_t n_units = *n_units_ptr;
    int64_t u_begin = blockIdx.x, u_end = n_units, u_step = gridDim.x;
    if (cta_off) {
        u_begin = cta_off[blockIdx.x];
        u_end = cta_off[blockIdx.x + 1];
        u_step = 1;
    }
    const int nk = K / kblk;

    if (warp == 0) {
        // ── TMA producer ──
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int64_t u = u_begin; u < u_end && ok; u += u_step) {
                const TcUnit un = units[u];
                const int ntile = (int)((un.r1 - un.r0 + TC_N - 1) / TC_N);
                for (int t = 0; t < ntile && ok; ++t)
                    for (int kb = 0; kb < nk && ok; ++kb, ++it) {
                        const int s = it % TC_STAGES;
                        const uint32_t ph = (it / TC_STAGES) & 1;
                        if (!mbar_wait(empty + s, ph ^ 1, verr)) { ok = false; break; }
                        uint8_t *sa = stage_base + s * TC_STAGE_BYTES;
                        mbar_expect_tx(full + s, TC_STAGE_BYTES);
                        tma_load_2d(sa, &tmA, kb * kblk, (int)un.a0, full + s);
                        tma_load_2d(sa + TC_A_BYTES, &tmB, kb * kblk, (int)(un.r0 + (int64_t)t * TC_N), full + s);
                    }
            }
        }
    } else if (warp == 1) {
        // ── MMA issuer ──
        if (lane == 0) {
            const uint32_t idesc = F8 ? idesc_e4m3_f32(TC_M, TC_N) : idesc_bf16_f32(TC_M, TC_N);
            uint32_t it = 0, tile_it = 0;
            bool ok = true;
            for (int64_t u = u_begin; u < u_end && ok; u += u_step) {
                const TcUnit un = units[u];
                const int ntile = (int)((un.r1 - un.r0 + TC_N - 1) / TC_N);
                for (int t = 0; t < ntile && ok; ++t, ++tile_it) {
                    const int b = tile_it & 1;
                    const uint32_t tph = (tile_it >> 1) & 1;
                    if (!mbar_wait(accempty + b, tph ^ 1, verr)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t dt = tmem + (uint32_t)(b * TC_N);
                    for (int kb = 0; kb < nk; ++kb, ++it) {
                        const int s = it % TC_STAGES;
                        const uint32_t ph = (it / TC_STAGES) & 1;
                        if (!mbar_wait(full + s, ph, verr)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t sa = smem_u32(stage_base + s * TC_STAGE_BYTES);
                        const uint64_t da = sdesc_sw128(sa), db = sdesc_sw128(sa + TC_A_BYTES);
                        // four MMAs of 32 bytes of K each (16 BF16 or 32 FP8 elements):
                        // the descriptors advance by 32 bytes (2 in 16-byte units)
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            if constexpr (F8) umma_f8(dt, da + 2 * kk, db + 2 * kk, idesc, (kb | kk) ? 1u : 0u);
                            else umma_bf16(dt, da + 2 * kk, db + 2 * kk, idesc, (kb | kk) ? 1u : 0u);
                        }
                        umma_commit(empty + s);
                    }
                    if (ok) umma_commit(accfull + b);
                }
            }
        }
    } else if constexpr (STORE) {
        // ── epilogue (store mode): scores of a 32x32 block go through a padded
        // shared tile so that each store instruction writes 32 consecutive
        // floats of one query's segment ──
        const int quad = warp & 3;
        const int grp = (warp - 2) >> 2;  // which half of the 256 columns
        constexpr int CPG = (TC_N / 32) / (NEPI / 4);
        float *xp = xpose + (warp - 2) * 32 * 33;
        float *sn = snorm + (warp - 2) * 32;
        uint32_t tile_it = 0;
        bool ok = true;
        for (int64_t u = u_begin; u < u_end && ok; u += u_step) {
            const TcUnit un = units[u];
            const int ntile = (int)((un.r1 - un.r0 + TC_N - 1) / TC_N);
            // segment base of each of this warp's 32 query rows (lane r holds row r's)
            const int qrow = quad * 32 + lane;
            const int64_t myseg = (qrow < un.na) ? arow_slot[un.a0 + qrow] - un.rbase : INT64_MIN;
            for (int t = 0; t < ntile; ++t, ++tile_it) {
                const int b = tile_it & 1;
                const uint32_t tph = (tile_it >> 1) & 1;
                const int64_t n0 = un.r0 + (int64_t)t * TC_N;
                float nrm[CPG];
#pragma unroll
                for (int cc = 0; cc < CPG; ++cc) {
                    const int64_t col = n0 + (grp * CPG + cc) * 32 + lane;
                    nrm[cc] = col < un.r1 ? __ldg(bnorm + col) : 0.f;
                }
                if (!mbar_wait(accfull + b, tph, verr)) { ok = false; break; }
                tc_fence_after();
#pragma unroll 1
                for (int cc = 0; cc < CPG; ++cc) {
                    const int c = grp * CPG + cc;
                    const int64_t col0 = n0 + c * 32;
                    __syncwarp();
                    sn[lane] = nrm[cc];
                    __syncwarp();
                    float acc[32];
                    tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * TC_N + c * 32), acc);
#pragma unroll
                    for (int j = 0; j < 32; ++j) xp[lane * 33 + j] = fmaf(-2.f, acc[j], sn[j]);
                    __syncwarp();
                    const bool colok = col0 + lane < un.r1;
#pragma unroll 4
                    for (int r = 0; r < 32; ++r) {
                        const int64_t seg = __shfl_sync(0xffffffffu, myseg, r);
                        if (seg != INT64_MIN && colok) scores[seg + col0 + lane] = xp[r * 33 + lane];
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(accempty + b);
            }
        }
    } else {
        // ── epilogue: warps 2..9, TMEM lane quadrant = warp % 4, column half =
        // (warp - 2) / 4; each thread keeps the S best keys of one query row
        // over its half of the columns at lists[(half * S + i) * TC_M + row]
        // (bank-conflict free) as a max-heap: a new key replaces the root (the
        // S-th best) and sifts down.  At the end of a unit the two halves of a
        // row are merged.
        const int quad = warp & 3, half = (warp - 2) >> 2;
        const int row = quad * 32 + lane;
        __shared__ volatile int pair_ok[8];
        uint64_t *L = lists + (size_t)half * S * TC_M + row;
        // the other half's heap root (its current S-th best key of this row):
        // only ever holds final root values, so it can be read at any time
        const volatile uint64_t *other_root = lists + (size_t)(half ^ 1) * S * TC_M + row;
        float *sn = snorm + (warp - 2) * 32;
        float *sc = sscale + (warp - 2) * 32;
        uint32_t tile_it = 0;
        bool ok = true;
        for (int64_t u = u_begin; u < u_end && ok; u += u_step) {
            const TcUnit un = units[u];
            const int ntile = (int)((un.r1 - un.r0 + TC_N - 1) / TC_N);
#pragma unroll 4
            for (int i = 0; i < S; ++i) L[i * TC_M] = KEY_EMPTY;
            uint64_t thr = KEY_EMPTY;  // the heap's root: the S-th best key so far
            // the query's bound from units already finished: the S-th best score of
            // some unit's S rows, so no key above it can reach the query's S best;
            // it caps the filter threshold for the whole unit (the list's own root
            // only takes over once it is lower)
            float gbound = __int_as_float(0x7f800000);  // +inf
            if (qbound && row < un.na) {
                const uint32_t g = *reinterpret_cast<volatile uint32_t *>(qbound + un.a0 + row);
                if (g != 0xffffffffu) gbound = ord2f(g);
            }
            float thr_f = gbound;
            // score = |x|^2 + qc * (column factor) * acc: qc = -2 (BF16) or
            // -2 scale_q (FP8, column factor scale_x)
            const float qc = F8 ? (row < un.na ? -2.f * __ldg(ascale + un.a0 + row) : 0.f) : -2.f;
            asm volatile("bar.sync %0, 64;" ::"r"(1 + quad) : "memory");  // both halves reset before either reads
            for (int t = 0; t < ntile; ++t, ++tile_it) {
                const int b = tile_it & 1;
                const uint32_t tph = (tile_it >> 1) & 1;
                const int64_t n0 = un.r0 + (int64_t)t * TC_N;
                // the query's bound as the units running beside this one (its other
                // database chunks) have lowered it so far, read before the wait
                uint32_t gnow = 0xffffffffu;
                if (qbound && row < un.na) gnow = *reinterpret_cast<volatile uint32_t *>(qbound + un.a0 + row);
                // row norms of this warp's 128 columns, fetched before the wait
                float nrm[TC_N / 64], csc[TC_N / 64];
#pragma unroll
                for (int c = 0; c < TC_N / 64; ++c) {
                    const int64_t col = n0 + (half * (TC_N / 64) + c) * 32 + lane;
                    nrm[c] = col < un.r1 ? __ldg(bnorm + col) : 0.f;
                    if constexpr (F8) csc[c] = col < un.r1 ? __ldg(bscale + col) : 0.f;
                }
                if (!mbar_wait(accfull + b, tph, verr)) { ok = false; break; }
                tc_fence_after();
                if (gnow != 0xffffffffu) {
                    gbound = fminf(gbound, ord2f(gnow));
                    thr_f = fminf(thr_f, gbound);
                }
                // the other half's S-th best also bounds this row: a key not below
                // it has S better keys in the other half
                {
                    const uint64_t o = *other_root;
                    if (o != KEY_EMPTY) thr_f = fminf(thr_f, ord2f(key_dist(o)));
                }
                // publish this half's S-th best (once its list is full) for the
                // query's other units
                if (qbound && thr != KEY_EMPTY && row < un.na && key_dist(thr) < gnow)
                    atomicMin(qbound + un.a0 + row, key_dist(thr));
#pragma unroll 1
                for (int cc = 0; cc < TC_N / 64; ++cc) {
                    const int c = half * (TC_N / 64) + cc;
                    const int64_t col0 = n0 + c * 32;
                    // columns past the unit's last row (the tail of its last tile,
                    // TMA zero fill) are never offered; col0 is warp-uniform
                    if (col0 >= un.r1) break;
                    __syncwarp();
                    sn[lane] = nrm[cc];
                    if constexpr (F8) sc[lane] = csc[cc];
                    __syncwarp();
                    float acc[32];
                    tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * TC_N + c * 32), acc);
                    // scores and their minimum (four independent chains)
                    const float4 *sn4 = reinterpret_cast<const float4 *>(sn);
                    const float4 *sc4 = reinterpret_cast<const float4 *>(sc);
                    const float inf = __int_as_float(0x7f800000);
                    float mn4[4] = {inf, inf, inf, inf};
#pragma unroll
                    for (int j4 = 0; j4 < 8; ++j4) {
                        const float4 nv = sn4[j4];
                        float4 cf = make_float4(qc, qc, qc, qc);
                        if constexpr (F8) {
                            const float4 sv = sc4[j4];
                            cf = make_float4(qc * sv.x, qc * sv.y, qc * sv.z, qc * sv.w);
                        }
                        acc[4 * j4 + 0] = fmaf(cf.x, acc[4 * j4 + 0], nv.x);
                        acc[4 * j4 + 1] = fmaf(cf.y, acc[4 * j4 + 1], nv.y);
                        acc[4 * j4 + 2] = fmaf(cf.z, acc[4 * j4 + 2], nv.z);
                        acc[4 * j4 + 3] = fmaf(cf.w, acc[4 * j4 + 3], nv.w);
                        mn4[0] = fminf(mn4[0], acc[4 * j4 + 0]);
                        mn4[1] = fminf(mn4[1], acc[4 * j4 + 1]);
                        mn4[2] = fminf(mn4[2], acc[4 * j4 + 2]);
                        mn4[3] = fminf(mn4[3], acc[4 * j4 + 3]);
                    }
                    if (!(fminf(fminf(mn4[0], mn4[1]), fminf(mn4[2], mn4[3])) <= thr_f)) continue;
                    const int nvalid = (int)min((int64_t)32, un.r1 - col0);  // 1..32
                    // filter: a pass mask from independent compares (four partial
                    // masks, no serial chain); the rare passing scores are offered
                    uint32_t pm4[4] = {0u, 0u, 0u, 0u};
#pragma unroll
                    for (int j = 0; j < 32; ++j) pm4[j & 3] |= (acc[j] <= thr_f ? 1u : 0u) << j;
                    uint32_t pm = (pm4[0] | pm4[1]) | (pm4[2] | pm4[3]);
                    if (nvalid < 32) pm &= (1u << nvalid) - 1u;
                    while (pm) {
                        const int j = __ffs(pm) - 1;
                        pm &= pm - 1;
                        float v = acc[0];
#pragma unroll
                        for (int jj = 1; jj < 32; ++jj) v = jj == j ? acc[jj] : v;
                        const uint64_t key = make_key(f2ord(v), (uint32_t)(col0 + j));
                        if (key < thr) {
                            tc_heap_replace_top(L, S, key);
                            thr = L[0];
                            thr_f = (thr == KEY_EMPTY) ? gbound : fminf(gbound, ord2f(key_dist(thr)));
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(accempty + b);
            }
            // merge the two halves of each row (the two warps of a quadrant meet
            // at a named barrier and agree on whether to go on), then the
            // first half sorts and writes
            if (lane == 0) pair_ok[quad * 2 + half] = ok ? 1 : 0;
            asm volatile("bar.sync %0, 64;" ::"r"(1 + quad) : "memory");
            ok = pair_ok[quad * 2] && pair_ok[quad * 2 + 1];
            if (half == 0 && ok) {
                const uint64_t *L2 = L + (size_t)S * TC_M;
                for (int i = 0; i < S; ++i) {
                    const uint64_t key = L2[i * TC_M];
                    if (key < thr) {
                        tc_heap_replace_top(L, S, key);
                        thr = L[0];
                    }
                }
                if (row < un.na) {
                    for (int i = 1; i < S; ++i) {  // ascending, for the re-rank's merge
                        const uint64_t key = L[i * TC_M];
                        int p = i;
                        while (p > 0 && L[(p - 1) * TC_M] > key) {
                            L[p * TC_M] = L[(p - 1) * TC_M];
                            --p;
                        }
                        L[p * TC_M] = key;
                    }
                    uint64_t *dst = part + (arow_slot[un.a0 + row] + un.rch) * S;
#pragma unroll 4
                    for (int i = 0; i < S; ++i) dst[i] = L[i * TC_M];
                    // a full list bounds the query's S-th best score for later units
                    if (qbound && thr != KEY_EMPTY) atomicMin(qbound + un.a0 + row, key_dist(thr));
                }
            }
            asm volatile("bar.sync %0, 64;" ::"r"(1 + quad) : "memory");
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, 512);
}

// ── host: tensor maps and launch ──────────────────────────────────────────
// K-major operand rows of K elements (BF16, or FP8 stored as bytes), boxes of
// 128 bytes of K by box_rows rows, 128-byte swizzle.
static int make_tmap_rows(CUtensorMap *map, const void *base, int64_t rows, int64_t K, int box_rows, bool f8) {
    return tmap_encode_2d(map, f8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, base,
                          (uint64_t)K, (uint64_t)rows, (uint64_t)K * (f8 ? 1 : 2), f8 ? TC_BK8 : TC_BK,
                          (uint32_t)box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

int tc_topk_launch(const TcLaunch &a, cudaStream_t st) {
    const int kblk = a.fp8 ? TC_BK8 : TC_BK;
    if (a.K % kblk)
        return fail(GN_ERR_INVALID, a.fp8 ? "tensor-core scan: FP8 K must be a multiple of 128"
                                          : "tensor-core scan: K must be a multiple of 64");
    if (a.fp8 && (a.S == 0 || a.S > 56 || !a.ascale || !a.bscale))
        return fail(GN_ERR_UNSUPPORTED, "FP8 shortlist: S must be 16, 32, 40, 48 or 56, with row scales");
    CUtensorMap ma, mb;
    GN_TRY(make_tmap_rows(&ma, a.A, std::max<int64_t>(a.a_rows, 1), a.K, TC_M, a.fp8));
    GN_TRY(make_tmap_rows(&mb, a.B, std::max<int64_t>(a.b_rows, 1), a.K, TC_N, a.fp8));
    auto launch = [&](auto SC, auto FC) -> int {
        constexpr int Sv = decltype(SC)::value;
        constexpr bool Fv = decltype(FC)::value;
        // 227 KB of shared memory per block, less the kernel's static 32 bytes
        static_assert(tc_smem_bytes(Sv, Fv) + 32 <= 227 * 1024, "shortlist stages and lists exceed shared memory");
        const size_t smem = tc_smem_bytes(Sv, Fv);
        GN_CUDA_TRY(cudaFuncSetAttribute(tc_topk_kernel<Sv, Fv>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
        tc_topk_kernel<Sv, Fv><<<a.grid, tc_threads(Sv), smem, st>>>(ma, mb, a.units, a.n_units, a.cta_off, a.K,
                                                                     kblk, a.bnorm, a.ascale, a.bscale, a.arow_slot,
                                                                     a.part, a.scores, a.qbound, a.err);
        return GN_OK;
    };
    using F0 = std::false_type;
    using F1 = std::true_type;
    if (a.fp8) switch (a.S) {
        case 16: return launch(std::integral_constant<int, 16>(), F1());
        case 32: return launch(std::integral_constant<int, 32>(), F1());
        case 40: return launch(std::integral_constant<int, 40>(), F1());
        case 48: return launch(std::integral_constant<int, 48>(), F1());
        case 56: return launch(std::integral_constant<int, 56>(), F1());
        default: break;
        }
    switch (a.S) {
    case 0: return launch(std::integral_constant<int, 0>(), F0());
    case 16: return launch(std::integral_constant<int, 16>(), F0());
    case 32: return launch(std::integral_constant<int, 32>(), F0());
    case 40: return launch(std::integral_constant<int, 40>(), F0());
    case 48: return launch(std::integral_constant<int, 48>(), F0());
    case 56: return launch(std::integral_constant<int, 56>(), F0());
    case 64: return launch(std::integral_constant<int, 64>(), F0());
    default: return fail(GN_ERR_UNSUPPORTED, "shortlist size must be 16, 32, 40, 48, 56 or 64");
    }
}

// ── conversion and norms ──────────────────────────────────────────────────
__global__ void f32_to_bf16_rows_kernel(const float *__restrict__ X, int64_t n, int d, int ldx,
                                        __nv_bfloat16 *__restrict__ out, int K) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * K) return;
    const int64_t i = t / K;
    const int j = (int)(t % K);
    out[t] = __float2bfloat16_rn(j < d ? X[i * ldx + j] : 0.f);
}

void to_bf16_rows(const float *X, int64_t n, int d, int ldx, void *out, int K, cudaStream_t st) {
    if (n > 0)
        f32_to_bf16_rows_kernel<<<(unsigned)ceil_div(n * K, 256), 256, 0, st>>>(
            X, n, d, ldx, reinterpret_cast<__nv_bfloat16 *>(out), K);
}

// FP8 E4M3 rows with one FP32 scale each: warp per row; scale = max|x| / 448
// (the largest E4M3 magnitude; 1 for an all-zero row), element = x / scale
// rounded to nearest E4M3 with saturation, zero beyond d up to K.
__global__ void f32_to_e4m3_rows_kernel(const float *__restrict__ X, int64_t n, int d, int ldx,
                                        uint8_t *__restrict__ out, float *__restrict__ scale, int K) {
    const int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= n) return;
    const float *x = X + r * ldx;
    float m = 0.f;
    for (int j = lane; j < d; j += 32) m = fmaxf(m, fabsf(x[j]));
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    const float sc = m > 0.f ? m / 448.f : 1.f;
    const float inv = m > 0.f ? 448.f / m : 1.f;
    if (lane == 0) scale[r] = sc;
    uint8_t *o = out + r * K;
    for (int j = lane; j < K; j += 32)
        o[j] = j < d ? (uint8_t)__nv_cvt_float_to_fp8(x[j] * inv, __NV_SATFINITE, __NV_E4M3) : (uint8_t)0;
}

void to_e4m3_rows(const float *X, int64_t n, int d, int ldx, void *out, float *scale, int K, cudaStream_t st) {
    if (n > 0)
        f32_to_e4m3_rows_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, st>>>(X, n, d, ldx,
                                                                          reinterpret_cast<uint8_t *>(out), scale, K);
}

// ── exact re-rank ─────────────────────────────────────────────────────────
// One warp per query: merge its nslot partial lists (S keys each, by BF16
// score), keep the S best, recompute their L2 distance in the reference's FP32
// order (bit-identical to the exact flat scan), return the k nearest.
template <int RS>
__global__ void tc_rerank_kernel(const uint64_t *__restrict__ part, int nslot, int S, const float *__restrict__ Q,
                                 const float *__restrict__ X, int d, int dp, const int32_t *__restrict__ ids,
                                 int64_t nq, int k, int sqrt_out, int64_t *__restrict__ out_idx,
                                 float *__restrict__ out_dist) {
    const int lane = threadIdx.x & 31;
    const int64_t q = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= nq) return;
    WarpTopK<RS> L;
    L.init();
    uint64_t thr = KEY_EMPTY;
    const uint64_t *p = part + q * (int64_t)nslot * S;
    for (int sl = 0; sl < nslot; ++sl)
        for (int j0 = 0; j0 < S; j0 += 32) {
            const int j = j0 + lane;
            const uint64_t key = (j < S) ? p[(int64_t)sl * S + j] : KEY_EMPTY;
            if (__all_sync(0xffffffffu, key >= thr)) break;
            L.offer(key, thr, S);
        }
    // exact distances of the shortlist, then top-k by (distance, id)
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
            float dd = fdist<M_L2>(Q + q * dp, X + row * dp, d);
            if (!sqrt_out) dd = __fmul_rn(dd, dd);
            const uint32_t oid = ids ? (uint32_t)ids[row] : (uint32_t)row;
            fk = make_key(__float_as_uint(dd), oid);
        }
        F.offer(fk, fthr, k);
    }
    if (lane < k) {
        const uint64_t key = F.v[0];
        const bool e = key == KEY_EMPTY;
        out_idx[q * k + lane] = e ? -1 : (int64_t)key_idx(key);
        out_dist[q * k + lane] = e ? 0.f : __uint_as_float(key_dist(key));
    }
}

int tc_rerank_launch(const uint64_t *part, int nslot, int S, const float *Q, const float *X, int d, int dp,
                     const int32_t *ids, int64_t nq, int k, int sqrt_out, int64_t *out_idx, float *out_dist,
                     cudaStream_t st) {
    if (k > 32) return fail(GN_ERR_UNSUPPORTED, "tensor-core path supports k <= 32");
    const unsigned blocks = (unsigned)ceil_div(nq, 4);
    if (S <= 32) tc_rerank_kernel<1><<<blocks, 128, 0, st>>>(part, nslot, S, Q, X, d, dp, ids, nq, k, sqrt_out, out_idx, out_dist);
    else tc_rerank_kernel<2><<<blocks, 128, 0, st>>>(part, nslot, S, Q, X, d, dp, ids, nq, k, sqrt_out, out_idx, out_dist);
    return GN_OK;
}

// ── flat tensor-core index (exact L2 via shortlist + re-rank) ─────────────
struct TcFlatState {
    int d = 0, dp = 0, K = 0;
    int S = 40;
    int fp8 = 0;  // 0: BF16 operands; 1: FP8 E4M3 with per-row scales
    int64_t n = 0;
    DBuf x32, x16, xnorm, xscale;  // fp32 rows (dp), low-precision rows (K), |x|^2, FP8 row scales
    DBuf q32, q16, qscale, units, nunits, aslot, part, qbound, err, out_idx, out_dist;
    int64_t planned_nq = -1;
    int nchunks = 1, grid = 0;
};

// The database's low-precision copy in the index's precision, from its FP32
// rows; it holds at least one full 256-row TMA box.
static int tcflat_lowp(TcFlatState &S, cudaStream_t st) {
    S.K = (int)round_up(S.d, S.fp8 ? TC_BK8 : TC_BK);
    const size_t bytes = (size_t)std::max<int64_t>(S.n, TC_N) * S.K * (S.fp8 ? 1 : 2);
    GN_TRY(S.x16.ensure(bytes));
    GN_CUDA_TRY(cudaMemsetAsync(S.x16.p, 0, bytes, st));
    if (S.fp8) {
        GN_TRY(S.xscale.ensure((size_t)S.n * 4));
        to_e4m3_rows(S.x32.as<float>(), S.n, S.d, S.dp, S.x16.p, S.xscale.as<float>(), S.K, st);
    } else {
        S.xscale.release();
        to_bf16_rows(S.x32.as<float>(), S.n, S.d, S.dp, S.x16.p, S.K, st);
    }
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

// Work units: (query tile, database chunk), chunk-major: the database is cut
// into C chunks and every query tile's unit for chunk c comes before any unit
// of chunk c + 1, the CTAs taking units in turn (unit u: CTA u mod grid).  So
// the CTAs running at any moment scan the same one or two chunks: each chunk
// comes from DRAM about once and is served to the other query tiles from L2.
// A unit starts its lists empty, but below the query's bound published by the
// units that finished before it (tc_topk_kernel), so later chunks insert few
// keys.  C is chosen so that the units fill whole waves of CTAs (chunks of at
// least 32 tiles, and of about 100k rows or more once there are enough units
// for every SM).
static int tcflat_plan(TcFlatState &S, int64_t nq, cudaStream_t st) {
    const int sms = dev_info().num_sms;
    const int64_t qt = ceil_div(nq, TC_M);
    const int64_t nt = ceil_div(S.n, TC_N);
    int64_t C = 1;
    double best = -1.0;
    // chunks of at least ~100k rows once the units fill the SMs: a unit's
    // lists start empty, so the longer its chunk the tighter its threshold
    // over most of it (1M x 128, 10k queries: 6.93 ms at 8 chunks, 7.35 ms at
    // 19, 9.93 ms at 48)
    const int64_t cmax = std::min<int64_t>(std::min<int64_t>(std::max<int64_t>(1, nt / 32), 64),
                                           std::max<int64_t>(ceil_div(sms, qt), S.n / 100000));
    for (int64_t c = 1; c <= cmax; ++c) {
        const int64_t units = qt * c;
        const double eff = (double)units / (double)(ceil_div(units, sms) * sms);
        if (eff > best + 0.02) {  // more chunks only for a clearly fuller last wave
            best = eff;
            C = c;
        }
    }
    std::vector<TcUnit> units;
    units.reserve((size_t)(qt * C));
    for (int64_t c = 0; c < C; ++c) {
        const int64_t t0 = nt * c / C, t1 = nt * (c + 1) / C;
        for (int64_t t = 0; t < qt; ++t) {
            TcUnit u{};
            u.a0 = t * TC_M;
            u.na = (int32_t)std::min<int64_t>(TC_M, nq - u.a0);
            u.r0 = t0 * TC_N;
            u.r1 = std::min<int64_t>(S.n, t1 * TC_N);
            u.rch = (int32_t)c;
            units.push_back(u);
        }
    }
    S.nchunks = (int)C;
    std::vector<int64_t> aslot((size_t)nq);
    for (int64_t q = 0; q < nq; ++q) aslot[(size_t)q] = q * C;
    const int64_t nu = (int64_t)units.size();
    GN_TRY(S.units.ensure(units.size() * sizeof(TcUnit)));
    GN_TRY(S.nunits.ensure(8));
    GN_TRY(S.aslot.ensure((size_t)nq * 8));
    GN_CUDA_TRY(cudaMemcpyAsync(S.units.p, units.data(), units.size() * sizeof(TcUnit), cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.nunits.p, &nu, 8, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.aslot.p, aslot.data(), (size_t)nq * 8, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    S.grid = (int)std::max<int64_t>(1, std::min<int64_t>(sms, nu));
    S.planned_nq = nq;
    return GN_OK;
}

}  // namespace gn

using namespace gn;

static TcFlatState *tcs(gn_index *ix) { return reinterpret_cast<TcFlatState *>(ix->ext); }

extern "C" {

int gn_tcflat_create(int32_t shortlist, gn_index **out) {
    if (!out) return fail(GN_ERR_INVALID, "out is NULL");
    if (shortlist != 16 && shortlist != 32 && shortlist != 40 && shortlist != 48 && shortlist != 56 &&
        shortlist != 64)
        return fail(GN_ERR_INVALID, "shortlist must be 16, 32, 40, 48, 56 or 64");
    gn_index *ix = new gn_index();
    ix->kind = K_TCFLAT;
    ix->metric = GN_METRIC_L2;
    TcFlatState *S = new TcFlatState();
    S->S = shortlist;
    ix->ext = S;
    ix->ext_free = [](void *p) { delete reinterpret_cast<TcFlatState *>(p); };
    *out = ix;
    return GN_OK;
}

int gn_tcflat_set(gn_index *ix, const float *data, int64_t n, int64_t d) {
    if (!ix || ix->kind != K_TCFLAT) return fail(GN_ERR_INVALID, "not a tensor-core flat index");
    if (n <= 0 || d <= 0 || !data) return fail(GN_ERR_INVALID, "data must be a non-empty (N, D) array");
    if (n >= 0x7fffffffLL) return fail(GN_ERR_UNSUPPORTED, "at most 2^31-2 rows");
    std::lock_guard<std::mutex> lk(ix->mu);
    GN_TRY(make_stream(ix));
    TcFlatState &S = *tcs(ix);
    cudaStream_t st = ix->stream;
    S.n = n;
    S.d = (int)d;
    S.dp = (int)round_up(d, 4);
    GN_TRY(upload_rows(S.x32, data, n, d * 4, S.dp / 4, st));
    GN_TRY(S.xnorm.ensure((size_t)n * 4));
    row_norms(S.x32.as<float>(), n, S.dp, S.xnorm.as<float>(), st);  // |x|^2 in FP32
    GN_TRY(tcflat_lowp(S, st));
    GN_TRY(S.err.ensure(4));
    GN_CUDA_TRY(cudaMemsetAsync(S.err.p, 0, 4, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    GN_CUDA_TRY(cudaGetLastError());
    S.planned_nq = -1;
    ix->n = n;
    ix->dim = d;
    return GN_OK;
}

// Argument checks shared by the device- and host-buffer searches.
static int tcflat_check(gn_index *ix, int64_t k) {
    if (!ix || ix->kind != K_TCFLAT) return fail(GN_ERR_INVALID, "not a tensor-core flat index");
    TcFlatState &S = *tcs(ix);
    if (S.n == 0) return fail(GN_ERR_EMPTY, "index is empty");
    if (k <= 0 || k > 32 || k > S.S) return fail(GN_ERR_INVALID, "k must be in [1, min(32, shortlist)]");
    return GN_OK;
}

// The search on device buffers, with the index's lock held by the caller.
static int tcflat_search_locked(gn_index *ix, const float *d_queries, int64_t nq, int64_t k, int64_t *d_idx,
                                float *d_dist, cudaStream_t st) {
    TcFlatState &S = *tcs(ix);
    if (S.planned_nq != nq) GN_TRY(tcflat_plan(S, nq, st));
    GN_TRY(S.q16.ensure((size_t)std::max<int64_t>(nq, TC_M) * S.K * (S.fp8 ? 1 : 2)));  // >= one 128-row TMA box
    GN_TRY(S.part.ensure((size_t)nq * S.nchunks * S.S * 8));
    if (S.fp8) {
        GN_TRY(S.qscale.ensure((size_t)nq * 4));
        to_e4m3_rows(d_queries, nq, S.d, S.dp, S.q16.p, S.qscale.as<float>(), S.K, st);
    } else {
        to_bf16_rows(d_queries, nq, S.d, S.dp, S.q16.p, S.K, st);
    }
    // no bounds yet (every unit of this search publishes into them)
    GN_TRY(S.qbound.ensure((size_t)nq * 4));
    GN_CUDA_TRY(cudaMemsetAsync(S.qbound.p, 0xff, (size_t)nq * 4, st));
    TcLaunch a;
    a.A = S.q16.p;
    a.a_rows = std::max<int64_t>(nq, TC_M);
    a.B = S.x16.p;
    a.b_rows = std::max<int64_t>(S.n, TC_N);
    a.K = S.K;
    a.units = S.units.as<TcUnit>();
    a.n_units = S.nunits.as<int64_t>();
    a.cta_off = nullptr;  // unit u on CTA u mod grid (chunk-major order)
    a.qbound = S.qbound.as<uint32_t>();
    a.bnorm = S.xnorm.as<float>();
    a.arow_slot = S.aslot.as<int64_t>();
    a.part = S.part.as<uint64_t>();
    a.err = S.err.as<int>();
    a.S = S.S;
    a.grid = S.grid;
    a.fp8 = S.fp8;
    a.ascale = S.fp8 ? S.qscale.as<float>() : nullptr;
    a.bscale = S.fp8 ? S.xscale.as<float>() : nullptr;
    timing_begin(st, "tc_topk_kernel");
    GN_TRY(tc_topk_launch(a, st));
    timing_end(st);
    GN_TRY(tc_rerank_launch(S.part.as<uint64_t>(), S.nchunks, S.S, d_queries, S.x32.as<float>(), S.d, S.dp,
                            nullptr, nq, (int)k, 1, d_idx, d_dist, st));
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

int gn_tcflat_search_knn_device(gn_index *ix, const float *d_queries, int64_t nq, int64_t k, int64_t *d_idx,
                                float *d_dist, void *stream) {
    GN_TRY(tcflat_check(ix, k));
    if (nq <= 0) return GN_OK;
    std::lock_guard<std::mutex> lk(ix->mu);
    return tcflat_search_locked(ix, d_queries, nq, k, d_idx, d_dist, (cudaStream_t)stream);
}

int gn_tcflat_search_knn(gn_index *ix, const float *queries, int64_t nq, int64_t k, int64_t *out_idx,
                         float *out_dist) {
    GN_TRY(tcflat_check(ix, k));
    if (nq < 0 || (nq > 0 && (!queries || !out_idx || !out_dist))) return fail(GN_ERR_INVALID, "bad arguments");
    if (nq == 0) return GN_OK;
    TcFlatState &S = *tcs(ix);
    cudaStream_t st = ix->stream;
    // the lock covers the whole call: the query, result and staging buffers are the index's
    std::lock_guard<std::mutex> lk(ix->mu);
    begin_blocking(ix);
    GN_TRY(upload_queries(ix, S.q32, queries, nq, S.d * 4, S.dp / 4, st));
    GN_TRY(S.out_idx.ensure((size_t)nq * k * 8));
    GN_TRY(S.out_dist.ensure((size_t)nq * k * 4));
    GN_TRY(tcflat_search_locked(ix, S.q32.as<float>(), nq, k, S.out_idx.as<int64_t>(), S.out_dist.as<float>(), st));
    GN_TRY(download_result(ix, out_idx, S.out_idx.p, (size_t)nq * k * 8, st));
    GN_TRY(download_result(ix, out_dist, S.out_dist.p, (size_t)nq * k * 4, st));
    return finish_blocking(ix, S.err.as<int>(), st, "tensor-core scan: a pipeline wait timed out");
}

int gn_tcflat_set_precision(gn_index *ix, int32_t precision) {
    if (!ix || ix->kind != K_TCFLAT) return fail(GN_ERR_INVALID, "not a tensor-core flat index");
    if (precision != 0 && precision != 1) return fail(GN_ERR_INVALID, "precision must be 0 (BF16) or 1 (FP8 E4M3)");
    std::lock_guard<std::mutex> lk(ix->mu);
    TcFlatState &S = *tcs(ix);
    if (precision == 1 && S.S > 56)
        return fail(GN_ERR_UNSUPPORTED, "FP8 shortlist: S must be 16, 32, 40, 48 or 56");
    if (S.fp8 == precision) return GN_OK;
    S.fp8 = precision;
    if (S.n > 0) {
        GN_TRY(tcflat_lowp(S, ix->stream));
        GN_CUDA_TRY(cudaStreamSynchronize(ix->stream));
    }
    return GN_OK;
}

int gn_tc_error(gn_index *ix, int32_t *err_out) {
    if (!ix || ix->kind != K_TCFLAT) return fail(GN_ERR_INVALID, "not a tensor-core flat index");
    int herr = 0;
    GN_CUDA_TRY(cudaMemcpy(&herr, tcs(ix)->err.p, 4, cudaMemcpyDeviceToHost));
    if (err_out) *err_out = herr;
    return GN_OK;
}

}  // extern "C"
