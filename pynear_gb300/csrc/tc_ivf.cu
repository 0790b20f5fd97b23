// tc_ivf.cu — tensor-core list scan of the float IVF index (store mode).
//
// Orientation: the list rows are the MMA's M side (128 rows per tile, one per
// TMEM lane) and the queries probing the list are the N side, N = 32, 64 or
// 128 (the smallest that holds the work unit's queries; a unit holds at most
// 128), so the MMA work follows the number of queries actually probing the
// list.  One persistent CTA per SM takes work units (list, chunk of <= 128
// queries, chunk of rows) from an atomic counter, largest lists first; warp 0
// hands each unit index to the other warps through a 4-slot ring of mbarriers:
//   warp 0     TMA: per 64-wide K slice, two tiles of 128 list rows (BF16)
//              and the unit's N query rows (BF16, bucket order) into a
//              4-stage ring — the queries are loaded once per tile pair;
//   warp 1     TMEM (4 accumulators x 128 columns) and tcgen05.mma M=128, N,
//              K=16, the pair's two tiles into two accumulators;
//   warps 2-17 epilogue, two sets of eight: set e takes the tiles whose
//              accumulator index is odd (e = 1) or even (e = 0), so two tiles
//              are drained at once (the drain is latency-bound: more warps in
//              flight hide the TMEM-load, shuffle and reduction latencies);
//              within a set, thread = list row; for each query column its score
//              |x|^2 - 2 q.x (exact FP32 |x|^2) goes to that (query, probe)
//              pair's segment at the row's offset — 32 lanes write 32
//              consecutive rows, so every store is one 128-byte line.  For
//              the list scan, the minimum score of each 32-row quarter of the
//              128-row tile goes to the pair's tile-minimum array, and the
//              quarter's scores are stored only when that minimum is not
//              above the query's score bound (an upper bound on its
//              shortlist-th best score, from the probe stage): the other
//              quarters hold no shortlist candidate and never reach memory.
#include <cuda_bf16.h>

#include <algorithm>

#include "index.cuh"
#include "tc_ivf.cuh"
#include "tc_sm100.cuh"
#include "tmap.cuh"

namespace gn {

constexpr int TI_M = 128, TI_NMAX = 128, TI_BK = 64, TI_STAGES = 4;
constexpr int TI_A_BYTES = TI_M * TI_BK * 2;       // 16 KB
constexpr int TI_B_BYTES = TI_NMAX * TI_BK * 2;    // 16 KB (max)
// a stage holds one K slice of two row tiles (a tile pair) and of the unit's
// queries: the queries' bytes are loaded once per two tiles
constexpr int TI_STAGE_BYTES = 2 * TI_A_BYTES + TI_B_BYTES;
constexpr int TI_NEPI = 16;   // epilogue warps: two sets of eight
constexpr int TI_SET = 8;     // warps per set (4 TMEM lane quadrants x 2 column groups)
constexpr int TI_NACC = 4;    // TMEM accumulators of TI_NMAX columns
constexpr int TI_THREADS = 64 + 32 * TI_NEPI;
constexpr int TI_UR = 4;  // ring of unit indices handed from the producer to the MMA and epilogue warps
constexpr size_t TI_SMEM = 1024 + (size_t)TI_STAGES * TI_STAGE_BYTES + 512;

// order-preserving map of a float to an unsigned key
__device__ __forceinline__ uint32_t ti_ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// its inverse (ordered key -> float); keys above +inf's (all ones: no bound) give +inf
__device__ __forceinline__ float ti_unord(uint32_t k) {
    return k >= 0xff800000u ? INFINITY : __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// minimum of v over the warp (every lane gets it)
__device__ __forceinline__ float ti_warp_min(float v) {
    float r;
    asm("redux.sync.min.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}

__device__ __forceinline__ int ti_nsel(int na) { return na <= 32 ? 32 : na <= 64 ? 64 : 128; }

__global__ void __launch_bounds__(TI_THREADS, 1)
    tc_ivf_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmQ32,
                  const __grid_constant__ CUtensorMap tmQ64, const __grid_constant__ CUtensorMap tmQ128,
                  const TcUnit *__restrict__ units,
                  const int64_t *__restrict__ n_units_ptr, int K, const float *__restrict__ xnorm,
                  const int64_t *__restrict__ aslot, int seg_mul, float *__restrict__ scores,
                  uint32_t *__restrict__ tmin4, const uint32_t *__restrict__ abound, int *__restrict__ err,
                  unsigned long long *__restrict__ next_unit,
                  long long wait_limit, int drill, int tiled) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + TI_STAGES * TI_STAGE_BYTES);
    uint64_t *full = bars, *empty = bars + TI_STAGES, *accfull = bars + 2 * TI_STAGES,
             *accempty = bars + 2 * TI_STAGES + TI_NACC;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * TI_STAGES + 2 * TI_NACC);
    uint64_t *ufull = bars + 2 * TI_STAGES + 2 * TI_NACC + 1, *uempty = ufull + TI_UR;
    volatile int64_t *uring = reinterpret_cast<volatile int64_t *>(uempty + TI_UR);
    // the units' descriptors travel with their indices: the MMA and epilogue
    // warps read them from shared memory, not from global memory at every unit
    TcUnit *uunit = reinterpret_cast<TcUnit *>(const_cast<int64_t *>(uring + TI_UR));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    volatile int *verr = err;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TI_STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < TI_NACC; ++b) {
            mbar_init(accfull + b, 1);
            mbar_init(accempty + b, TI_SET);  // drained by one set
        }
        for (int r = 0; r < TI_UR; ++r) {
            mbar_init(ufull + r, 1);
            mbar_init(uempty + r, 1 + TI_NEPI);
        }
        mbar_fence_init();
    }
    if (warp == 1) tmem_alloc(tmem_slot, 512);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int64_t n_units = *n_units_ptr;
    const int nk = K / TI_BK;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            // units are taken dynamically (atomic counter): unit costs vary
            // by orders of magnitude, a static split would leave SMs idle.
            // The next unit is claimed and its descriptor loaded one unit
            // ahead, so that neither round trip stalls the copies.
            int64_t u_next = (int64_t)atomicAdd(next_unit, 1ull);
            TcUnit un_next = {};
            if (u_next < n_units) un_next = units[u_next];
            for (uint32_t ui = 0; ok; ++ui) {
                const int r = ui % TI_UR;
                if (!mbar_wait(uempty + r, ((ui / TI_UR) & 1) ^ 1, verr, wait_limit)) break;
                const int64_t u = u_next < n_units ? u_next : -1;
                const TcUnit un = un_next;
                if (u >= 0) {
                    u_next = (int64_t)atomicAdd(next_unit, 1ull);
                    if (u_next < n_units) un_next = units[u_next];
                }
                uring[r] = u;
                uunit[r] = un;
                mbar_arrive(ufull + r);
                if (u < 0) break;
                const int nsel = ti_nsel(un.na);
                const CUtensorMap *mq = nsel == 32 ? &tmQ32 : nsel == 64 ? &tmQ64 : &tmQ128;
                const int ntile = (int)((un.r1 - un.r0 + TI_M - 1) / TI_M);
                for (int t = 0; t < ntile && ok; t += 2) {  // tile pairs (the last may be single)
                    const int nt = t + 1 < ntile ? 2 : 1;
                    const uint32_t bytes = (uint32_t)nt * TI_A_BYTES + (uint32_t)nsel * TI_BK * 2;
                    for (int kb = 0; kb < nk; ++kb, ++it) {
                        const int s = it % TI_STAGES;
                        const uint32_t ph = (it / TI_STAGES) & 1;
                        if (!mbar_wait(empty + s, ph ^ 1, verr, wait_limit)) { ok = false; break; }
                        uint8_t *sa = smem + s * TI_STAGE_BYTES;
                        if (drill) continue;  // failure drill: no copies, so the MMA's waits run out
                        mbar_expect_tx(full + s, bytes);
                        for (int h = 0; h < nt; ++h) {
                            if (tiled)  // the tile's K slice kb: one contiguous 16 KB block
                                tma_load_2d(sa + h * TI_A_BYTES, &tmX, 0,
                                            (int)((((un.xrow >> 7) + t + h) * nk + kb) * TI_M), full + s);
                            else
                                tma_load_2d(sa + h * TI_A_BYTES, &tmX, kb * TI_BK,
                                            (int)(un.r0 + (int64_t)(t + h) * TI_M), full + s);
                        }
                        tma_load_2d(sa + 2 * TI_A_BYTES, mq, kb * TI_BK, (int)un.a0, full + s);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t it = 0, tile_it = 0;
            bool ok = true;
            for (uint32_t ui = 0; ok; ++ui) {
                const int r = ui % TI_UR;
                if (!mbar_wait(ufull + r, (ui / TI_UR) & 1, verr, wait_limit)) break;
                const int64_t u = uring[r];
                const TcUnit un = uunit[r];
                mbar_arrive(uempty + r);
                if (u < 0) break;
                const int nsel = ti_nsel(un.na);
                const uint32_t idesc = idesc_bf16_f32(TI_M, nsel);
                const int ntile = (int)((un.r1 - un.r0 + TI_M - 1) / TI_M);
                for (int t = 0; t < ntile && ok; t += 2) {  // tile pairs: two accumulators, one B
                    const int nt = t + 1 < ntile ? 2 : 1;
                    uint32_t dt[2];
                    int bb[2];
                    for (int h = 0; h < nt && ok; ++h) {
                        bb[h] = (tile_it + h) % TI_NACC;
                        const uint32_t tph = ((tile_it + h) / TI_NACC) & 1;
                        if (!mbar_wait(accempty + bb[h], tph ^ 1, verr, wait_limit)) ok = false;
                        dt[h] = tmem + (uint32_t)(bb[h] * TI_NMAX);
                    }
                    if (!ok) break;
                    tc_fence_after();
                    for (int kb = 0; kb < nk; ++kb, ++it) {
                        const int s = it % TI_STAGES;
                        const uint32_t ph = (it / TI_STAGES) & 1;
                        if (!mbar_wait(full + s, ph, verr, wait_limit)) { ok = false; break; }
                        tc_fence_after();
                        const uint32_t sa = smem_u32(smem + s * TI_STAGE_BYTES);
                        const uint64_t db = sdesc_sw128(sa + 2 * TI_A_BYTES);
                        for (int h = 0; h < nt; ++h) {
                            const uint64_t da = sdesc_sw128(sa + h * TI_A_BYTES);
#pragma unroll
                            for (int kk = 0; kk < TI_BK / 16; ++kk)
                                umma_bf16(dt[h], da + 2 * kk, db + 2 * kk, idesc, (kb | kk) ? 1u : 0u);
                        }
                        umma_commit(empty + s);
                    }
                    if (!ok) break;
                    for (int h = 0; h < nt; ++h) umma_commit(accfull + bb[h]);
                    tile_it += nt;
                }
            }
        }
    } else {
        const int quad = warp & 3;
        const int set = (warp - 2) / TI_SET;      // tiles whose accumulator index has parity `set`
        const int grp = ((warp - 2) >> 2) & 1;    // column chunks grp, grp + 2, ...
        uint32_t tile_it = 0;
        bool ok = true;
        for (uint32_t ui = 0; ok; ++ui) {
            const int r = ui % TI_UR;
            if (!mbar_wait(ufull + r, (ui / TI_UR) & 1, verr, wait_limit)) break;
            const int64_t u = uring[r];
            const TcUnit un = uunit[r];
            __syncwarp();
            if (lane == 0) mbar_arrive(uempty + r);
            if (u < 0) break;
            const int nsel = ti_nsel(un.na);
            const int nchunk = nsel / 32;
            // segment base (aslot x seg_mul, minus the list start) and score
            // bound of query column c*32 + lane
            int64_t segv[TI_NMAX / 32 / 2];
            float bndv[TI_NMAX / 32 / 2];
#pragma unroll
            for (int cc = 0; cc < TI_NMAX / 32 / 2; ++cc) {
                const int col = (grp + 2 * cc) * 32 + lane;
                segv[cc] = (col < un.na) ? aslot[un.a0 + col] * seg_mul - un.rbase : INT64_MIN;
                bndv[cc] = (col < un.na && abound) ? ti_unord(abound[un.a0 + col]) : INFINITY;
            }
            const int ntile = (int)((un.r1 - un.r0 + TI_M - 1) / TI_M);
            // |x|^2 of this lane's row in tile t; rows past the list's end (zero
            // rows of the tiled layout) score +inf.  Loaded one of the set's
            // tiles ahead, so that a full accumulator never waits on it.
            auto xload = [&](int t) -> float {
                const int64_t rw = un.r0 + (int64_t)t * TI_M + quad * 32 + lane;
                return rw < un.r1 ? __ldg(xnorm + rw) : INFINITY;
            };
            const int t_first = (set - (int)(tile_it & 1)) & 1;  // the set takes tiles t_first, t_first + 2, ...
            float xn_next = t_first < ntile ? xload(t_first) : 0.f;
            for (int t = 0; t < ntile; ++t, ++tile_it) {
                const int b = tile_it % TI_NACC;
                if ((b & 1) != set) continue;  // the other set's tile
                const uint32_t tph = (tile_it / TI_NACC) & 1;
                const int64_t row = un.r0 + (int64_t)t * TI_M + quad * 32 + lane;
                const bool rok = row < un.r1;
                const float xn = xn_next;
                if (t + 2 < ntile) xn_next = xload(t + 2);
                if (!mbar_wait(accfull + b, tph, verr, wait_limit)) { ok = false; break; }
                tc_fence_after();
#pragma unroll 1
                for (int cc = 0; grp + 2 * cc < nchunk; ++cc) {
                    const int c = grp + 2 * cc;
                    float acc[32];
                    tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * TI_NMAX + c * 32), acc);
                    int64_t sv = segv[0];
                    float bv = bndv[0];
#pragma unroll
                    for (int z = 1; z < TI_NMAX / 32 / 2; ++z)
                        if (cc == z) {
                            sv = segv[z];
                            bv = bndv[z];
                        }
#pragma unroll
                    for (int j = 0; j < 32; ++j) acc[j] = fmaf(-2.f, acc[j], xn);  // the scores
                    unsigned keep = 0xffffffffu;  // columns whose quarter is stored
                    if (tmin4) {
                        // the 32-row minimum of every column (one warp reduction each),
                        // then lane j takes column j's by a select tree on its lane bits
                        float m[32];
#pragma unroll
                        for (int j = 0; j < 32; ++j) m[j] = ti_warp_min(acc[j]);
#pragma unroll
                        for (int h = 16; h >= 1; h >>= 1)
#pragma unroll
                            for (int i = 0; i < h; ++i) m[i] = (lane & h) ? m[i + h] : m[i];
                        const float mymin = m[0];
                        // tile minimum, one word per 32-row quarter: slot = segment base / 128
                        // + the tile's index in the list (segments are 128-aligned)
                        if (sv != INT64_MIN) {
                            const int64_t tile = (sv + un.rbase) / TI_M + (un.r0 - un.rbase) / TI_M + t;
                            tmin4[tile * 4 + quad] = ti_ord(mymin);
                        }
                        // a quarter whose minimum is above its query's bound holds none
                        // of the query's shortlist: its scores are not stored
                        keep = __ballot_sync(0xffffffffu, sv != INT64_MIN && mymin <= bv);
                    }
                    if (keep) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            if (!((keep >> j) & 1u)) continue;  // warp-uniform
                            const int64_t seg = __shfl_sync(0xffffffffu, sv, j);
                            if (seg != INT64_MIN && rok) scores[seg + row] = acc[j];
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(accempty + b);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) tmem_dealloc(tmem, 512);
}

// K-major BF16 rows, boxes of 64 elements (one 128-byte swizzle row) x box_rows rows.
static int tmap(CUtensorMap *m, const void *base, int64_t rows, int K, int box_rows) {
    return tmap_encode_2d(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, base, (uint64_t)K, (uint64_t)rows, (uint64_t)K * 2,
                          TI_BK, (uint32_t)box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

int tc_ivf_launch(const TcIvfLaunch &a, cudaStream_t st) {
    if (a.K % TI_BK) return fail(GN_ERR_INVALID, "tensor-core list scan: K must be a multiple of 64");
    if (a.x_rows < TI_M || a.q_rows < 256) return fail(GN_ERR_INVALID, "tensor-core list scan: buffers too small");
    CUtensorMap mx, m32, m64, m128;
    if (a.tiled) {  // (x_rows / 128) tiles x K/64 slices of 128 rows x 64 values: 64-wide rows of 128 bytes
        if ((a.x_rows & 127) || a.x_rows * (a.K / TI_BK) >= ((int64_t)1 << 31))
            return fail(GN_ERR_INVALID, "tensor-core list scan: tiled rows must be a multiple of 128, below 2^31 slices");
        GN_TRY(tmap(&mx, a.X, a.x_rows * (a.K / TI_BK), TI_BK, TI_M));
    } else {
        GN_TRY(tmap(&mx, a.X, a.x_rows, a.K, TI_M));
    }
    GN_TRY(tmap(&m32, a.Q, a.q_rows, a.K, 32));
    GN_TRY(tmap(&m64, a.Q, a.q_rows, a.K, 64));
    GN_TRY(tmap(&m128, a.Q, a.q_rows, a.K, 128));
    static bool attr = false;
    if (!attr) {
        GN_CUDA_TRY(cudaFuncSetAttribute(tc_ivf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TI_SMEM));
        attr = true;
    }
    if (!a.next_unit) return fail(GN_ERR_INVALID, "tensor-core list scan: no unit counter");
    GN_CUDA_TRY(cudaMemsetAsync(a.next_unit, 0, sizeof(unsigned long long), st));
    tc_ivf_kernel<<<a.grid, TI_THREADS, TI_SMEM, st>>>(mx, m32, m64, m128, a.units, a.n_units, a.K, a.xnorm,
                                                        a.aslot, a.seg_mul, a.scores, a.tmin4, a.abound, a.err,
                                                        a.next_unit,
                                                        a.wait_limit > 0 ? a.wait_limit : TC_TIMEOUT_CYCLES, a.drill,
                                                        a.tiled);
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

}  // namespace gn
