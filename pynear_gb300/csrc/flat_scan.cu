// flat_scan.cu — exact exhaustive k-NN scans (Hamming and float metrics).
//
// Work decomposition: the query set is cut into groups of WARPS*QW queries and
// the database into n_slices row slices; one CTA handles one (slice, group)
// unit.  Units are numbered slice-major so that the CTAs resident at the same
// time read the same slice and share it through L2.  Each warp owns QW queries;
// lane l scores row base+l against all of them (the row stays in registers,
// query words come from shared memory as broadcasts), then offers the keys to
// the warp's register top-k lists.  Each (query, slice) writes its sorted k
// keys to a partial buffer; flat_merge_kernel reduces the slices.
//
// Reference semantics (pynear/include/VPTree.hpp:143-191): exact k nearest rows
// per query; here ties go to the lower row index.
#include "distance.cuh"
#include "flat_scan.cuh"
#include "timing.cuh"
#include "topk.cuh"

namespace gn {

__device__ __forceinline__ uint32_t smem_u32_fs(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

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
// reference's eight-accumulator order needs it).  The rows are not read from
// global memory lane by lane (32 lines per load instruction, which made the L1
// the bottleneck): the CTA stages blocks of rows x 64 floats into shared
// memory with coalesced cp.async copies, double-buffered, at a row stride of
// an odd number of 16-byte words so that the lanes' 16-byte reads of 32
// different rows are free of bank conflicts; the four warps (16 queries)
// share each staged block.  Rows of at most 64 floats are staged 128 rows at
// a time (four row blocks per barrier), longer rows 32 rows x 64 floats.
constexpr int FS_KC4 = 16;  // float4 columns per staged block (64 floats)

struct FsTile {
    int cw;   // float4 columns staged per row (<= FS_KC4)
    int ts4;  // row stride in float4 (odd)
    int rb;   // 32-row blocks per stage
};
__host__ __device__ inline FsTile fs_tile(int dp4) {
    FsTile t;
    t.cw = dp4 < FS_KC4 ? dp4 : FS_KC4;
    t.ts4 = t.cw | 1;
    t.rb = dp4 <= FS_KC4 ? 4 : 1;
    return t;
}
inline size_t fs_tile_bytes(int dp4) {
    const FsTile t = fs_tile(dp4);
    return 2ull * t.rb * 32 * t.ts4 * 16;  // double buffer
}

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32_fs(smem_dst)), "l"(gsrc),
                 "r"(src_bytes)
                 : "memory");
}

template <int METRIC, int QW, int R>
__global__ void __launch_bounds__(128) float_scan_kernel(const float *__restrict__ db, int64_t n, int d, int dp,
                                                         const float *__restrict__ q, int64_t nq, int k,
                                                         int n_slices, int64_t slice_rows, int n_groups,
                                                         uint64_t *__restrict__ part) {
    extern __shared__ float4 sqf[];  // [WARPS*QW][dp/4] queries, then [2][rb * 32][ts4] row blocks
    const int warps = blockDim.x >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int unit = blockIdx.x;
    const int slice = unit / n_groups, group = unit % n_groups;
    const int64_t q0 = (int64_t)group * warps * QW;
    const int dp4 = dp >> 2;
    float4 *tile = sqf + warps * QW * dp4;

    const float4 *q4 = reinterpret_cast<const float4 *>(q);
    for (int i = threadIdx.x; i < warps * QW * dp4; i += blockDim.x) {
        int64_t qi = q0 + i / dp4;
        sqf[i] = (qi < nq) ? q4[qi * dp4 + (i % dp4)] : make_float4(0.f, 0.f, 0.f, 0.f);
    }

    const int64_t r0 = (int64_t)slice * slice_rows;
    const int64_t r1 = min(n, r0 + slice_rows);
    const float4 *myq = sqf + warp * QW * dp4;
    const int nb = d >> 3, rem = d & 7;
    const int tail4 = 2 * nb;  // float4 index of the remainder pair (when rem > 0)
    const int nchunk = (dp4 + FS_KC4 - 1) / FS_KC4;
    const FsTile ft = fs_tile(dp4);
    const int srows = ft.rb * 32;  // rows per stage
    const int64_t nrb = (r1 - r0 + srows - 1) / srows;
    const int64_t nstage = nrb * nchunk;
    const float4 *db4 = reinterpret_cast<const float4 *>(db);

    // stage si = (row group si / nchunk, column block si % nchunk) into buffer buf
    auto issue = [&](int64_t si, int buf) {
        const int64_t base = r0 + (si / nchunk) * srows;
        const int c0 = (int)(si % nchunk) * FS_KC4;
        const int cw = min(FS_KC4, dp4 - c0);
        float4 *dst = tile + buf * srows * ft.ts4;
        for (int i = threadIdx.x; i < srows * cw; i += blockDim.x) {
            const int r = i / cw, c = i - r * cw;
            const int64_t row = base + r;
            const bool ok = row < r1;
            cp_async16(dst + r * ft.ts4 + c, db4 + (ok ? row : r0) * dp4 + c0 + c, ok ? 16 : 0);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };

    WarpTopK<R> lists[QW];
    uint64_t thr[QW];
#pragma unroll
    for (int j = 0; j < QW; ++j) { lists[j].init(); thr[j] = KEY_EMPTY; }

    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    FAcc<METRIC> acc[QW];
    float4 x0t = zero4, x1t = zero4;  // the row's remainder pair
    if (nstage > 0) issue(0, 0);
    for (int64_t si = 0; si < nstage; ++si) {
        if (si + 1 < nstage) {
            issue(si + 1, (int)((si + 1) & 1));
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();  // stage si (and, the first time, the queries) visible to every warp
        const int kc = (int)(si % nchunk);
        const int c0 = kc * FS_KC4;
        const int cb0 = c0 >> 1, cb1 = min(nb, (c0 + FS_KC4) >> 1);  // full blocks of eight in this column block
        // rb > 1 only when the whole row is one column block (kc == 0 == nchunk - 1)
        for (int rb = 0; rb < ft.rb; ++rb) {
            // rp[c] = float4 c of this lane's row
            const float4 *rp = tile + ((si & 1) * srows + rb * 32 + lane) * ft.ts4 - c0;
            if (kc == 0) {
#pragma unroll
                for (int j = 0; j < QW; ++j) acc[j].zero();
            }
#pragma unroll 2
            for (int c = cb0; c < cb1; ++c) {
                const float4 x0 = rp[2 * c], x1 = rp[2 * c + 1];
#pragma unroll
                for (int j = 0; j < QW; ++j) acc[j].block8(myq[j * dp4 + 2 * c], myq[j * dp4 + 2 * c + 1], x0, x1);
            }
            if (rem > 0 && tail4 >= c0 && tail4 < c0 + FS_KC4) {
                x0t = rp[tail4];
                if (rem > 4) x1t = rp[tail4 + 1];
            }
            if (kc == nchunk - 1) {
                const int64_t row = r0 + (si / nchunk) * srows + rb * 32 + lane;
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
        __syncthreads();  // buffer si & 1 is refilled by the next iteration's issue
    }
#pragma unroll
    for (int j = 0; j < QW; ++j) {
        int64_t qi = q0 + warp * QW + j;
        if (qi < nq) lists[j].store(part + ((size_t)qi * n_slices + slice) * k, k);
    }
}

// ── merge of per-slice partial lists → final output ───────────────────────
// One warp per query.  Output: idx (int64, -1 for empty), dist as float32
// (float metrics) or int64 (Hamming).
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
    for (int s = 0; s < n_slices; ++s) {
        for (int j0 = 0; j0 < k; j0 += 32) {
            int j = j0 + lane;
            uint64_t key = (j < k) ? p[(size_t)s * k + j] : KEY_EMPTY;
            // partial lists are sorted: once the smallest unseen key of this
            // chunk is above the threshold the rest of the list is too
            if (__all_sync(0xffffffffu, key >= thr)) break;
            L.offer(key, thr, k);
        }
    }
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
static void launch_scan(const FlatScanArgs &a, int n_groups, int threads, size_t smem, uint64_t *part,
                        cudaStream_t st) {
    const int units = n_groups * a.n_slices;
    timing_begin(st, a.metric == M_HAMMING ? "hamming_scan_kernel" : "float_scan_kernel");
    if (a.metric == M_HAMMING) {
        auto kern = hamming_scan_kernel<8, R>;
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        kern<<<units, threads, smem, st>>>(reinterpret_cast<const uint4 *>(a.db), a.n, a.stride4,
                                           reinterpret_cast<const uint4 *>(a.q), a.nq, a.k, a.n_slices, a.slice_rows,
                                           n_groups, part);
    } else {
#define GN_FLOAT_SCAN(M)                                                                                          \
    do {                                                                                                          \
        auto kern = float_scan_kernel<M, 4, R>;                                                                   \
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        kern<<<units, threads, smem, st>>>(reinterpret_cast<const float *>(a.db), a.n, a.d, a.stride4 * 4,        \
                                           reinterpret_cast<const float *>(a.q), a.nq, a.k, a.n_slices,           \
                                           a.slice_rows, n_groups, part);                                         \
    } while (0)
        if (a.metric == M_L2) GN_FLOAT_SCAN(M_L2);
        else if (a.metric == M_L1) GN_FLOAT_SCAN(M_L1);
        else GN_FLOAT_SCAN(M_LINF);
#undef GN_FLOAT_SCAN
    }
    timing_end(st);
    const int qpb = 4;  // queries (warps) per merge block
    flat_merge_kernel<R><<<(unsigned)ceil_div(a.nq, qpb), qpb * 32, 0, st>>>(
        part, a.n_slices, a.k, a.nq, a.metric == M_HAMMING, a.out_idx, a.out_dist);
}

// CTAs of the float scan resident per SM for this metric and list size.
template <int R>
static int float_scan_occupancy(int metric, int threads, size_t smem) {
    int nb = 0;
    cudaError_t e;
    if (metric == M_L2)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, float_scan_kernel<M_L2, 4, R>, threads, smem);
    else if (metric == M_L1)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, float_scan_kernel<M_L1, 4, R>, threads, smem);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, float_scan_kernel<M_LINF, 4, R>, threads, smem);
    if (e != cudaSuccess) {  // a refused query (e.g. shared memory above the default) reads as 0
        cudaGetLastError();
        nb = 0;
    }
    return nb;
}

void flat_plan(FlatScanArgs &a) {
    const DevInfo &di = dev_info();
    const int qw = (a.metric == M_HAMMING) ? 8 : 4;
    const size_t per_warp = (size_t)qw * a.stride4 * 16;
    int warps = 4;
    while (warps > 1 && per_warp * warps > 200 * 1024) warps >>= 1;
    a.warps = warps;
    a.qw = qw;
    const int64_t n_groups = ceil_div(a.nq, (int64_t)warps * qw);
    const int64_t max_slices = std::max<int64_t>(1, a.n / 512);  // slices of at least 512 rows
    int64_t slices;
    if (a.metric == M_HAMMING) {
        // aim for ~16 CTAs per SM over the launch
        slices = std::min<int64_t>(std::max<int64_t>(1, ceil_div(16LL * di.num_sms, n_groups)), max_slices);
    } else {
        // units of equal cost: pick the slice count (up to about four waves of
        // resident CTAs) whose last wave is fullest, the fewest slices on a tie
        const int threads = warps * 32;
        const size_t smem = (size_t)warps * qw * a.stride4 * 16 + fs_tile_bytes(a.stride4);
        int occ = a.k <= 32 ? float_scan_occupancy<1>(a.metric, threads, smem)
                  : a.k <= 64 ? float_scan_occupancy<2>(a.metric, threads, smem)
                  : a.k <= 128 ? float_scan_occupancy<4>(a.metric, threads, smem)
                               : float_scan_occupancy<8>(a.metric, threads, smem);
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
    a.slice_rows = round_up(ceil_div(a.n, slices), 32);
    a.n_slices = (int)ceil_div(a.n, a.slice_rows);
    a.n_groups = (int)n_groups;
}

size_t flat_part_bytes(const FlatScanArgs &a) { return (size_t)a.nq * a.n_slices * a.k * sizeof(uint64_t); }

static size_t flat_smem_bytes(const FlatScanArgs &a) {
    return (size_t)a.warps * a.qw * a.stride4 * 16 + (a.metric == M_HAMMING ? 0 : fs_tile_bytes(a.stride4));
}

int flat_smem_ok(const FlatScanArgs &a) {
    return flat_smem_bytes(a) <= (size_t)dev_info().max_smem_optin;
}

// Launch the warp-select path (k <= 256).  part: flat_part_bytes(a) scratch.
void flat_launch(const FlatScanArgs &a, uint64_t *part, cudaStream_t st) {
    const int threads = a.warps * 32;
    const size_t smem = flat_smem_bytes(a);
    if (a.k <= 32) launch_scan<1>(a, a.n_groups, threads, smem, part, st);
    else if (a.k <= 64) launch_scan<2>(a, a.n_groups, threads, smem, part, st);
    else if (a.k <= 128) launch_scan<4>(a, a.n_groups, threads, smem, part, st);
    else launch_scan<8>(a, a.n_groups, threads, smem, part, st);
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
                         (const void *)flat_merge_kernel<4>,      (const void *)flat_merge_kernel<8>};
    for (const void *f : fns) GN_CUDA_TRY(cudaFuncGetAttributes(&fa, f));
    return GN_OK;
}

}  // namespace gn
