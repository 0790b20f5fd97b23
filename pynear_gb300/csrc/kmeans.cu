// kmeans.cu — float and binary k-means on the device.
//
// Float (replaces kmeans_l2, pynear/include/KMeans.hpp:25-126):
//   seeding   k-means++ exactly as the reference: mt19937(seed) draws on the
//             host (taken up front: they do not depend on the data), squared
//             dist_l2_f_avx2 distances computed on the device in the
//             reference's arithmetic order, the weighted pick on the device
//             from double running sums, with the reference's serial double
//             sums deciding where the two orders could disagree (so the seeds
//             are the reference's);
//   assign    argmin_c (|c|^2 - 2 x.c) from an FP32 tile GEMM with a fused
//             argmin epilogue (first minimum wins, like the reference);
//   update    per-cluster sums in FP64 (atomic adds), divided once and rounded
//             to float; empty clusters re-seeded with pick_point(rng) in
//             cluster order, as the reference does.
// Binary (replaces IVFFlatBinaryIndex::_build, pynear/include/BinaryIVF.hpp:
// 127-227): integer arithmetic throughout, so the device build reproduces the
// reference's centroids and labels exactly: the same mt19937 stream (pick, then
// wsel over [0,total)), exact int64 sums and prefix search, first-minimum
// Hamming assignment, majority vote count > n_c/2, empty clusters re-seeded.
#include <algorithm>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#include "distance.cuh"
#include "gemm_topk.cuh"
#include "index.cuh"
#include "kmeans.cuh"

namespace gn {

// ── float seeding ─────────────────────────────────────────────────────────
__global__ void kpp_update_kernel(const float *__restrict__ X, int64_t n, int d, int dp,
                                  const float *__restrict__ c, float *__restrict__ min_sq) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = fdist<M_L2>(c, X + i * dp, d);
    v = __fmul_rn(v, v);
    if (v < min_sq[i]) min_sq[i] = v;
}

// Per chunk of min_sq (block b: elements [b * chunk, (b + 1) * chunk)), the sum
// in double, in a fixed order (thread-strided, then a fixed tree).
__global__ void __launch_bounds__(256) kpp_partial_kernel(const float *__restrict__ min_sq, int64_t n,
                                                          int64_t chunk, double *__restrict__ part) {
    __shared__ double red[256];
    const int64_t b0 = (int64_t)blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    double s = 0.0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += 256) s += (double)min_sq[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// k-means++ draw of centroid ci (one block of 1024 threads), the reference's
// rule (KMeans.hpp:45-70): r = u * sum(min_sq), the first point whose running
// sum reaches r (n - 1 if none).  The reference sums in double in point order;
// here the sums are the chunk partials, scanned, then the chosen chunk's
// elements.  Both orders' running sums lie within 2 (n - 1) 2^-53 total of the
// exact ones, so when r is farther than twice that from the chosen point's
// running sums on both sides, the serial order chooses the same point; if not,
// thread 0 repeats the reference's serial loop (rare).  The chosen row is
// copied to C[ci].
__global__ void __launch_bounds__(1024) kpp_pick_kernel(const float *__restrict__ min_sq, int64_t n, int64_t chunk,
                                                        int P, const double *__restrict__ part, float u,
                                                        const float *__restrict__ X, int dp, float *__restrict__ C,
                                                        int64_t ci) {
    __shared__ double pre[1024], wsum[32];
    __shared__ int s_b, s_amb, s_found;
    __shared__ int64_t s_chosen;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // exclusive scan of the chunk sums (P <= 1024)
    const double v = t < P ? part[t] : 0.0;
    double inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    if (t == 0) {
        s_b = P;
        s_amb = 0;
        s_found = 0;
        s_chosen = n - 1;
    }
    __syncthreads();
    double wb = 0.0;
    for (int w = 0; w < warp; ++w) wb += wsum[w];
    pre[t] = wb + inc - v;
    double total = 0.0;
    for (int w = 0; w < 32; ++w) total += wsum[w];
    const double r = (double)u * total;
    const double band = 4.0 * (double)n * 1.1102230246251565e-16 * total;  // 2 x 2 (n - 1) 2^-53 total, rounded up
    __syncthreads();
    if (t < P && pre[t] + v >= r) atomicMin(&s_b, t);
    __syncthreads();
    const int b = s_b;
    if (b < P) {
        // running sums inside chunk b: each thread takes a contiguous piece
        const int64_t c0 = (int64_t)b * chunk, c1 = min(n, c0 + chunk);
        const int64_t per = (c1 - c0 + 1023) / 1024;
        const int64_t p0 = min(c1, c0 + t * per), p1 = min(c1, p0 + per);
        double ls = 0.0;
        for (int64_t i = p0; i < p1; ++i) ls += (double)min_sq[i];
        double li = ls;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, li, o);
            if (lane >= o) li += y;
        }
        if (lane == 31) wsum[warp] = li;
        __syncthreads();
        double base = pre[b];
        for (int w = 0; w < warp; ++w) base += wsum[w];
        double cum = base + li - ls;  // running sum before this thread's piece
        int64_t found = -1;
        double before = 0.0, at = 0.0;
        for (int64_t i = p0; i < p1; ++i) {
            const double nx = cum + (double)min_sq[i];
            if (nx >= r) {
                found = i;
                before = cum;
                at = nx;
                break;
            }
            cum = nx;
        }
        // the first piece holding the point: pieces are ordered, so the lowest index wins
        if (found >= 0) {
            atomicMin(reinterpret_cast<unsigned long long *>(&s_chosen), (unsigned long long)found);
            s_found = 1;
        }
        __syncthreads();
        if (found >= 0 && found == s_chosen && !(at - r > band && r - before > band)) s_amb = 1;
        // the chunk's elements summed in this order fell short of r: the serial rule decides
        if (t == 0 && !s_found) s_amb = 1;
    } else if (t == 0) {
        s_amb = 1;  // r beyond every partial sum: the serial rule decides
    }
    __syncthreads();
    if (s_amb && t == 0) {
        double tot = 0.0;
        for (int64_t i = 0; i < n; ++i) tot += (double)min_sq[i];
        const double rr = (double)u * tot;
        double c = 0.0;
        int64_t ch = n - 1;
        for (int64_t i = 0; i < n; ++i) {
            c += (double)min_sq[i];
            if (c >= rr) {
                ch = i;
                break;
            }
        }
        s_chosen = ch;
    }
    __syncthreads();
    const int64_t ch = s_chosen;
    for (int j = t; j < dp; j += 1024) C[ci * dp + j] = X[ch * dp + j];
}

__global__ void fill_float_kernel(float *p, int64_t n, float v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// ── row norms ─────────────────────────────────────────────────────────────
__global__ void row_norms_kernel(const float *__restrict__ X, int64_t n, int dp, float *__restrict__ out) {
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    float s = 0.f;
    for (int j = lane; j < dp; j += 32) {
        float v = X[row * dp + j];
        s = fmaf(v, v, s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[row] = s;
}

// ── float assignment: tile GEMM + argmin ──────────────────────────────────
__global__ void __launch_bounds__(GT_THREADS) kmeans_assign_kernel(const float *__restrict__ X, int64_t n, int dp,
                                                                   const float *__restrict__ C,
                                                                   const float *__restrict__ cnorm, int k,
                                                                   int32_t *__restrict__ labels,
                                                                   unsigned long long *__restrict__ n_changed) {
    __shared__ GemmTileSmem s;
    __shared__ int64_t arow[GT_BM];
    const int64_t p0 = (int64_t)blockIdx.x * GT_BM;
    if (threadIdx.x < GT_BM) arow[threadIdx.x] = (p0 + threadIdx.x < n) ? p0 + threadIdx.x : -1;
    __syncthreads();
    const int tm = threadIdx.x >> 5, tn = threadIdx.x & 31;
    uint64_t best[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) best[i] = KEY_EMPTY;
    float acc[8][4];
    for (int c0 = 0; c0 < k; c0 += GT_BN) {
        gt_tile(s, acc, X, arow, dp, C, c0, k, dp, dp);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + tn * 4 + j;
            if (c < k) {
                const float cn = cnorm[c];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float v = fmaf(-2.f, acc[i][j], cn);
                    const uint64_t key = make_key(f2ord(v), (uint32_t)c);
                    best[i] = key < best[i] ? key : best[i];
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        uint64_t b = best[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            uint64_t other = __shfl_xor_sync(0xffffffffu, b, o);
            b = other < b ? other : b;
        }
        best[i] = b;
    }
    if (tn == 0) {
        unsigned long long changed = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int64_t p = p0 + tm * 8 + i;
            if (p < n) {
                const int32_t lab = (int32_t)key_idx(best[i]);
                if (labels[p] != lab) { labels[p] = lab; ++changed; }
            }
        }
        if (changed) atomicAdd(n_changed, changed);
    }
}

// ── float update: FP64 sums ───────────────────────────────────────────────
__global__ void kmeans_accumulate_kernel(const float *__restrict__ X, int64_t n, int d, int dp,
                                         const int32_t *__restrict__ labels, double *__restrict__ sums,
                                         int64_t *__restrict__ counts) {
    const int64_t p = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= n) return;
    const int32_t c = labels[p];
    if (lane == 0) atomicAdd(reinterpret_cast<unsigned long long *>(counts + c), 1ull);
    for (int j = lane; j < d; j += 32) atomicAdd(sums + (int64_t)c * dp + j, (double)X[p * dp + j]);
}

__global__ void kmeans_finalize_kernel(const double *__restrict__ sums, const int64_t *__restrict__ counts, int k,
                                       int d, int dp, float *__restrict__ C) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)k * dp) return;
    const int c = (int)(t / dp), j = (int)(t % dp);
    if (counts[c] > 0) C[t] = (j < d) ? (float)(sums[t] / (double)counts[c]) : 0.f;
}

int kmeans_l2_device(const float *X, int64_t n, int d, int dp, int64_t k, int64_t max_iter, uint32_t seed,
                     float *C, float *cnorm, int32_t *labels, int64_t *iters_out, cudaStream_t st) {
    if (dp % GT_BK) return fail(GN_ERR_INVALID, "kmeans: row stride must be a multiple of 16 floats");
    std::mt19937 rng(seed);
    std::uniform_int_distribution<size_t> pick_point(0, (size_t)n - 1);
    std::uniform_real_distribution<float> unif01(0.f, 1.f);
    const size_t row_bytes = (size_t)dp * sizeof(float);

    // k-means++ seeding, all on the device: the reference's draws (the first
    // point, then one uniform per further centroid) do not depend on the data,
    // so they are taken from the mt19937 stream up front in the reference's
    // order; each further centroid is then picked by kpp_pick_kernel
    GN_CUDA_TRY(cudaMemcpyAsync(C, X + pick_point(rng) * dp, row_bytes, cudaMemcpyDeviceToDevice, st));
    std::vector<float> draws((size_t)std::max<int64_t>(k, 1));
    for (int64_t ci = 1; ci < k; ++ci) draws[(size_t)ci] = unif01(rng);
    DBuf dmin, dpart;
    GN_TRY(dmin.ensure((size_t)n * sizeof(float)));
    const int64_t chunk = std::max<int64_t>(256, ceil_div(n, 1024));
    const int P = (int)ceil_div(n, chunk);  // <= 1024 chunk sums
    GN_TRY(dpart.ensure((size_t)P * sizeof(double)));
    const unsigned nb = (unsigned)ceil_div(n, 256);
    fill_float_kernel<<<nb, 256, 0, st>>>(dmin.as<float>(), n, std::numeric_limits<float>::max());
    for (int64_t ci = 1; ci < k; ++ci) {
        kpp_update_kernel<<<nb, 256, 0, st>>>(X, n, d, dp, C + (ci - 1) * dp, dmin.as<float>());
        kpp_partial_kernel<<<(unsigned)P, 256, 0, st>>>(dmin.as<float>(), n, chunk, dpart.as<double>());
        kpp_pick_kernel<<<1, 1024, 0, st>>>(dmin.as<float>(), n, chunk, P, dpart.as<double>(), draws[(size_t)ci], X,
                                            dp, C, ci);
    }
    GN_CUDA_TRY(cudaGetLastError());

    // Lloyd iterations
    DBuf dsum, dcnt, dchg;
    GN_TRY(dsum.ensure((size_t)k * dp * sizeof(double)));
    GN_TRY(dcnt.ensure((size_t)k * sizeof(int64_t)));
    GN_TRY(dchg.ensure(sizeof(unsigned long long)));
    GN_CUDA_TRY(cudaMemsetAsync(labels, 0, (size_t)n * sizeof(int32_t), st));
    std::vector<int64_t> hcnt((size_t)k);
    int64_t it = 0;
    for (; it < max_iter; ++it) {
        row_norms_kernel<<<(unsigned)ceil_div(k, 8), 256, 0, st>>>(C, k, dp, cnorm);
        GN_CUDA_TRY(cudaMemsetAsync(dchg.p, 0, sizeof(unsigned long long), st));
        kmeans_assign_kernel<<<(unsigned)ceil_div(n, GT_BM), GT_THREADS, 0, st>>>(
            X, n, dp, C, cnorm, (int)k, labels, dchg.as<unsigned long long>());
        unsigned long long changed = 0;
        GN_CUDA_TRY(cudaMemcpyAsync(&changed, dchg.p, sizeof(changed), cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        if (changed == 0) break;
        GN_CUDA_TRY(cudaMemsetAsync(dsum.p, 0, (size_t)k * dp * sizeof(double), st));
        GN_CUDA_TRY(cudaMemsetAsync(dcnt.p, 0, (size_t)k * sizeof(int64_t), st));
        kmeans_accumulate_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, st>>>(X, n, d, dp, labels, dsum.as<double>(),
                                                                          dcnt.as<int64_t>());
        kmeans_finalize_kernel<<<(unsigned)ceil_div(k * dp, 256), 256, 0, st>>>(dsum.as<double>(),
                                                                              dcnt.as<int64_t>(), (int)k, d, dp, C);
        GN_CUDA_TRY(cudaMemcpyAsync(hcnt.data(), dcnt.p, (size_t)k * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        for (int64_t c = 0; c < k; ++c)
            if (hcnt[(size_t)c] == 0)
                GN_CUDA_TRY(cudaMemcpyAsync(C + c * dp, X + pick_point(rng) * dp, row_bytes,
                                            cudaMemcpyDeviceToDevice, st));
    }
    row_norms_kernel<<<(unsigned)ceil_div(k, 8), 256, 0, st>>>(C, k, dp, cnorm);
    GN_CUDA_TRY(cudaGetLastError());
    if (iters_out) *iters_out = it;
    return GN_OK;
}

void row_norms(const float *X, int64_t n, int dp, float *out, cudaStream_t st) {
    if (n > 0) row_norms_kernel<<<(unsigned)ceil_div(n, 8), 256, 0, st>>>(X, n, dp, out);
}

// ── binary k-means ────────────────────────────────────────────────────────
__global__ void bin_kpp_update_kernel(const uint4 *__restrict__ X, int64_t n, int w4, const uint4 *__restrict__ c,
                                      int64_t *__restrict__ min_d) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t v = hdist(c, X + i * w4, w4);
    if (v < min_d[i]) min_d[i] = v;
}

__global__ void fill_i64_kernel(int64_t *p, int64_t n, int64_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

constexpr int SCAN_CHUNK = 4096;

// per-chunk sums of min_d (exact int64)
__global__ void chunk_sum_kernel(const int64_t *__restrict__ v, int64_t n, int64_t *__restrict__ sums) {
    __shared__ int64_t red[32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_CHUNK;
    int64_t s = 0;
    for (int i = threadIdx.x; i < SCAN_CHUNK; i += blockDim.x)
        if (base + i < n) s += v[base + i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        sums[blockIdx.x] = t;
    }
}

// first index i with prefix_sum(v)[0..i] > r (exact int64), one block
__global__ void find_weighted_kernel(const int64_t *__restrict__ v, int64_t n, const int64_t *__restrict__ sums,
                                     int64_t nchunks, int64_t r, int64_t *__restrict__ out) {
    __shared__ int64_t s_chunk, s_before;
    if (threadIdx.x == 0) {
        int64_t cum = 0, c = 0;
        for (; c < nchunks; ++c) {
            if (cum + sums[c] > r) break;
            cum += sums[c];
        }
        s_chunk = c;
        s_before = cum;
        int64_t res = -1;
        if (c < nchunks) {
            const int64_t base = c * SCAN_CHUNK;
            for (int64_t i = base; i < min(n, base + SCAN_CHUNK); ++i) {
                cum += v[i];
                if (cum > r) { res = i; break; }
            }
        }
        *out = res;
    }
}

// assignment to the first nearest centroid; centroids staged in shared memory
__global__ void bin_assign_kernel(const uint4 *__restrict__ X, int64_t n, int w4, const uint4 *__restrict__ C, int k,
                                  int32_t *__restrict__ labels, unsigned long long *__restrict__ n_changed) {
    extern __shared__ uint4 sc[];
    for (int i = threadIdx.x; i < k * w4; i += blockDim.x) sc[i] = C[i];
    __syncthreads();
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool changed = false;
    if (p < n) {
        uint32_t best = 0xffffffffu;
        int32_t bc = 0;
        const uint4 *x = X + p * w4;
        if (w4 == 4) {
            const uint4 x0 = x[0], x1 = x[1], x2 = x[2], x3 = x[3];
            for (int c = 0; c < k; ++c) {
                const uint4 *cc = sc + c * 4;
                const uint32_t dd = popc4(x0, cc[0]) + popc4(x1, cc[1]) + popc4(x2, cc[2]) + popc4(x3, cc[3]);
                if (dd < best) { best = dd; bc = c; }
            }
        } else {
            for (int c = 0; c < k; ++c) {
                const uint32_t dd = hdist(x, sc + c * w4, w4);
                if (dd < best) { best = dd; bc = c; }
            }
        }
        if (labels[p] != bc) { labels[p] = bc; changed = true; }
    }
    const unsigned m = __ballot_sync(0xffffffffu, changed);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(n_changed, (unsigned long long)__popc(m));
}

// bit counts per cluster: one thread per (point, 32-bit word)
__global__ void bin_bitcount_kernel(const uint32_t *__restrict__ X, int64_t n, int w32, int nbits,
                                    const int32_t *__restrict__ labels, int32_t *__restrict__ counts,
                                    int32_t *__restrict__ cc) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * w32) return;
    const int64_t p = t / w32;
    const int w = (int)(t % w32);
    const int32_t c = labels[p];
    if (w == 0) atomicAdd(cc + c, 1);
    uint32_t bits = X[p * w32 + w];
    while (bits) {
        const int b = __ffs(bits) - 1;
        bits &= bits - 1;
        const int bit = w * 32 + b;
        if (bit < nbits) atomicAdd(counts + (int64_t)c * nbits + bit, 1);
    }
}

// majority vote (count > n_c / 2); clusters with no point are left for the host
__global__ void bin_majority_kernel(const int32_t *__restrict__ counts, const int32_t *__restrict__ cc, int k,
                                    int nbits, int w32, uint32_t *__restrict__ C) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)k * w32) return;
    const int c = (int)(t / w32), w = (int)(t % w32);
    if (cc[c] == 0) return;
    const int32_t half = cc[c] / 2;
    uint32_t word = 0;
    for (int b = 0; b < 32; ++b) {
        const int bit = w * 32 + b;
        if (bit < nbits && counts[(int64_t)c * nbits + bit] > half) word |= 1u << b;
    }
    C[t] = word;
}

int kmeans_bin_device(const uint8_t *X, int64_t n, int nbytes, int w4, int32_t k, int32_t max_iter, uint32_t seed,
                      uint8_t *C, int32_t *labels, cudaStream_t st) {
    std::mt19937 rng(seed);
    std::uniform_int_distribution<size_t> pick(0, (size_t)n - 1);
    const size_t row = (size_t)w4 * 16;
    const uint4 *X4 = reinterpret_cast<const uint4 *>(X);
    GN_CUDA_TRY(cudaMemcpyAsync(C, X + pick(rng) * row, row, cudaMemcpyDeviceToDevice, st));
    DBuf dmin, dsums, dout;
    const int64_t nchunks = ceil_div(n, SCAN_CHUNK);
    GN_TRY(dmin.ensure((size_t)n * 8));
    GN_TRY(dsums.ensure((size_t)nchunks * 8));
    GN_TRY(dout.ensure(8));
    const unsigned nb = (unsigned)ceil_div(n, 256);
    fill_i64_kernel<<<nb, 256, 0, st>>>(dmin.as<int64_t>(), n, std::numeric_limits<int64_t>::max());
    std::vector<int64_t> hs((size_t)nchunks);
    for (int32_t ci = 1; ci < k; ++ci) {
        bin_kpp_update_kernel<<<nb, 256, 0, st>>>(X4, n, w4, reinterpret_cast<const uint4 *>(C + (size_t)(ci - 1) * row),
                                                  dmin.as<int64_t>());
        chunk_sum_kernel<<<(unsigned)nchunks, 256, 0, st>>>(dmin.as<int64_t>(), n, dsums.as<int64_t>());
        GN_CUDA_TRY(cudaMemcpyAsync(hs.data(), dsums.p, (size_t)nchunks * 8, cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        int64_t total = 0;
        for (int64_t v : hs) total += v;
        size_t chosen = pick(rng);
        if (total > 0) {
            std::uniform_int_distribution<int64_t> wsel(0, total - 1);
            const int64_t r = wsel(rng);
            find_weighted_kernel<<<1, 32, 0, st>>>(dmin.as<int64_t>(), n, dsums.as<int64_t>(), nchunks, r,
                                                   dout.as<int64_t>());
            int64_t res = -1;
            GN_CUDA_TRY(cudaMemcpyAsync(&res, dout.p, 8, cudaMemcpyDeviceToHost, st));
            GN_CUDA_TRY(cudaStreamSynchronize(st));
            if (res >= 0) chosen = (size_t)res;
        }
        GN_CUDA_TRY(cudaMemcpyAsync(C + (size_t)ci * row, X + chosen * row, row, cudaMemcpyDeviceToDevice, st));
    }

    const int nbits = nbytes * 8;
    const int w32 = w4 * 4;
    DBuf dcounts, dcc, dchg;
    GN_TRY(dcounts.ensure((size_t)k * nbits * 4));
    GN_TRY(dcc.ensure((size_t)k * 4));
    GN_TRY(dchg.ensure(8));
    GN_CUDA_TRY(cudaMemsetAsync(labels, 0, (size_t)n * 4, st));
    const size_t smem = (size_t)k * row;
    if (smem > (size_t)dev_info().max_smem_optin)
        return fail(GN_ERR_UNSUPPORTED, "binary k-means: nlist * row bytes exceeds shared memory");
    if (smem > 48 * 1024)
        GN_CUDA_TRY(cudaFuncSetAttribute(bin_assign_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    std::vector<int32_t> hcc((size_t)k);
    for (int32_t it = 0; it < max_iter; ++it) {
        GN_CUDA_TRY(cudaMemsetAsync(dchg.p, 0, 8, st));
        bin_assign_kernel<<<nb, 256, smem, st>>>(X4, n, w4, reinterpret_cast<const uint4 *>(C), k, labels,
                                                 dchg.as<unsigned long long>());
        unsigned long long changed = 0;
        GN_CUDA_TRY(cudaMemcpyAsync(&changed, dchg.p, 8, cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        if (changed == 0) break;
        GN_CUDA_TRY(cudaMemsetAsync(dcounts.p, 0, (size_t)k * nbits * 4, st));
        GN_CUDA_TRY(cudaMemsetAsync(dcc.p, 0, (size_t)k * 4, st));
        bin_bitcount_kernel<<<(unsigned)ceil_div(n * w32, 256), 256, 0, st>>>(
            reinterpret_cast<const uint32_t *>(X), n, w32, nbits, labels, dcounts.as<int32_t>(), dcc.as<int32_t>());
        bin_majority_kernel<<<(unsigned)ceil_div((int64_t)k * w32, 256), 256, 0, st>>>(
            dcounts.as<int32_t>(), dcc.as<int32_t>(), k, nbits, w32, reinterpret_cast<uint32_t *>(C));
        GN_CUDA_TRY(cudaMemcpyAsync(hcc.data(), dcc.p, (size_t)k * 4, cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        for (int32_t c = 0; c < k; ++c)
            if (hcc[(size_t)c] == 0)
                GN_CUDA_TRY(cudaMemcpyAsync(C + (size_t)c * row, X + pick(rng) * row, row, cudaMemcpyDeviceToDevice, st));
    }
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

}  // namespace gn
