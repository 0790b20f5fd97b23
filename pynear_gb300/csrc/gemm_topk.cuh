// gemm_topk.cuh — FP32 CUDA-core tile GEMM with fused selection epilogues.
//
// One CTA of 256 threads multiplies a tile of BM=64 "A" rows (queries or
// points, gathered through an index list) with tiles of BN=128 "B" rows
// (centroids or database rows, contiguous) over K = dp (a multiple of 16,
// zero padded).  Thread t owns A rows 8*(t/32) .. +8 and B rows 4*(t%32) .. +4,
// so warp w owns eight whole A rows across the full B tile: a fused top-k
// epilogue can offer the warp's 32x4 scores per A row straight to that row's
// register list without staging through shared memory.
#pragma once

#include "common.cuh"

namespace gn {

constexpr int GT_BM = 64, GT_BN = 128, GT_BK = 16, GT_THREADS = 256;

struct GemmTileSmem {
    float As[2][GT_BK][GT_BM + 4];
    float Bs[2][GT_BK][GT_BN + 4];
};

// Orderable transform of a float (total order, negatives below positives).
__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float ord2f(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// Load one BK-wide slice of the A tile (rows arow[0..BM), gathered) and the B
// tile (rows b0..b0+BN) into shared buffer `buf`.  Rows past the end read 0.
__device__ __forceinline__ void gt_load(GemmTileSmem &s, int buf, const float *__restrict__ A,
                                        const int64_t *arow, int64_t lda, const float *__restrict__ B, int64_t b0,
                                        int64_t b1, int64_t ldb, int k0) {
    const int t = threadIdx.x;
    {   // A: 64 rows x 16 k = 256 float4, one per thread
        const int r = t >> 2, k4 = t & 3;
        const int64_t ar = arow[r];
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ar >= 0) v = *reinterpret_cast<const float4 *>(A + ar * lda + k0 + 4 * k4);
        s.As[buf][4 * k4 + 0][r] = v.x;
        s.As[buf][4 * k4 + 1][r] = v.y;
        s.As[buf][4 * k4 + 2][r] = v.z;
        s.As[buf][4 * k4 + 3][r] = v.w;
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // B: 128 rows x 16 k = 512 float4, two per thread
        const int idx = t + h * GT_THREADS;
        const int r = idx >> 2, k4 = idx & 3;
        const int64_t br = b0 + r;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (br < b1) v = *reinterpret_cast<const float4 *>(B + br * ldb + k0 + 4 * k4);
        s.Bs[buf][4 * k4 + 0][r] = v.x;
        s.Bs[buf][4 * k4 + 1][r] = v.y;
        s.Bs[buf][4 * k4 + 2][r] = v.z;
        s.Bs[buf][4 * k4 + 3][r] = v.w;
    }
}

// acc[i][j] = dot(A row 8*(t/32)+i, B row b0 + 4*(t%32)+j) over K = dp.
// arow must be visible to all threads (shared memory) before the call.
__device__ __forceinline__ void gt_tile(GemmTileSmem &s, float (&acc)[8][4], const float *__restrict__ A,
                                        const int64_t *arow, int64_t lda, const float *__restrict__ B, int64_t b0,
                                        int64_t b1, int64_t ldb, int dp) {
    const int t = threadIdx.x;
    const int tm = t >> 5, tn = t & 31;
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    const int nk = dp / GT_BK;
    gt_load(s, 0, A, arow, lda, B, b0, b1, ldb, 0);
    __syncthreads();
    for (int kc = 0; kc < nk; ++kc) {
        const int cur = kc & 1;
        if (kc + 1 < nk) gt_load(s, cur ^ 1, A, arow, lda, B, b0, b1, ldb, (kc + 1) * GT_BK);
#pragma unroll
        for (int kk = 0; kk < GT_BK; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4 *>(&s.As[cur][kk][tm * 8]);
            const float4 a1 = *reinterpret_cast<const float4 *>(&s.As[cur][kk][tm * 8 + 4]);
            const float4 b = *reinterpret_cast<const float4 *>(&s.Bs[cur][kk][tn * 4]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
}

}  // namespace gn
