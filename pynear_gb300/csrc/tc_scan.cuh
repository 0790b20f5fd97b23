// tc_scan.cuh — launcher interface of the tensor-core candidate stage.
#pragma once

#include "common.cuh"

namespace gn {

// One work unit: A rows [a0, a0 + na) against B rows [r0, r1).  Query row
// a0 + i writes its S best keys to partial slot arow_slot[a0 + i] + rch.
struct TcUnit {
    int64_t a0;
    int64_t r0;
    int64_t r1;
    int64_t rbase;  // store mode: first B row of the list the unit belongs to
    int64_t xrow;   // IVF list scan, tiled row layout: the padded row of r0 (a multiple of 128)
    int32_t na;
    int32_t rch;
};

struct TcLaunch {
    const void *A = nullptr;  // BF16 (or FP8) [a_rows x K], K-major
    int64_t a_rows = 0;
    const void *B = nullptr;  // BF16 (or FP8) [b_rows x K], K-major
    int64_t b_rows = 0;
    int K = 0;                // elements: multiple of 64 (BF16) or 128 (FP8)
    const TcUnit *units = nullptr;
    const int64_t *n_units = nullptr;  // device scalar
    const int64_t *cta_off = nullptr;  // optional [grid+1] unit range per CTA (else strided)
    const float *bnorm = nullptr;      // |B row|^2, FP32
    const int64_t *arow_slot = nullptr;
    uint64_t *part = nullptr;          // slots x S keys
    uint32_t *qbound = nullptr;        // optional, per A row: bound of its S-th best score (ordered key;
                                       // all ones = none), read at each unit's start, lowered at its end
    int *err = nullptr;                // device error word (0 = ok)
    int S = 40;
    int grid = 0;
    // store mode (S == 0): write every score instead of keeping the top S;
    // query row a0 + i stores column c at scores[arow_slot[a0 + i] + c - rbase]
    float *scores = nullptr;
    // FP8 E4M3 operands (K a multiple of 128) with one FP32 scale per row
    int fp8 = 0;
    const float *ascale = nullptr;
    const float *bscale = nullptr;
};

int tc_topk_launch(const TcLaunch &a, cudaStream_t st);
void to_bf16_rows(const float *X, int64_t n, int d, int ldx, void *out, int K, cudaStream_t st);
void to_e4m3_rows(const float *X, int64_t n, int d, int ldx, void *out, float *scale, int K, cudaStream_t st);
int tc_rerank_launch(const uint64_t *part, int nslot, int S, const float *Q, const float *X, int d, int dp,
                     const int32_t *ids, int64_t nq, int k, int sqrt_out, int64_t *out_idx, float *out_dist,
                     cudaStream_t st);

}  // namespace gn
