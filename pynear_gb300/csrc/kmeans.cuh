// kmeans.cuh — device k-means entry points (float and binary).
#pragma once

#include "common.cuh"

namespace gn {

// X: n rows of dp floats (dp % 16 == 0, zero padded past d), on the device.
// Outputs on the device: C (k*dp), cnorm (k), labels (n).
int kmeans_l2_device(const float *X, int64_t n, int d, int dp, int64_t k, int64_t max_iter, uint32_t seed,
                     float *C, float *cnorm, int32_t *labels, int64_t *iters_out, cudaStream_t st);

// X: n rows of w4*16 bytes (zero padded past nbytes).  C: k rows, same layout.
int kmeans_bin_device(const uint8_t *X, int64_t n, int nbytes, int w4, int32_t k, int32_t max_iter, uint32_t seed,
                      uint8_t *C, int32_t *labels, cudaStream_t st);

void row_norms(const float *X, int64_t n, int dp, float *out, cudaStream_t st);

}  // namespace gn
