// prober.cuh — learned probe selection (see prober.cu).
#pragma once

#include "common.cuh"

struct gn_index;

namespace gn {

constexpr int PROBER_CAND = 64;    // candidate lists per query (MLP inputs)
constexpr int PROBER_HIDDEN = 256;  // hidden width

// Device pointers of an attached prober's inference weights.
struct ProberWeights {
    const void *W1 = nullptr, *W2 = nullptr, *W3 = nullptr;  // BF16
    const float *b1 = nullptr, *b2 = nullptr, *b3 = nullptr;
};
int prober_weights(gn_index *pr, ProberWeights *w);

// Probes of nq device queries of `ivf` chosen by the prober `pr`: probes
// [nq x 64] list ids in distance order, -1 padded; nprobed[q] = count.
int prober_apply(gn_index *pr, gn_index *ivf, const float *dQ, int64_t nq, float logit_tau, int32_t *probes,
                 int32_t *nprobed, cudaStream_t st);

}  // namespace gn
