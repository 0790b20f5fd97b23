// tc_ivf.cuh — launcher of the tensor-core IVF list scan (see tc_ivf.cu).
#pragma once

#include "tc_scan.cuh"

namespace gn {

struct TcIvfLaunch {
    const void *X = nullptr;  // BF16 rows [x_rows x K] (x_rows >= 128), plain or (tiled) as IvfL2State::x16
    int tiled = 0;            // X in the tiled layout: units address it by TcUnit::xrow
    int64_t x_rows = 0;
    const void *Q = nullptr;  // BF16 query rows in bucket order [q_rows x K] (q_rows >= 256)
    int64_t q_rows = 0;
    int K = 0;                // multiple of 64
    const TcUnit *units = nullptr;  // a0/na: query rows, r0/r1: list rows, rbase: list start
    const int64_t *n_units = nullptr;
    const float *xnorm = nullptr;   // |x|^2 of the list rows
    const int64_t *aslot = nullptr; // per query row: segment base of its (query, probe) pair, in seg_mul units
    int seg_mul = 1;                // 128 for the list scan: segments are 128-row slots
    float *scores = nullptr;
    uint32_t *tmin4 = nullptr;      // optional: per (slot, 32-row quarter) minimum ordered score
    // with tmin4: per query row, the ordered score bound of its query; a
    // quarter's scores are stored only when its minimum is not above it
    const uint32_t *abound = nullptr;
    int *err = nullptr;
    unsigned long long *next_unit = nullptr;  // device counter of the dynamic unit schedule (reset per launch)
    long long wait_limit = 0;       // cycles a pipeline wait may take (0: the default, about 2 s)
    int drill = 0;                  // failure drill: the producer issues no copies, so the waits run out
    int grid = 0;
};

int tc_ivf_launch(const TcIvfLaunch &a, cudaStream_t st);

}  // namespace gn
