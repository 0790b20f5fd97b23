// flat_scan.cuh — launcher interface of the exact flat scans.
#pragma once

#include "common.cuh"

namespace gn {

struct FlatScanArgs {
    int metric = M_L2;
    const void *db = nullptr;  // n rows, stride4 * 16 bytes each (zero padded)
    int64_t n = 0;
    int d = 0;                 // real dimension (floats) or bytes (Hamming)
    int stride4 = 0;           // row stride in 16-byte units
    const void *q = nullptr;   // nq rows, same layout as db
    int64_t nq = 0;
    int k = 0;
    int64_t *out_idx = nullptr;  // nq*k
    void *out_dist = nullptr;    // nq*k float32 or int64
    int *err = nullptr;          // float metrics: device error word of the scan's bounded waits
    // filled by flat_plan
    int warps = 4, qw = 8, n_slices = 1, n_groups = 1;
    int64_t slice_rows = 0;
};

constexpr int FLAT_MAX_K_WARP = 256;

void flat_plan(FlatScanArgs &a);
size_t flat_part_bytes(const FlatScanArgs &a);
int flat_smem_ok(const FlatScanArgs &a);
int flat_launch(const FlatScanArgs &a, uint64_t *part, cudaStream_t st);
int flat_preload_hamming();
int64_t next_pow2(int64_t v);
void flat_large_k_launch(const FlatScanArgs &a, int64_t q_begin, int64_t qc, uint64_t *keys, uint64_t *sorted,
                         cudaStream_t st);

}  // namespace gn
