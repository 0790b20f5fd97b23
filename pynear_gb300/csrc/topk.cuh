// topk.cuh — warp-level top-k selection over 64-bit (distance, index) keys.
//
// A warp keeps one sorted list of up to 32*R keys in registers: element
// p = r*32 + lane lives in register r of that lane.  Candidates that beat the
// current k-th key are inserted one at a time (warp-uniform), which costs a
// few shuffles per register; after the first few hundred rows almost every
// candidate fails the threshold test, so the steady-state cost is one 64-bit
// compare and one ballot per candidate.
#pragma once

#include "common.cuh"

namespace gn {

template <int R>
struct WarpTopK {
    uint64_t v[R];

    __device__ __forceinline__ void init() {
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = KEY_EMPTY;
    }

    // key at sorted position p (warp-uniform p), broadcast to all lanes
    __device__ __forceinline__ uint64_t at(int p) const {
        uint64_t x = v[0];
#pragma unroll
        for (int r = 1; r < R; ++r)
            if (p / 32 == r) x = v[r];
        return __shfl_sync(0xffffffffu, x, p & 31);
    }

    // insert a warp-uniform key c (must not already be present)
    __device__ __forceinline__ void insert(uint64_t c) {
        const int lane = threadIdx.x & 31;
        int pos = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) pos += __popc(__ballot_sync(0xffffffffu, v[r] < c));
        if (pos >= 32 * R) return;
#pragma unroll
        for (int r = R - 1; r >= 0; --r) {
            uint64_t up = __shfl_up_sync(0xffffffffu, v[r], 1);
            uint64_t carry = (r > 0) ? __shfl_sync(0xffffffffu, v[r > 0 ? r - 1 : 0], 31) : KEY_EMPTY;
            if (lane == 0) up = carry;
            const int p = r * 32 + lane;
            v[r] = (p > pos) ? up : (p == pos ? c : v[r]);
        }
    }

    // Offer each lane's candidate key; keys >= thresh are dropped.  thresh is
    // warp-uniform and updated in place to the new k-th key.
    __device__ __forceinline__ void offer(uint64_t cand, uint64_t &thresh, int k) {
        unsigned m = __ballot_sync(0xffffffffu, cand < thresh);
        while (m) {
            int src = __ffs(m) - 1;
            m &= m - 1;
            uint64_t c = __shfl_sync(0xffffffffu, cand, src);
            if (c < thresh) {
                insert(c);
                thresh = at(k - 1);
            }
        }
    }

    // write the first k keys to out[0..k) (sorted ascending)
    __device__ __forceinline__ void store(uint64_t *out, int k) const {
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            int p = r * 32 + lane;
            if (p < k) out[p] = v[r];
        }
    }
};

}  // namespace gn
