// distance.cuh — device distance arithmetic in the reference's exact order.
//
// The float metrics reproduce PyNear's x86 AVX2 kernels bit for bit
// (pynear/include/DistanceFunctions.hpp):
//   L2   (dist_l2_f_avx2, :304-345): eight FMA lane accumulators over blocks of
//        eight; fold lanes j and j+4; a 4-wide FMA tail; a masked FMA remainder;
//        ((s0+s1)+(s2+s3)); correctly rounded sqrt.
//   L1   (dist_l1_f_avx2, :347-382): eight lane sums of |q-x|, lanes summed 0..7
//        in order, scalar remainder appended in order.
//   Linf (dist_chebyshev_f_avx2, :384-420): running max of |q-x| (exact).
// Every operation uses an explicit _rn intrinsic so nvcc cannot contract or
// reorder it.  Rows and queries are zero-padded to a multiple of four floats;
// padded lanes contribute exactly 0 to each accumulation above.
#pragma once

#include "common.cuh"

namespace gn {

// Per-pair accumulator state for the float metrics.
template <int METRIC>
struct FAcc {
    float a[8];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = 0.f;
    }
    // one block of eight coordinates: lane i gets q[i]-x[i]
    __device__ __forceinline__ void block8(const float4 &q0, const float4 &q1, const float4 &x0, const float4 &x1) {
        float t[8] = {__fsub_rn(q0.x, x0.x), __fsub_rn(q0.y, x0.y), __fsub_rn(q0.z, x0.z), __fsub_rn(q0.w, x0.w),
                      __fsub_rn(q1.x, x1.x), __fsub_rn(q1.y, x1.y), __fsub_rn(q1.z, x1.z), __fsub_rn(q1.w, x1.w)};
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            if (METRIC == M_L2) a[i] = __fmaf_rn(t[i], t[i], a[i]);
            else if (METRIC == M_L1) a[i] = __fadd_rn(a[i], fabsf(t[i]));
            else a[i] = fmaxf(a[i], fabsf(t[i]));
        }
    }
    // Finish after the blocks of eight.  rem = d % 8 (0..7); tail = the float4
    // pair that holds coordinates [d - rem, d - rem + 8) (zero beyond d).
    __device__ __forceinline__ float finish(int rem, const float4 &q0, const float4 &q1, const float4 &x0,
                                            const float4 &x1) const {
        if (METRIC == M_L2) {
            float s0 = __fadd_rn(a[4], a[0]), s1 = __fadd_rn(a[5], a[1]);
            float s2 = __fadd_rn(a[6], a[2]), s3 = __fadd_rn(a[7], a[3]);
            if (rem > 0) {
                // first four tail coordinates: the 4-wide FMA step when rem >= 4,
                // otherwise the masked remainder (padding makes masking implicit)
                float t0 = __fsub_rn(q0.x, x0.x), t1 = __fsub_rn(q0.y, x0.y);
                float t2 = __fsub_rn(q0.z, x0.z), t3 = __fsub_rn(q0.w, x0.w);
                s0 = __fmaf_rn(t0, t0, s0); s1 = __fmaf_rn(t1, t1, s1);
                s2 = __fmaf_rn(t2, t2, s2); s3 = __fmaf_rn(t3, t3, s3);
                if (rem > 4) {
                    float u0 = __fsub_rn(q1.x, x1.x), u1 = __fsub_rn(q1.y, x1.y);
                    float u2 = __fsub_rn(q1.z, x1.z), u3 = __fsub_rn(q1.w, x1.w);
                    s0 = __fmaf_rn(u0, u0, s0); s1 = __fmaf_rn(u1, u1, s1);
                    s2 = __fmaf_rn(u2, u2, s2); s3 = __fmaf_rn(u3, u3, s3);
                }
            }
            return __fsqrt_rn(__fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3)));
        } else if (METRIC == M_L1) {
            float tot = 0.f;
#pragma unroll
            for (int i = 0; i < 8; ++i) tot = __fadd_rn(tot, a[i]);
            if (rem > 0) {
                float t[8] = {__fsub_rn(q0.x, x0.x), __fsub_rn(q0.y, x0.y), __fsub_rn(q0.z, x0.z),
                              __fsub_rn(q0.w, x0.w), __fsub_rn(q1.x, x1.x), __fsub_rn(q1.y, x1.y),
                              __fsub_rn(q1.z, x1.z), __fsub_rn(q1.w, x1.w)};
#pragma unroll
                for (int i = 0; i < 7; ++i)
                    if (i < rem) tot = __fadd_rn(tot, fabsf(t[i]));
            }
            return tot;
        } else {
            float m = 0.f;
#pragma unroll
            for (int i = 0; i < 8; ++i) m = fmaxf(m, a[i]);
            if (rem > 0) {
                m = fmaxf(m, fmaxf(fmaxf(fabsf(__fsub_rn(q0.x, x0.x)), fabsf(__fsub_rn(q0.y, x0.y))),
                                   fmaxf(fabsf(__fsub_rn(q0.z, x0.z)), fabsf(__fsub_rn(q0.w, x0.w)))));
                m = fmaxf(m, fmaxf(fmaxf(fabsf(__fsub_rn(q1.x, x1.x)), fabsf(__fsub_rn(q1.y, x1.y))),
                                   fmaxf(fabsf(__fsub_rn(q1.z, x1.z)), fabsf(__fsub_rn(q1.w, x1.w)))));
            }
            return m;
        }
    }
};

// Full distance between two padded rows (dp floats, dp % 4 == 0), d real dims.
template <int METRIC>
__device__ __forceinline__ float fdist(const float *__restrict__ q, const float *__restrict__ x, int d) {
    FAcc<METRIC> acc;
    acc.zero();
    const float4 *q4 = reinterpret_cast<const float4 *>(q);
    const float4 *x4 = reinterpret_cast<const float4 *>(x);
    const int nb = d >> 3, rem = d & 7;
    for (int c = 0; c < nb; ++c) acc.block8(q4[2 * c], q4[2 * c + 1], x4[2 * c], x4[2 * c + 1]);
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 q0 = z, q1 = z, x0 = z, x1 = z;
    if (rem > 0) { q0 = q4[2 * nb]; x0 = x4[2 * nb]; }
    if (rem > 4) { q1 = q4[2 * nb + 1]; x1 = x4[2 * nb + 1]; }
    return acc.finish(rem, q0, q1, x0, x1);
}

__device__ __forceinline__ uint32_t popc4(const uint4 &a, const uint4 &b) {
    return __popc(a.x ^ b.x) + __popc(a.y ^ b.y) + __popc(a.z ^ b.z) + __popc(a.w ^ b.w);
}

// Hamming distance between two rows of w4 uint4 words (zero-padded).
__device__ __forceinline__ uint32_t hdist(const uint4 *__restrict__ q, const uint4 *__restrict__ x, int w4) {
    uint32_t s = 0;
    for (int c = 0; c < w4; ++c) s += popc4(q[c], x[c]);
    return s;
}

__device__ __forceinline__ uint4 ldg_nc_u4(const uint4 *p) {
    uint4 r;
    asm volatile("ld.global.nc.v4.u32 {%0,%1,%2,%3}, [%4];" : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
    return r;
}
__device__ __forceinline__ float4 ldg_nc_f4(const float4 *p) {
    float4 r;
    asm volatile("ld.global.nc.v4.f32 {%0,%1,%2,%3}, [%4];" : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
    return r;
}

}  // namespace gn
