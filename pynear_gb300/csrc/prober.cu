// prober.cu — learned probe selection for the float IVF index.
//
// A small MLP looks at a query's 64 nearest centroids (ids c_i and squared
// distances d_i, nearest first) and predicts, for each of those 64 lists, the
// probability that it holds one of the query's exact 10 nearest neighbours:
//   f_i   = max(0, 1 - (d_i - d_1) / d_1)               relative-gap feature
//   h1    = ReLU(b1 + sum_i f_i * W1[c_i])               64 active rows of W1 [L x 256]
//   h2    = ReLU(W2 h1 + b2)                             W2 [256 x 256]
//   z_i   = W3[c_i] . h2 + b3[c_i]                        logits of the 64 candidates, W3 [L x 256]
// The index probes the candidates with sigmoid(z_i) >= tau (always the
// nearest), in distance order.  Training minimises the mean binary
// cross-entropy against labels y_i = [list c_i holds a true neighbour], with
// labels made by exact GPU search; forward, backward (scatter-adds for the
// gathered rows, a tiled GEMM for dW2) and Adam are kernels of this file.
// Inference uses BF16 copies of the weights with FP32 accumulation and is fused
// with the merge of the coarse top-64 (one kernel per batch).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "gemm_topk.cuh"
#include "index.cuh"
#include "ivf.cuh"
#include "prober.cuh"
#include "topk.cuh"

namespace gn {

constexpr int PB_C = PROBER_CAND, PB_H = PROBER_HIDDEN;

struct ProberState {
    int L = 0;                // lists (W1 / W3 rows)
    uint32_t seed = 1;
    size_t n_params = 0;
    DBuf params, grads, m1, m2;  // FP32 master weights, gradients, Adam moments
    DBuf wbf;                    // BF16 copies for inference: W1 | W2 | W3
    int64_t step = 0;
    bool trained = false;
    // training scratch
    DBuf cand, feat, lab, h1p, h2p, dlog, dh2, loss;
    // offsets into the flat parameter array
    size_t oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
    void layout() {
        oW1 = 0;
        ob1 = oW1 + (size_t)L * PB_H;
        oW2 = ob1 + PB_H;
        ob2 = oW2 + (size_t)PB_H * PB_H;
        oW3 = ob2 + PB_H;
        ob3 = oW3 + (size_t)L * PB_H;
        n_params = ob3 + L;
    }
};

// ── forward (training; keeps the pre-activations) ─────────────────────────
// block per query, 256 threads (= PB_H)
__global__ void __launch_bounds__(PB_H) mlp_fwd_kernel(const float *__restrict__ P, int L, size_t oW1, size_t ob1,
                                                        size_t oW2, size_t ob2, size_t oW3, size_t ob3,
                                                        const int32_t *__restrict__ cand,
                                                        const float *__restrict__ feat,
                                                        const float *__restrict__ lab, int64_t B,
                                                        float *__restrict__ h1p, float *__restrict__ h2p,
                                                        float *__restrict__ dlog, float *__restrict__ loss,
                                                        float inv_norm) {
    __shared__ float sh1[PB_H], sh2[PB_H];
    __shared__ int32_t sc[PB_C];
    __shared__ float sf[PB_C];
    const int64_t b = blockIdx.x;
    const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
    if (j < PB_C) {
        sc[j] = cand[b * PB_C + j];
        sf[j] = feat[b * PB_C + j];
    }
    __syncthreads();
    float a = P[ob1 + j];
    for (int i = 0; i < PB_C; ++i)
        if (sc[i] >= 0) a = fmaf(sf[i], P[oW1 + (size_t)sc[i] * PB_H + j], a);
    h1p[b * PB_H + j] = a;
    sh1[j] = fmaxf(a, 0.f);
    __syncthreads();
    // h2: warp w computes outputs w*32 .. w*32+31, lanes stride the inputs
    for (int o = warp * 32; o < warp * 32 + 32; ++o) {
        const float *w2 = P + oW2 + (size_t)o * PB_H;
        float s = 0.f;
#pragma unroll
        for (int k = lane; k < PB_H; k += 32) s = fmaf(w2[k], sh1[k], s);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) {
            const float v = s + P[ob2 + o];
            h2p[b * PB_H + o] = v;
            sh2[o] = fmaxf(v, 0.f);
        }
    }
    __syncthreads();
    // logits of the candidates: warp w takes candidates w, w+8, ...
    float lsum = 0.f;
    for (int i = warp; i < PB_C; i += PB_H / 32) {
        const int c = sc[i];
        if (c < 0) {
            if (lane == 0) dlog[b * PB_C + i] = 0.f;
            continue;
        }
        const float *w3 = P + oW3 + (size_t)c * PB_H;
        float s = 0.f;
#pragma unroll
        for (int k = lane; k < PB_H; k += 32) s = fmaf(w3[k], sh2[k], s);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) {
            const float z = s + P[ob3 + c];
            const float y = lab[b * PB_C + i];
            const float p = 1.f / (1.f + expf(-z));
            dlog[b * PB_C + i] = (p - y) * inv_norm;
            // log(1 + e^-|z|) + max(z, 0) - y z : numerically stable BCE
            lsum += (fmaxf(z, 0.f) - y * z + log1pf(expf(-fabsf(z)))) * inv_norm;
        }
    }
    if (lane == 0 && lsum != 0.f) atomicAdd(loss, lsum);
}

// ── backward: W3/b3 scatter, dh2, dh1, W1/b1 scatter, b2 ──────────────────
__global__ void __launch_bounds__(PB_H) mlp_bwd_kernel(const float *__restrict__ P, float *__restrict__ G, int L,
                                                        size_t oW1, size_t ob1, size_t oW2, size_t ob2, size_t oW3,
                                                        size_t ob3, const int32_t *__restrict__ cand,
                                                        const float *__restrict__ feat, int64_t B,
                                                        const float *__restrict__ h1p, const float *__restrict__ h2p,
                                                        const float *__restrict__ dlog, float *__restrict__ dh2out) {
    __shared__ float sd2[PB_H], sdl[PB_C];
    __shared__ int32_t sc[PB_C];
    __shared__ float sf[PB_C];
    const int64_t b = blockIdx.x;
    const int j = threadIdx.x;
    if (j < PB_C) {
        sc[j] = cand[b * PB_C + j];
        sf[j] = feat[b * PB_C + j];
        sdl[j] = dlog[b * PB_C + j];
    }
    __syncthreads();
    const float h2 = fmaxf(h2p[b * PB_H + j], 0.f);
    float d2 = 0.f;
    for (int i = 0; i < PB_C; ++i) {
        const int c = sc[i];
        if (c < 0) continue;
        d2 = fmaf(sdl[i], P[oW3 + (size_t)c * PB_H + j], d2);
        atomicAdd(G + oW3 + (size_t)c * PB_H + j, sdl[i] * h2);
        if (j == 0) atomicAdd(G + ob3 + c, sdl[i]);
    }
    d2 = h2p[b * PB_H + j] > 0.f ? d2 : 0.f;
    sd2[j] = d2;
    dh2out[b * PB_H + j] = d2;
    atomicAdd(G + ob2 + j, d2);
    __syncthreads();
    // dh1[m] = sum_o W2[o][m] * dh2[o]   (thread m, coalesced over m)
    float d1 = 0.f;
    for (int o = 0; o < PB_H; ++o) d1 = fmaf(P[oW2 + (size_t)o * PB_H + j], sd2[o], d1);
    d1 = h1p[b * PB_H + j] > 0.f ? d1 : 0.f;
    atomicAdd(G + ob1 + j, d1);
    for (int i = 0; i < PB_C; ++i)
        if (sc[i] >= 0) atomicAdd(G + oW1 + (size_t)sc[i] * PB_H + j, sf[i] * d1);
}

// dW2[o][m] = sum_b dh2[b][o] * relu(h1p[b][m]) — 16x16 tiles over the batch
__global__ void mlp_dw2_kernel(const float *__restrict__ dh2, const float *__restrict__ h1p, int64_t B,
                               float *__restrict__ G, size_t oW2) {
    __shared__ float sa[16][17], sb[16][17];
    const int o = blockIdx.y * 16 + threadIdx.y, m = blockIdx.x * 16 + threadIdx.x;
    float acc = 0.f;
    for (int64_t b0 = 0; b0 < B; b0 += 16) {
        const int64_t ba = b0 + threadIdx.x, bb = b0 + threadIdx.y;
        sa[threadIdx.y][threadIdx.x] = ba < B ? dh2[ba * PB_H + blockIdx.y * 16 + threadIdx.y] : 0.f;
        sb[threadIdx.y][threadIdx.x] = bb < B ? fmaxf(h1p[bb * PB_H + blockIdx.x * 16 + threadIdx.x], 0.f) : 0.f;
        __syncthreads();
#pragma unroll
        for (int t = 0; t < 16; ++t) acc = fmaf(sa[threadIdx.y][t], sb[t][threadIdx.x], acc);
        __syncthreads();
    }
    G[oW2 + (size_t)o * PB_H + m] += acc;
}

__global__ void adam_kernel(float *__restrict__ P, const float *__restrict__ G, float *__restrict__ m1,
                            float *__restrict__ m2, size_t n, float lr, float b1, float b2, float eps, float c1,
                            float c2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float a = b1 * m1[i] + (1.f - b1) * g;
    const float v = b2 * m2[i] + (1.f - b2) * g * g;
    m1[i] = a;
    m2[i] = v;
    P[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

__global__ void to_bf16_kernel(const float *__restrict__ x, size_t n, __nv_bfloat16 *__restrict__ y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// ── features and labels from coarse keys ──────────────────────────────────
__device__ __forceinline__ float gap_feature(float d, float d1) {
    return fmaxf(0.f, 1.f - (d - d1) / fmaxf(d1, 1e-12f));
}

// keys: [nq x PB_C] sorted coarse keys (squared distance bits, list id)
__global__ void prober_features_kernel(const uint64_t *__restrict__ keys, int64_t nq, int32_t *__restrict__ cand,
                                       float *__restrict__ feat) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq * PB_C) return;
    const int64_t q = t / PB_C;
    const uint64_t k0 = keys[q * PB_C], k = keys[t];
    const bool e = k == KEY_EMPTY;
    cand[t] = e ? -1 : (int32_t)key_idx(k);
    feat[t] = e ? 0.f : gap_feature(__uint_as_float(key_dist(k)), __uint_as_float(key_dist(k0)));
}

// y[q][i] = 1 if list cand[q][i] holds one of the query's exact k neighbours
__global__ void prober_labels_kernel(const int32_t *__restrict__ cand, const int64_t *__restrict__ gt, int k,
                                     const int32_t *__restrict__ list_of, int64_t nq, float *__restrict__ lab) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nq * PB_C) return;
    const int64_t q = t / PB_C;
    const int32_t c = cand[t];
    float y = 0.f;
    if (c >= 0)
        for (int j = 0; j < k; ++j) {
            const int64_t r = gt[q * k + j];
            if (r >= 0 && list_of[r] == c) { y = 1.f; break; }
        }
    lab[t] = y;
}

// ── inference, fused with the merge of the coarse top-64 ──────────────────
// block per query, 256 threads.  part: nsplit sorted partial lists of PB_C
// coarse keys per query.  Writes probes[q][0..PB_C): selected list ids in
// distance order, then -1.
__global__ void __launch_bounds__(PB_H) prober_select_kernel(const uint64_t *__restrict__ part, int nsplit, int64_t nq,
                                                              const __nv_bfloat16 *__restrict__ W1,
                                                              const float *__restrict__ b1,
                                                              const __nv_bfloat16 *__restrict__ W2,
                                                              const float *__restrict__ b2,
                                                              const __nv_bfloat16 *__restrict__ W3,
                                                              const float *__restrict__ b3, float logit_tau,
                                                              int32_t *__restrict__ probes,
                                                              int32_t *__restrict__ nprobed) {
    __shared__ float sh1[PB_H], sh2[PB_H], sf[PB_C], sz[PB_C];
    __shared__ int32_t sc[PB_C];
    const int64_t q = blockIdx.x;
    const int j = threadIdx.x, lane = j & 31, warp = j >> 5;
    if (warp == 0) {
        WarpTopK<PB_C / 32> L;
        L.init();
        uint64_t thr = KEY_EMPTY;
        for (int sp = 0; sp < nsplit; ++sp)
            for (int i0 = 0; i0 < PB_C; i0 += 32)
                L.offer(part[((size_t)q * nsplit + sp) * PB_C + i0 + lane], thr, PB_C);
        const float d1 = __uint_as_float(key_dist(L.at(0)));
#pragma unroll
        for (int r = 0; r < PB_C / 32; ++r) {
            const uint64_t k = L.v[r];
            const bool e = k == KEY_EMPTY;
            sc[r * 32 + lane] = e ? -1 : (int32_t)key_idx(k);
            sf[r * 32 + lane] = e ? 0.f : gap_feature(__uint_as_float(key_dist(k)), d1);
        }
    }
    __syncthreads();
    float a = b1[j];
    for (int i = 0; i < PB_C; ++i)
        if (sc[i] >= 0) a = fmaf(sf[i], __bfloat162float(W1[(size_t)sc[i] * PB_H + j]), a);
    sh1[j] = fmaxf(a, 0.f);
    __syncthreads();
    for (int o = warp * 32; o < warp * 32 + 32; ++o) {
        const __nv_bfloat16 *w2 = W2 + (size_t)o * PB_H;
        float s = 0.f;
#pragma unroll
        for (int k = lane; k < PB_H; k += 32) s = fmaf(__bfloat162float(w2[k]), sh1[k], s);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) sh2[o] = fmaxf(s + b2[o], 0.f);
    }
    __syncthreads();
    for (int i = warp; i < PB_C; i += PB_H / 32) {
        const int c = sc[i];
        float s = 0.f;
        if (c >= 0) {
            const __nv_bfloat16 *w3 = W3 + (size_t)c * PB_H;
#pragma unroll
            for (int k = lane; k < PB_H; k += 32) s = fmaf(__bfloat162float(w3[k]), sh2[k], s);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        }
        if (lane == 0) sz[i] = c >= 0 ? s + b3[c] : -INFINITY;
    }
    __shared__ int s_cnt0;
    __syncthreads();
    bool keep = false;
    unsigned m = 0;
    const int i = warp * 32 + lane;
    if (warp < PB_C / 32) {
        keep = sc[i] >= 0 && (i == 0 || sz[i] >= logit_tau);
        m = __ballot_sync(0xffffffffu, keep);
        if (warp == 0 && lane == 0) s_cnt0 = __popc(m);
    }
    __syncthreads();
    if (warp < PB_C / 32) {
        // compaction in distance order: warp 0's survivors first, then warp 1's
        const int base = (warp == 0) ? 0 : s_cnt0;
        const int pos = base + __popc(m & ((1u << lane) - 1u));
        if (keep) probes[q * PB_C + pos] = sc[i];
        if (warp == 1) {
            const int total = s_cnt0 + __popc(m);
            for (int t = total + lane; t < PB_C; t += 32) probes[q * PB_C + t] = -1;
            if (lane == 0 && nprobed) nprobed[q] = total;
        }
    }
}

// ── host ──────────────────────────────────────────────────────────────────
static ProberState *pst(gn_index *ix) { return reinterpret_cast<ProberState *>(ix->ext); }

static int prober_init(ProberState &S, cudaStream_t st) {
    S.layout();
    GN_TRY(S.params.ensure(S.n_params * 4));
    GN_TRY(S.grads.ensure(S.n_params * 4));
    GN_TRY(S.m1.ensure(S.n_params * 4));
    GN_TRY(S.m2.ensure(S.n_params * 4));
    GN_TRY(S.wbf.ensure(S.n_params * 2));
    std::vector<float> h(S.n_params, 0.f);
    std::mt19937 rng(S.seed);
    auto fill = [&](size_t off, size_t n, float bound) {
        std::uniform_real_distribution<float> u(-bound, bound);
        for (size_t i = 0; i < n; ++i) h[off + i] = u(rng);
    };
    fill(S.oW1, (size_t)S.L * PB_H, 1.0f / std::sqrt((float)PB_C));
    fill(S.oW2, (size_t)PB_H * PB_H, 1.0f / std::sqrt((float)PB_H));
    fill(S.oW3, (size_t)S.L * PB_H, 1.0f / std::sqrt((float)PB_H));
    GN_CUDA_TRY(cudaMemcpyAsync(S.params.p, h.data(), S.n_params * 4, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemsetAsync(S.m1.p, 0, S.n_params * 4, st));
    GN_CUDA_TRY(cudaMemsetAsync(S.m2.p, 0, S.n_params * 4, st));
    S.step = 0;
    return GN_OK;
}

static int prober_refresh_bf16(ProberState &S, cudaStream_t st) {
    to_bf16_kernel<<<(unsigned)ceil_div((int64_t)S.n_params, 256), 256, 0, st>>>(S.params.as<float>(), S.n_params,
                                                                                S.wbf.as<__nv_bfloat16>());
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

// One forward + backward over B examples already on the device (cand, feat,
// lab); accumulates into zeroed gradients; returns the loss on the host.
static int prober_fwd_bwd(ProberState &S, int64_t B, const int32_t *cand, const float *feat, const float *lab,
                          float *loss_host, cudaStream_t st) {
    GN_TRY(S.h1p.ensure((size_t)B * PB_H * 4));
    GN_TRY(S.h2p.ensure((size_t)B * PB_H * 4));
    GN_TRY(S.dh2.ensure((size_t)B * PB_H * 4));
    GN_TRY(S.dlog.ensure((size_t)B * PB_C * 4));
    GN_TRY(S.loss.ensure(4));
    GN_CUDA_TRY(cudaMemsetAsync(S.grads.p, 0, S.n_params * 4, st));
    GN_CUDA_TRY(cudaMemsetAsync(S.loss.p, 0, 4, st));
    const float inv = 1.f / (float)(B * PB_C);
    float *P = S.params.as<float>();
    mlp_fwd_kernel<<<(unsigned)B, PB_H, 0, st>>>(P, S.L, S.oW1, S.ob1, S.oW2, S.ob2, S.oW3, S.ob3, cand, feat, lab, B,
                                                 S.h1p.as<float>(), S.h2p.as<float>(), S.dlog.as<float>(),
                                                 S.loss.as<float>(), inv);
    mlp_bwd_kernel<<<(unsigned)B, PB_H, 0, st>>>(P, S.grads.as<float>(), S.L, S.oW1, S.ob1, S.oW2, S.ob2, S.oW3,
                                                 S.ob3, cand, feat, B, S.h1p.as<float>(), S.h2p.as<float>(),
                                                 S.dlog.as<float>(), S.dh2.as<float>());
    mlp_dw2_kernel<<<dim3(PB_H / 16, PB_H / 16), dim3(16, 16), 0, st>>>(S.dh2.as<float>(), S.h1p.as<float>(), B,
                                                                       S.grads.as<float>(), S.oW2);
    if (loss_host) {
        GN_CUDA_TRY(cudaMemcpyAsync(loss_host, S.loss.p, 4, cudaMemcpyDeviceToHost, st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
    }
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

static void prober_adam(ProberState &S, float lr, cudaStream_t st) {
    ++S.step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)S.step), c2 = 1.f - std::pow(b2, (float)S.step);
    adam_kernel<<<(unsigned)ceil_div((int64_t)S.n_params, 256), 256, 0, st>>>(
        S.params.as<float>(), S.grads.as<float>(), S.m1.as<float>(), S.m2.as<float>(), S.n_params, lr, b1, b2, 1e-8f,
        c1, c2);
}

int prober_apply(gn_index *pr, gn_index *ivf, const float *dQ, int64_t nq, float logit_tau, int32_t *probes,
                 int32_t *nprobed, cudaStream_t st) {
    ProberState &P = *pst(pr);
    IvfL2State &V = *ivf->ivfl2;
    IvfScratch &T = V.s;
    int nsplit = 0;
    GN_TRY(ivfl2_coarse_run(ivf, dQ, nq, PB_C, true, &nsplit, st));  // T.cpart: nsplit sorted lists per query
    const __nv_bfloat16 *w = P.wbf.as<__nv_bfloat16>();
    const float *pf = P.params.as<float>();
    prober_select_kernel<<<(unsigned)nq, PB_H, 0, st>>>(T.cpart.as<uint64_t>(), nsplit, nq, w + P.oW1, pf + P.ob1,
                                                       w + P.oW2, pf + P.ob2, w + P.oW3, pf + P.ob3, logit_tau,
                                                       probes, nprobed);
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

int prober_weights(gn_index *pr, ProberWeights *w) {
    if (!pr || pr->kind != K_PROBER) return fail(GN_ERR_INVALID, "not a prober");
    ProberState &P = *pst(pr);
    const __nv_bfloat16 *wb = P.wbf.as<__nv_bfloat16>();
    const float *pf = P.params.as<float>();
    w->W1 = wb + P.oW1;
    w->W2 = wb + P.oW2;
    w->W3 = wb + P.oW3;
    w->b1 = pf + P.ob1;
    w->b2 = pf + P.ob2;
    w->b3 = pf + P.ob3;
    return GN_OK;
}

}  // namespace gn

using namespace gn;

extern "C" {

int gn_prober_create(int32_t nlist, uint32_t seed, gn_index **out) {
    if (!out) return fail(GN_ERR_INVALID, "out is NULL");
    if (nlist < PB_C) return fail(GN_ERR_INVALID, "the prober needs at least 64 lists");
    gn_index *ix = new gn_index();
    ix->kind = K_PROBER;
    ProberState *S = new ProberState();
    S->L = nlist;
    S->seed = seed;
    ix->ext = S;
    ix->ext_free = [](void *p) { delete reinterpret_cast<ProberState *>(p); };
    int st = make_stream(ix);
    if (st == GN_OK) st = prober_init(*S, ix->stream);
    if (st == GN_OK) st = prober_refresh_bf16(*S, ix->stream);
    if (st == GN_OK && cudaStreamSynchronize(ix->stream) != cudaSuccess) st = fail(GN_ERR_CUDA, "prober init failed");
    if (st != GN_OK) {
        delete ix;
        return st;
    }
    *out = ix;
    return GN_OK;
}

int gn_prober_num_params(gn_index *pr, int64_t *n) {
    if (!pr || pr->kind != K_PROBER) return fail(GN_ERR_INVALID, "not a prober");
    *n = (int64_t)pst(pr)->n_params;
    return GN_OK;
}

int gn_prober_get_params(gn_index *pr, float *out) {
    if (!pr || pr->kind != K_PROBER) return fail(GN_ERR_INVALID, "not a prober");
    ProberState &S = *pst(pr);
    GN_CUDA_TRY(cudaMemcpy(out, S.params.p, S.n_params * 4, cudaMemcpyDeviceToHost));
    return GN_OK;
}

int gn_prober_set_params(gn_index *pr, const float *in) {
    if (!pr || pr->kind != K_PROBER) return fail(GN_ERR_INVALID, "not a prober");
    ProberState &S = *pst(pr);
    GN_CUDA_TRY(cudaMemcpy(S.params.p, in, S.n_params * 4, cudaMemcpyHostToDevice));
    GN_TRY(prober_refresh_bf16(S, pr->stream));
    GN_CUDA_TRY(cudaStreamSynchronize(pr->stream));
    S.trained = true;
    return GN_OK;
}

// Loss and gradients for B explicit examples (host arrays): cand [B x 64]
// list ids (-1 = none), feat [B x 64], lab [B x 64] in {0, 1}.  grads_out gets
// the gradient of the mean BCE in the flat parameter layout.
int gn_prober_loss_grad(gn_index *pr, int64_t B, const int32_t *cand, const float *feat, const float *lab,
                        float *loss_out, float *grads_out) {
    if (!pr || pr->kind != K_PROBER) return fail(GN_ERR_INVALID, "not a prober");
    if (B <= 0) return fail(GN_ERR_INVALID, "B must be positive");
    ProberState &S = *pst(pr);
    std::lock_guard<std::mutex> lk(pr->mu);
    cudaStream_t st = pr->stream;
    GN_TRY(S.cand.ensure((size_t)B * PB_C * 4));
    GN_TRY(S.feat.ensure((size_t)B * PB_C * 4));
    GN_TRY(S.lab.ensure((size_t)B * PB_C * 4));
    GN_CUDA_TRY(cudaMemcpyAsync(S.cand.p, cand, (size_t)B * PB_C * 4, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.feat.p, feat, (size_t)B * PB_C * 4, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.lab.p, lab, (size_t)B * PB_C * 4, cudaMemcpyHostToDevice, st));
    float loss = 0.f;
    GN_TRY(prober_fwd_bwd(S, B, S.cand.as<int32_t>(), S.feat.as<float>(), S.lab.as<float>(), &loss, st));
    if (loss_out) *loss_out = loss;
    if (grads_out) GN_CUDA_TRY(cudaMemcpy(grads_out, S.grads.p, S.n_params * 4, cudaMemcpyDeviceToHost));
    return GN_OK;
}

// Train on nq queries (host, d floats each) against a built IVF index; gt:
// host [nq x k] exact neighbour ids.  Mini-batches of `batch`, `epochs` passes,
// Adam with learning rate lr.  loss_out[e] = mean loss of epoch e.
int gn_prober_train(gn_index *pr, gn_index *ivf, const float *queries, int64_t nq, const int64_t *gt, int32_t k,
                    int32_t epochs, int32_t batch, float lr, float *loss_out) {
    if (!pr || pr->kind != K_PROBER) return fail(GN_ERR_INVALID, "not a prober");
    if (!ivf || ivf->kind != K_IVFL2 || !ivf->ivfl2 || ivf->ivfl2->nc == 0)
        return fail(GN_ERR_INVALID, "a built IVFFlatL2 index is required");
    ProberState &S = *pst(pr);
    IvfL2State &V = *ivf->ivfl2;
    if (V.nc != S.L) return fail(GN_ERR_INVALID, "prober list count does not match the index");
    if (nq <= 0 || k <= 0 || batch <= 0 || epochs <= 0) return fail(GN_ERR_INVALID, "bad training arguments");
    std::lock_guard<std::mutex> lk(pr->mu);
    std::lock_guard<std::mutex> lk2(ivf->mu);
    cudaStream_t st = ivf->stream;
    // features and labels for all training queries (chunks of 8192)
    DBuf dq, keys, cand, feat, lab, dgt, list_of;
    GN_TRY(cand.ensure((size_t)nq * PB_C * 4));
    GN_TRY(feat.ensure((size_t)nq * PB_C * 4));
    GN_TRY(lab.ensure((size_t)nq * PB_C * 4));
    GN_TRY(list_of.ensure((size_t)V.n * 4));
    {
        std::vector<int32_t> ids((size_t)V.n), lo((size_t)V.n);
        GN_CUDA_TRY(cudaMemcpy(ids.data(), V.ids.p, (size_t)V.n * 4, cudaMemcpyDeviceToHost));
        for (int32_t l = 0; l < V.nc; ++l)
            for (int64_t r = V.h_off[(size_t)l]; r < V.h_off[(size_t)l + 1]; ++r) lo[(size_t)ids[(size_t)r]] = l;
        GN_CUDA_TRY(cudaMemcpy(list_of.p, lo.data(), (size_t)V.n * 4, cudaMemcpyHostToDevice));
    }
    const int64_t chunk = 8192;
    for (int64_t q0 = 0; q0 < nq; q0 += chunk) {
        const int64_t nc = std::min(chunk, nq - q0);
        GN_TRY(upload_rows(dq, queries + q0 * V.d, nc, (int64_t)V.d * 4, V.dp / 4, st));
        GN_TRY(keys.ensure((size_t)nc * PB_C * 8));
        GN_TRY(ivfl2_coarse_sorted_keys(ivf, dq.as<float>(), nc, PB_C, keys.as<uint64_t>(), st));
        GN_CUDA_TRY(cudaStreamSynchronize(st));
        GN_TRY(dgt.ensure((size_t)nc * k * 8));
        GN_CUDA_TRY(cudaMemcpyAsync(dgt.p, gt + q0 * k, (size_t)nc * k * 8, cudaMemcpyHostToDevice, st));
        const unsigned blocks = (unsigned)ceil_div(nc * PB_C, 256);
        prober_features_kernel<<<blocks, 256, 0, st>>>(keys.as<uint64_t>(), nc, cand.as<int32_t>() + q0 * PB_C,
                                                      feat.as<float>() + q0 * PB_C);
        prober_labels_kernel<<<blocks, 256, 0, st>>>(cand.as<int32_t>() + q0 * PB_C, dgt.as<int64_t>(), k,
                                                    list_of.as<int32_t>(), nc, lab.as<float>() + q0 * PB_C);
        GN_CUDA_TRY(cudaStreamSynchronize(st));
    }
    // mini-batch training; examples visited in a seeded shuffled order
    std::vector<int64_t> order((size_t)nq);
    for (int64_t i = 0; i < nq; ++i) order[(size_t)i] = i;
    std::mt19937 rng(S.seed + 17);
    DBuf bc, bf, bl, perm;
    GN_TRY(bc.ensure((size_t)batch * PB_C * 4));
    GN_TRY(bf.ensure((size_t)batch * PB_C * 4));
    GN_TRY(bl.ensure((size_t)batch * PB_C * 4));
    std::vector<int32_t> hc((size_t)nq * PB_C);
    std::vector<float> hf((size_t)nq * PB_C), hl((size_t)nq * PB_C);
    GN_CUDA_TRY(cudaMemcpy(hc.data(), cand.p, hc.size() * 4, cudaMemcpyDeviceToHost));
    GN_CUDA_TRY(cudaMemcpy(hf.data(), feat.p, hf.size() * 4, cudaMemcpyDeviceToHost));
    GN_CUDA_TRY(cudaMemcpy(hl.data(), lab.p, hl.size() * 4, cudaMemcpyDeviceToHost));
    std::vector<int32_t> sc((size_t)batch * PB_C);
    std::vector<float> sf((size_t)batch * PB_C), sl((size_t)batch * PB_C);
    for (int32_t e = 0; e < epochs; ++e) {
        std::shuffle(order.begin(), order.end(), rng);
        double esum = 0;
        int64_t nb = 0;
        for (int64_t b0 = 0; b0 + batch <= nq; b0 += batch, ++nb) {
            for (int32_t i = 0; i < batch; ++i) {
                const int64_t src = order[(size_t)(b0 + i)];
                std::memcpy(&sc[(size_t)i * PB_C], &hc[(size_t)src * PB_C], PB_C * 4);
                std::memcpy(&sf[(size_t)i * PB_C], &hf[(size_t)src * PB_C], PB_C * 4);
                std::memcpy(&sl[(size_t)i * PB_C], &hl[(size_t)src * PB_C], PB_C * 4);
            }
            GN_CUDA_TRY(cudaMemcpyAsync(bc.p, sc.data(), sc.size() * 4, cudaMemcpyHostToDevice, st));
            GN_CUDA_TRY(cudaMemcpyAsync(bf.p, sf.data(), sf.size() * 4, cudaMemcpyHostToDevice, st));
            GN_CUDA_TRY(cudaMemcpyAsync(bl.p, sl.data(), sl.size() * 4, cudaMemcpyHostToDevice, st));
            float loss = 0.f;
            GN_TRY(prober_fwd_bwd(S, batch, bc.as<int32_t>(), bf.as<float>(), bl.as<float>(),
                                  (nb % 16 == 0) ? &loss : nullptr, st));
            prober_adam(S, lr, st);
            if (nb % 16 == 0) esum += loss;
        }
        if (loss_out) loss_out[e] = (float)(esum / std::max<int64_t>(1, (nb + 15) / 16));
    }
    GN_TRY(prober_refresh_bf16(S, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    GN_CUDA_TRY(cudaGetLastError());
    S.trained = true;
    return GN_OK;
}

}  // extern "C"

extern "C" {

// Attach (or detach, with pr = NULL) a trained prober to a float IVF index:
// its searches then probe the candidates whose logit is >= logit_tau.
int gn_ivfl2_set_prober(gn_index *ivf, gn_index *pr, float logit_tau) {
    if (!ivf || ivf->kind != K_IVFL2 || !ivf->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    if (pr && pr->kind != K_PROBER) return fail(GN_ERR_INVALID, "not a prober");
    if (pr && pst(pr)->L != ivf->ivfl2->nc) return fail(GN_ERR_INVALID, "prober list count does not match the index");
    std::lock_guard<std::mutex> lk(ivf->mu);
    ivf->ivfl2->prober = pr;
    ivf->ivfl2->prober_tau = logit_tau;
    ivf->ivfl2->cfg++;
    return GN_OK;
}

// Lists probed per query by the last search with a prober (host array of nq).
int gn_ivfl2_last_nprobed(gn_index *ivf, int64_t nq, int32_t *out) {
    if (!ivf || ivf->kind != K_IVFL2 || !ivf->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    IvfScratch &T = ivf->ivfl2->s;
    if (!ivf->ivfl2->prober || !T.nprobed.p || T.nprobed.cap < (size_t)nq * 4)
        return fail(GN_ERR_INVALID, "no learned-probing search has run for that many queries");
    GN_CUDA_TRY(cudaMemcpy(out, T.nprobed.p, (size_t)nq * 4, cudaMemcpyDeviceToHost));
    return GN_OK;
}

}  // extern "C"
