// voronoi.cu — headless Voronoi raster: every pixel of a w×h grid gets the
// index of its nearest seed (exact 1-NN in 2-D, L2), optionally its distance
// and an RGBA colour from a palette, written to device or host buffers.
//
// The reference computes the same raster by building a pixel grid on the host
// (pixel (r, c) = (xs[c], ys[r]), xs/ys = linspace(0, 1)) and running one
// search1NN of all pixels against the seeds (demo/voronoi.py:93-110).  Here the
// grid is never materialised: the kernel reads the two coordinate vectors.
//
// Layout: one block per (row, 1024-column strip); 256 threads, 4 pixels per
// thread at stride 256 so every store is coalesced.  Seeds stream through
// shared memory in tiles of 2048 as (sx, dy²), dy² = (py − sy)² computed once
// per row, so a pixel–seed pair costs one subtract, one multiply, one add and
// (seeds taken four at a time) three quarters of a minimum and a quarter of a
// compare.  The distance is the flat L2 kernel's arithmetic for d = 2,
// sqrt(rn(rn(dx²) + rn(dy²))) with dx = px − sx, dy = py − sy; the argmin is
// over that sqrt value with ties to the lower seed index, the same answer the
// exact flat search1NN gives.  The squared sum prefilters: sqrt is monotone,
// so a pair can only win if its squared sum is below the current best one,
// and the sqrt is taken only then (about ln(ns) times per pixel).  Seeds go
// four at a time: one compare of the four squared sums' minimum against the
// best decides (almost always) that none of them can win, and only otherwise
// are the four offered one by one in seed order, so the branch is taken
// rarely and costs a quarter of a compare per pair.
#include <cmath>

#include "index.cuh"

namespace gn {

constexpr int VR_NT = 256;    // threads per block
constexpr int VR_PX = 4;      // pixels per thread
constexpr int VR_TILE = 2048; // seeds per shared-memory tile (16 KB)
constexpr int VR_STRIP = VR_NT * VR_PX;

__global__ void __launch_bounds__(VR_NT) voronoi_kernel(const float2 *__restrict__ seeds, int ns,
                                                        const float *__restrict__ xs, const float *__restrict__ ys,
                                                        int w, int h, int32_t *__restrict__ ids,
                                                        float *__restrict__ dist,
                                                        const uchar4 *__restrict__ palette, int npal,
                                                        uchar4 *__restrict__ rgba) {
    __shared__ __align__(16) float2 sm[VR_TILE];
    const int cbase = blockIdx.x * VR_STRIP + threadIdx.x;
    float px[VR_PX];
#pragma unroll
    for (int p = 0; p < VR_PX; ++p) {
        const int c = cbase + p * VR_NT;
        px[p] = c < w ? xs[c] : 0.f;
    }
    for (int row = blockIdx.y; row < h; row += gridDim.y) {
        const float py = ys[row];
        float bs[VR_PX], br[VR_PX];
        int bi[VR_PX];
#pragma unroll
        for (int p = 0; p < VR_PX; ++p) {
            bs[p] = INFINITY;
            br[p] = INFINITY;
            bi[p] = 0;
        }
        for (int t0 = 0; t0 < ns; t0 += VR_TILE) {
            const int tn = min(VR_TILE, ns - t0);
            __syncthreads();  // the previous tile (or row) is no longer read
            for (int j = threadIdx.x; j < tn; j += VR_NT) {
                const float2 s = seeds[t0 + j];
                const float dy = __fsub_rn(py, s.y);
                sm[j] = make_float2(s.x, __fmul_rn(dy, dy));
            }
            __syncthreads();
            // offer seed `idx` with squared sum s to pixel p (seed order is kept)
            auto offer = [&](int p, float s, int idx) {
                if (s < bs[p]) {
                    const float r = __fsqrt_rn(s);
                    if (r < br[p]) {  // strictly nearer: equal distances keep the lower index
                        bs[p] = s;
                        br[p] = r;
                        bi[p] = idx;
                    }
                }
            };
            int j = 0;
#pragma unroll 2
            for (; j + 4 <= tn; j += 4) {
                const float4 e01 = *reinterpret_cast<const float4 *>(sm + j);      // (x, dy²) of seeds j, j + 1
                const float4 e23 = *reinterpret_cast<const float4 *>(sm + j + 2);  // seeds j + 2, j + 3
#pragma unroll
                for (int p = 0; p < VR_PX; ++p) {
                    const float d0 = __fsub_rn(px[p], e01.x), d1 = __fsub_rn(px[p], e01.z);
                    const float d2 = __fsub_rn(px[p], e23.x), d3 = __fsub_rn(px[p], e23.z);
                    const float s0 = __fadd_rn(__fmul_rn(d0, d0), e01.y);
                    const float s1 = __fadd_rn(__fmul_rn(d1, d1), e01.w);
                    const float s2 = __fadd_rn(__fmul_rn(d2, d2), e23.y);
                    const float s3 = __fadd_rn(__fmul_rn(d3, d3), e23.w);
                    if (fminf(fminf(s0, s1), fminf(s2, s3)) < bs[p]) {
                        offer(p, s0, t0 + j);
                        offer(p, s1, t0 + j + 1);
                        offer(p, s2, t0 + j + 2);
                        offer(p, s3, t0 + j + 3);
                    }
                }
            }
            for (; j < tn; ++j) {
                const float2 e = sm[j];
#pragma unroll
                for (int p = 0; p < VR_PX; ++p) {
                    const float dx = __fsub_rn(px[p], e.x);
                    offer(p, __fadd_rn(__fmul_rn(dx, dx), e.y), t0 + j);
                }
            }
        }
        const int64_t rowoff = (int64_t)row * w;
#pragma unroll
        for (int p = 0; p < VR_PX; ++p) {
            const int c = cbase + p * VR_NT;
            if (c >= w) continue;
            if (ids) ids[rowoff + c] = bi[p];
            if (dist) dist[rowoff + c] = br[p];
            if (rgba) rgba[rowoff + c] = palette[bi[p] % npal];
        }
    }
}

static int voronoi_check(int64_t ns, int64_t w, int64_t h, const void *seeds, const void *xs, const void *ys,
                         const void *ids, const void *dist, const void *palette, int64_t npal, const void *rgba) {
    if (ns <= 0) return fail(GN_ERR_EMPTY, "voronoi raster needs at least one seed");
    if (ns > 0x7fffffffLL) return fail(GN_ERR_INVALID, "too many seeds");
    if (w <= 0 || h <= 0 || w > 0x7fffffffLL || h > 0x7fffffffLL)
        return fail(GN_ERR_INVALID, "raster width and height must be positive");
    if (!seeds || !xs || !ys) return fail(GN_ERR_INVALID, "NULL pointer argument");
    if (!ids && !dist && !rgba) return fail(GN_ERR_INVALID, "no output requested");
    if (rgba && (!palette || npal <= 0 || npal > 0x7fffffffLL))
        return fail(GN_ERR_INVALID, "an RGBA output needs a non-empty palette");
    return GN_OK;
}

static int voronoi_launch(const float *seeds, int64_t ns, const float *xs, const float *ys, int64_t w, int64_t h,
                          int32_t *ids, float *dist, const uint8_t *palette, int64_t npal, uint8_t *rgba,
                          cudaStream_t st) {
    if ((reinterpret_cast<uintptr_t>(seeds) & 7) || (reinterpret_cast<uintptr_t>(palette) & 3) ||
        (reinterpret_cast<uintptr_t>(rgba) & 3))
        return fail(GN_ERR_INVALID, "seeds must be 8-byte aligned, palette and RGBA output 4-byte aligned");
    dim3 grid((unsigned)ceil_div(w, VR_STRIP), (unsigned)std::min<int64_t>(h, 65535));
    voronoi_kernel<<<grid, VR_NT, 0, st>>>(reinterpret_cast<const float2 *>(seeds), (int)ns, xs, ys, (int)w, (int)h,
                                           ids, dist, reinterpret_cast<const uchar4 *>(palette), (int)npal,
                                           reinterpret_cast<uchar4 *>(rgba));
    GN_CUDA_TRY(cudaGetLastError());
    return GN_OK;
}

}  // namespace gn

using namespace gn;

extern "C" int gn_voronoi_raster_device(const float *d_seeds, int64_t n_seeds, const float *d_xs, int64_t width,
                                        const float *d_ys, int64_t height, int32_t *d_ids, float *d_dist,
                                        const uint8_t *d_palette, int64_t n_palette, uint8_t *d_rgba,
                                        void *stream) {
    GN_TRY(voronoi_check(n_seeds, width, height, d_seeds, d_xs, d_ys, d_ids, d_dist, d_palette, n_palette, d_rgba));
    return voronoi_launch(d_seeds, n_seeds, d_xs, d_ys, width, height, d_ids, d_dist, d_palette, n_palette, d_rgba,
                          (cudaStream_t)stream);
}

extern "C" int gn_voronoi_raster(const float *seeds, int64_t n_seeds, const float *xs, int64_t width,
                                 const float *ys, int64_t height, int32_t *out_ids, float *out_dist,
                                 const uint8_t *palette, int64_t n_palette, uint8_t *out_rgba) {
    GN_TRY(voronoi_check(n_seeds, width, height, seeds, xs, ys, out_ids, out_dist, palette, n_palette, out_rgba));
    // per-thread scratch, reused by later calls of the same thread
    struct Scratch {
        DBuf seeds, xs, ys, ids, dist, pal, rgba;
        cudaStream_t st = nullptr;
    };
    static thread_local Scratch S;
    if (!S.st) GN_CUDA_TRY(cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking));
    const size_t npx = (size_t)width * height;
    GN_TRY(S.seeds.ensure((size_t)n_seeds * 8));
    GN_TRY(S.xs.ensure((size_t)width * 4));
    GN_TRY(S.ys.ensure((size_t)height * 4));
    if (out_ids) GN_TRY(S.ids.ensure(npx * 4));
    if (out_dist) GN_TRY(S.dist.ensure(npx * 4));
    if (out_rgba) {
        GN_TRY(S.pal.ensure((size_t)n_palette * 4));
        GN_TRY(S.rgba.ensure(npx * 4));
    }
    GN_CUDA_TRY(cudaMemcpyAsync(S.seeds.p, seeds, (size_t)n_seeds * 8, cudaMemcpyHostToDevice, S.st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.xs.p, xs, (size_t)width * 4, cudaMemcpyHostToDevice, S.st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.ys.p, ys, (size_t)height * 4, cudaMemcpyHostToDevice, S.st));
    if (out_rgba)
        GN_CUDA_TRY(cudaMemcpyAsync(S.pal.p, palette, (size_t)n_palette * 4, cudaMemcpyHostToDevice, S.st));
    GN_TRY(voronoi_launch(S.seeds.as<float>(), n_seeds, S.xs.as<float>(), S.ys.as<float>(), width, height,
                          out_ids ? S.ids.as<int32_t>() : nullptr, out_dist ? S.dist.as<float>() : nullptr,
                          out_rgba ? S.pal.as<uint8_t>() : nullptr, n_palette,
                          out_rgba ? S.rgba.as<uint8_t>() : nullptr, S.st));
    if (out_ids) GN_CUDA_TRY(cudaMemcpyAsync(out_ids, S.ids.p, npx * 4, cudaMemcpyDeviceToHost, S.st));
    if (out_dist) GN_CUDA_TRY(cudaMemcpyAsync(out_dist, S.dist.p, npx * 4, cudaMemcpyDeviceToHost, S.st));
    if (out_rgba) GN_CUDA_TRY(cudaMemcpyAsync(out_rgba, S.rgba.p, npx * 4, cudaMemcpyDeviceToHost, S.st));
    GN_CUDA_TRY(cudaStreamSynchronize(S.st));
    return GN_OK;
}
