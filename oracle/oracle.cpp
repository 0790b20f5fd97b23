/*
 * oracle.cpp — CPU restatement of PyNear's search-path arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it through ctypes.
 * Nothing in the shipped library (pynear_gb300/) links, loads or calls it.
 *
 * Every function restates one reference routine, cited as file:line within the
 * PyNear 2.2.0 source tree:
 *   - distance kernels          pynear/include/DistanceFunctions.hpp
 *   - exact k-NN                semantics of VPTree::searchKNN/search1NN
 *                               (pynear/include/VPTree.hpp:143-191) computed by
 *                               exhaustive scan, ties broken by lower index
 *   - float k-means             pynear/include/KMeans.hpp:25-126
 *   - binary IVF build/search   pynear/include/BinaryIVF.hpp:65-227
 *   - float IVF search          pynear/forest.py:63-111,189-204
 *
 * Floating-point order: the float distances follow the x86 AVX2 lane order of
 * the reference (the path its published numbers use).  The file must be built
 * with -ffp-contract=off so that every mul/add/fma below rounds exactly where
 * the reference's intrinsics round.
 *
 * Pinned against the reference extension built from its own sources (see
 * build_ref.sh) by tests/test_oracle_pin.py and the committed fixtures in
 * tests/golden/.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <queue>
#include <random>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

/* ── distances ──────────────────────────────────────────────────────────── */

/* Hamming distance = popcount(a XOR b) over nbytes bytes: the value
 * hamming_u64 / hamming_u32 / hamming_u16 compute (DistanceFunctions.hpp:50-63,
 * 74-86, 98-110, 166-169).  Exact for every width. */
int64_t or_hamming(const uint8_t *a, const uint8_t *b, int64_t nbytes) {
    int64_t h = 0, i = 0;
    for (; i + 8 <= nbytes; i += 8) {  // 64-bit words, as hamming_u64 does
        uint64_t x, y;
        std::memcpy(&x, a + i, 8);
        std::memcpy(&y, b + i, 8);
        h += __builtin_popcountll(x ^ y);
    }
    for (; i < nbytes; ++i) h += __builtin_popcount((unsigned)(a[i] ^ b[i]));
    return h;
}

/* The reference's generic width dispatch dist_hamming (DistanceFunctions.hpp:
 * 431-443) including its accumulator widths: widths that are a multiple of 8/4
 * bytes sum in int64/int32, a multiple of 2 in int16, odd widths in int8
 * (hamming_u8, :121-133), which wraps once the count passes 127.  Used only to
 * document that divergence; the library returns the true count. */
int64_t or_hamming_ref_dispatch(const uint8_t *a, const uint8_t *b, int64_t nbytes) {
    if (nbytes % 4 == 0) return or_hamming(a, b, nbytes);
    if (nbytes % 2 == 0) {
        int16_t h = 0;
        for (int64_t i = 0; i < nbytes; i += 2) {
            uint16_t x = (uint16_t)(a[i] | (a[i + 1] << 8)), y = (uint16_t)(b[i] | (b[i + 1] << 8));
            h = (int16_t)(h + __builtin_popcount((unsigned)(x ^ y)));
        }
        return h;
    }
    int8_t h = 0;
    for (int64_t i = 0; i < nbytes; ++i) h = (int8_t)(h + __builtin_popcount((unsigned)(a[i] ^ b[i])));
    return h;
}

/* dist_l2_f_avx2 (DistanceFunctions.hpp:304-345): eight FMA lane accumulators
 * over blocks of 8, fold high+low 128-bit halves, a 4-wide tail, a masked
 * remainder, two horizontal adds, sqrt.  The tail and remainder are written as
 * mul then add in the reference; its build (-O3 -march=native) contracts each
 * pair into one FMA, and the bit-for-bit pin against that build confirms it,
 * so they are FMAs here. */
static inline float l2sq_avx_order(const float *x, const float *y, int64_t d) {
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int64_t i = 0;
    for (; d - i >= 8; i += 8)
        for (int j = 0; j < 8; ++j) {
            float t = x[i + j] - y[i + j];
            acc[j] = std::fma(t, t, acc[j]);
        }
    float s[4];
    for (int j = 0; j < 4; ++j) s[j] = acc[j + 4] + acc[j];
    if (d - i >= 4) {
        for (int j = 0; j < 4; ++j) {
            float t = x[i + j] - y[i + j];
            s[j] = std::fma(t, t, s[j]);
        }
        i += 4;
    }
    if (d - i > 0) {
        for (int j = 0; j < 4; ++j) {
            float t = (j < d - i) ? (x[i + j] - y[i + j]) : 0.0f;
            s[j] = std::fma(t, t, s[j]);
        }
    }
    float lo = s[0] + s[1];
    float hi = s[2] + s[3];
    return lo + hi;
}

float or_l2(const float *x, const float *y, int64_t d) { return std::sqrt(l2sq_avx_order(x, y, d)); }

/* dist_l1_f_avx2 (DistanceFunctions.hpp:347-382): eight lane sums of |x-y|,
 * lanes added 0..7 in sequence, scalar remainder appended. */
float or_l1(const float *x, const float *y, int64_t d) {
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int64_t i = 0;
    for (; i + 8 <= d; i += 8)
        for (int j = 0; j < 8; ++j) acc[j] = acc[j] + std::fabs(x[i + j] - y[i + j]);
    float total = 0.f;
    for (int j = 0; j < 8; ++j) total += acc[j];
    for (; i < d; ++i) total += std::fabs(x[i] - y[i]);
    return total;
}

/* dist_chebyshev_f_avx2 (DistanceFunctions.hpp:384-420): max |x-y|, which is
 * exact in any order. */
float or_linf(const float *x, const float *y, int64_t d) {
    float m = 0.f;
    for (int64_t i = 0; i < d; ++i) m = std::max(m, std::fabs(x[i] - y[i]));
    return m;
}

typedef float (*fdist_t)(const float *, const float *, int64_t);
static fdist_t pick_metric(int metric) {
    switch (metric) {
    case 0: return or_l2;
    case 1: return or_l1;
    case 2: return or_linf;
    default: return nullptr;
    }
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* ── exact k-NN by exhaustive scan ──────────────────────────────────────── */

/* Exact k nearest neighbours, nearest-first, ties broken by lower index.  The
 * distance values are the reference's (above); the ordering is the contract of
 * VPTree::searchKNN (VPTree.hpp:143-166) with its arbitrary tie order replaced
 * by the lexicographic (distance, index) order.  metric: 0 L2, 1 L1, 2 Linf. */
int or_knn_float(int metric, const float *db, int64_t n, int64_t d, const float *q, int64_t nq, int64_t k,
                 int64_t *out_idx, float *out_dist, int nthreads) {
    fdist_t f = pick_metric(metric);
    if (!f || n <= 0 || k <= 0) return 1;
    int64_t kk = std::min(k, n);
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
    for (int64_t qi = 0; qi < nq; ++qi) {
        std::vector<std::pair<float, int64_t>> v((size_t)n);
        for (int64_t i = 0; i < n; ++i) v[(size_t)i] = {f(q + qi * d, db + i * d, d), i};
        std::partial_sort(v.begin(), v.begin() + kk, v.end());
        for (int64_t j = 0; j < kk; ++j) {
            out_idx[qi * k + j] = v[(size_t)j].second;
            out_dist[qi * k + j] = v[(size_t)j].first;
        }
        for (int64_t j = kk; j < k; ++j) { out_idx[qi * k + j] = -1; out_dist[qi * k + j] = 0.f; }
    }
    return 0;
}

/* Exact Hamming k-NN (true popcount), nearest-first, ties by lower index. */
int or_knn_hamming(const uint8_t *db, int64_t n, int64_t nbytes, const uint8_t *q, int64_t nq, int64_t k,
                   int64_t *out_idx, int64_t *out_dist, int nthreads) {
    if (n <= 0 || k <= 0) return 1;
    int64_t kk = std::min(k, n);
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
    for (int64_t qi = 0; qi < nq; ++qi) {
        // Counting select: distances are small integers, so bucket by distance
        // and walk buckets in ascending order; indices inside a bucket ascend.
        const uint8_t *qq = q + qi * nbytes;
        std::vector<int32_t> dist((size_t)n);
        int64_t maxd = nbytes * 8;
        std::vector<int64_t> hist((size_t)maxd + 2, 0);
        for (int64_t i = 0; i < n; ++i) {
            int32_t dd = (int32_t)or_hamming(qq, db + i * nbytes, nbytes);
            dist[(size_t)i] = dd;
            hist[(size_t)dd]++;
        }
        int64_t cut = 0, acc = 0;
        for (; cut <= maxd; ++cut) {
            acc += hist[(size_t)cut];
            if (acc >= kk) break;
        }
        int64_t below = acc - hist[(size_t)cut];  // count strictly below cut
        int64_t need_at_cut = kk - below;
        std::vector<std::pair<int32_t, int64_t>> sel;
        sel.reserve((size_t)kk);
        for (int64_t i = 0; i < n; ++i) {
            if (dist[(size_t)i] < cut) sel.push_back({dist[(size_t)i], i});
            else if (dist[(size_t)i] == cut && need_at_cut > 0) { sel.push_back({dist[(size_t)i], i}); --need_at_cut; }
        }
        std::sort(sel.begin(), sel.end());
        for (int64_t j = 0; j < kk; ++j) {
            out_idx[qi * k + j] = sel[(size_t)j].second;
            out_dist[qi * k + j] = sel[(size_t)j].first;
        }
        for (int64_t j = kk; j < k; ++j) { out_idx[qi * k + j] = -1; out_dist[qi * k + j] = 0; }
    }
    return 0;
}

/* ── float k-means (KMeans.hpp:25-126) ──────────────────────────────────── */

/* Lloyd's k-means with k-means++ seeding, restated step for step: mt19937(seed)
 * drives the first pick, the D^2-weighted picks (squared dist_l2_f_avx2 values,
 * double running sums, first index with cum >= r) and the re-seeding of empty
 * clusters; assignment takes the first minimum of the sqrt distance; the update
 * sums in float in point order.  Stops when no label changes. */
int or_kmeans_l2(const float *data, int64_t n, int64_t d, int64_t k, int64_t max_iter, uint32_t seed,
                 int32_t *labels_out, float *centroids_out, int64_t *iters_out, int nthreads) {
    if (k <= 0 || k > n) return 1;
    set_threads(nthreads);
    std::mt19937 rng(seed);
    std::uniform_int_distribution<size_t> pick_point(0, (size_t)n - 1);
    std::uniform_real_distribution<float> unif01(0.f, 1.f);

    std::vector<float> centroids((size_t)(k * d));
    std::memcpy(centroids.data(), data + pick_point(rng) * d, (size_t)d * sizeof(float));
    std::vector<float> min_sq((size_t)n, std::numeric_limits<float>::max());
    for (int64_t ci = 1; ci < k; ++ci) {
        const float *prev = centroids.data() + (ci - 1) * d;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            float v = or_l2(data + i * d, prev, d);
            v = v * v;
            if (v < min_sq[(size_t)i]) min_sq[(size_t)i] = v;
        }
        double total = 0.0;
        for (float v : min_sq) total += (double)v;
        double r = (double)unif01(rng) * total;
        double cum = 0.0;
        int64_t chosen = n - 1;
        for (int64_t i = 0; i < n; ++i) {
            cum += (double)min_sq[(size_t)i];
            if (cum >= r) { chosen = i; break; }
        }
        std::memcpy(centroids.data() + ci * d, data + chosen * d, (size_t)d * sizeof(float));
    }

    std::vector<int32_t> labels((size_t)n, 0);
    std::vector<float> newc((size_t)(k * d));
    std::vector<int64_t> counts((size_t)k);
    int64_t it = 0;
    for (; it < max_iter; ++it) {
        int64_t n_changed = 0;
#pragma omp parallel for schedule(static) reduction(+ : n_changed)
        for (int64_t i = 0; i < n; ++i) {
            float best = std::numeric_limits<float>::max();
            int32_t bc = 0;
            for (int64_t c = 0; c < k; ++c) {
                float dd = or_l2(data + i * d, centroids.data() + c * d, d);
                if (dd < best) { best = dd; bc = (int32_t)c; }
            }
            if (labels[(size_t)i] != bc) { labels[(size_t)i] = bc; ++n_changed; }
        }
        if (n_changed == 0) break;
        std::fill(newc.begin(), newc.end(), 0.f);
        std::fill(counts.begin(), counts.end(), 0);
        for (int64_t i = 0; i < n; ++i) {
            int32_t c = labels[(size_t)i];
            float *cp = newc.data() + c * d;
            const float *xi = data + i * d;
            ++counts[(size_t)c];
            for (int64_t j = 0; j < d; ++j) cp[j] += xi[j];
        }
        for (int64_t c = 0; c < k; ++c) {
            float *cp = newc.data() + c * d;
            if (counts[(size_t)c] > 0) {
                float inv = 1.f / (float)counts[(size_t)c];
                for (int64_t j = 0; j < d; ++j) cp[j] *= inv;
            } else {
                std::memcpy(cp, data + pick_point(rng) * d, (size_t)d * sizeof(float));
            }
        }
        centroids.swap(newc);
    }
    std::memcpy(labels_out, labels.data(), (size_t)n * sizeof(int32_t));
    std::memcpy(centroids_out, centroids.data(), (size_t)(k * d) * sizeof(float));
    if (iters_out) *iters_out = it;
    return 0;
}

/* ── binary IVF (BinaryIVF.hpp) ─────────────────────────────────────────── */

/* IVFFlatBinaryIndex::_build (BinaryIVF.hpp:127-227): binary k-means++ with
 * integer D weights (mt19937(seed); pick, then wsel over [0,total) and the first
 * index whose running sum exceeds r), Lloyd iterations assigning to the first
 * nearest centroid, majority vote per bit (count > n_c/2), empty clusters
 * re-seeded by pick(rng) in cluster order.  Outputs k = min(nlist, n) centroids
 * and the final labels; inverted lists are the points of each label in
 * ascending index order (:224-226). */
int or_ivfbin_build(const uint8_t *db, int64_t n, int64_t nbytes, int32_t nlist, int32_t max_iter, uint32_t seed,
                    uint8_t *centroids_out, int32_t *labels_out, int32_t *k_out, int nthreads) {
    if (n <= 0) return 1;
    set_threads(nthreads);
    int32_t k = std::min<int32_t>(nlist, (int32_t)n);
    std::mt19937 rng(seed);
    std::uniform_int_distribution<size_t> pick(0, (size_t)n - 1);
    std::vector<uint8_t> cent((size_t)k * nbytes);
    std::memcpy(cent.data(), db + pick(rng) * nbytes, (size_t)nbytes);
    std::vector<int64_t> min_d((size_t)n, std::numeric_limits<int64_t>::max());
    for (int32_t ci = 1; ci < k; ++ci) {
        const uint8_t *prev = cent.data() + (size_t)(ci - 1) * nbytes;
        for (int64_t i = 0; i < n; ++i) {
            int64_t dd = or_hamming(db + i * nbytes, prev, nbytes);
            if (dd < min_d[(size_t)i]) min_d[(size_t)i] = dd;
        }
        int64_t total = 0;
        for (int64_t v : min_d) total += v;
        size_t chosen = pick(rng);
        if (total > 0) {
            std::uniform_int_distribution<int64_t> wsel(0, total - 1);
            int64_t r = wsel(rng), cum = 0;
            for (int64_t i = 0; i < n; ++i) {
                cum += min_d[(size_t)i];
                if (cum > r) { chosen = (size_t)i; break; }
            }
        }
        std::memcpy(cent.data() + (size_t)ci * nbytes, db + chosen * nbytes, (size_t)nbytes);
    }
    std::vector<int32_t> labels((size_t)n, 0);
    std::vector<int32_t> bit_counts((size_t)k * nbytes * 8);
    std::vector<int32_t> cc((size_t)k);
    for (int32_t it = 0; it < max_iter; ++it) {
        int64_t n_changed = 0;
#pragma omp parallel for schedule(static) reduction(+ : n_changed)
        for (int64_t i = 0; i < n; ++i) {
            int64_t best = std::numeric_limits<int64_t>::max();
            int32_t bc = 0;
            for (int32_t c = 0; c < k; ++c) {
                int64_t dd = or_hamming(db + i * nbytes, cent.data() + (size_t)c * nbytes, nbytes);
                if (dd < best) { best = dd; bc = c; }
            }
            if (labels[(size_t)i] != bc) { labels[(size_t)i] = bc; ++n_changed; }
        }
        if (n_changed == 0) break;
        std::fill(bit_counts.begin(), bit_counts.end(), 0);
        std::fill(cc.begin(), cc.end(), 0);
        for (int64_t i = 0; i < n; ++i) {
            int32_t c = labels[(size_t)i];
            ++cc[(size_t)c];
            int32_t *bcp = bit_counts.data() + (size_t)c * nbytes * 8;
            for (int64_t b = 0; b < nbytes; ++b) {
                uint8_t byte = db[i * nbytes + b];
                for (int bit = 0; bit < 8; ++bit)
                    if ((byte >> bit) & 1) ++bcp[b * 8 + bit];
            }
        }
        for (int32_t c = 0; c < k; ++c) {
            uint8_t *cp = cent.data() + (size_t)c * nbytes;
            std::memset(cp, 0, (size_t)nbytes);
            if (cc[(size_t)c] == 0) {
                std::memcpy(cp, db + pick(rng) * nbytes, (size_t)nbytes);
                continue;
            }
            int32_t half = cc[(size_t)c] / 2;
            const int32_t *bcp = bit_counts.data() + (size_t)c * nbytes * 8;
            for (int64_t b = 0; b < nbytes; ++b) {
                uint8_t byte = 0;
                for (int bit = 0; bit < 8; ++bit)
                    if (bcp[b * 8 + bit] > half) byte |= (uint8_t)(1 << bit);
                cp[b] = byte;
            }
        }
    }
    std::memcpy(centroids_out, cent.data(), cent.size());
    std::memcpy(labels_out, labels.data(), (size_t)n * sizeof(int32_t));
    *k_out = k;
    return 0;
}

/* IVFFlatBinaryIndex::searchKNN (BinaryIVF.hpp:65-111): probe the nprobe
 * centroids first in (distance, centroid id) order, scan their lists in
 * ascending point order.  tie_mode 0 reproduces the reference's max-heap with
 * strict '<' admission (the first scanned item wins a tie at the k-th place and
 * equal distances come out in heap order); tie_mode 1 returns the lexicographic
 * (distance, index) top-k of the same candidate set, which is the library's
 * contract.  Fewer than k results are returned when the probed lists hold fewer
 * than k points; out_cnt[q] gives the count and the rest is -1. */
int or_ivfbin_search(const uint8_t *db, int64_t n, int64_t nbytes, const uint8_t *cent, int32_t kc,
                     const int32_t *labels, const uint8_t *q, int64_t nq, int64_t k, int32_t nprobe, int tie_mode,
                     int64_t *out_idx, int64_t *out_dist, int64_t *out_cnt, int nthreads) {
    set_threads(nthreads);
    std::vector<std::vector<int32_t>> inv((size_t)kc);
    for (int64_t i = 0; i < n; ++i) inv[(size_t)labels[i]].push_back((int32_t)i);
    int32_t np = std::min(nprobe, kc);
#pragma omp parallel for schedule(dynamic)
    for (int64_t qi = 0; qi < nq; ++qi) {
        const uint8_t *qq = q + qi * nbytes;
        std::vector<std::pair<int64_t, int32_t>> cd((size_t)kc);
        for (int32_t c = 0; c < kc; ++c) cd[(size_t)c] = {or_hamming(qq, cent + (size_t)c * nbytes, nbytes), c};
        std::partial_sort(cd.begin(), cd.begin() + np, cd.end());
        std::vector<std::pair<int64_t, int64_t>> res;
        if (tie_mode == 0) {
            std::priority_queue<std::pair<int64_t, int64_t>> heap;
            for (int32_t p = 0; p < np; ++p)
                for (int32_t idx : inv[(size_t)cd[(size_t)p].second]) {
                    int64_t dd = or_hamming(qq, db + (int64_t)idx * nbytes, nbytes);
                    if ((int64_t)heap.size() < k || dd < heap.top().first) {
                        heap.push({dd, (int64_t)idx});
                        if ((int64_t)heap.size() > k) heap.pop();
                    }
                }
            while (!heap.empty()) { res.push_back(heap.top()); heap.pop(); }
            std::reverse(res.begin(), res.end());
        } else {
            for (int32_t p = 0; p < np; ++p)
                for (int32_t idx : inv[(size_t)cd[(size_t)p].second])
                    res.push_back({or_hamming(qq, db + (int64_t)idx * nbytes, nbytes), (int64_t)idx});
            int64_t kk = std::min<int64_t>(k, (int64_t)res.size());
            std::partial_sort(res.begin(), res.begin() + kk, res.end());
            res.resize((size_t)kk);
        }
        out_cnt[qi] = (int64_t)res.size();
        for (int64_t j = 0; j < k; ++j) {
            if (j < (int64_t)res.size()) { out_idx[qi * k + j] = res[(size_t)j].second; out_dist[qi * k + j] = res[(size_t)j].first; }
            else { out_idx[qi * k + j] = -1; out_dist[qi * k + j] = 0; }
        }
    }
    return 0;
}

/* ── float IVF search (forest.py:63-111, 189-204) ───────────────────────── */

/* _IVFFlatIndex.searchKNN for IVFFlatL2Index: coarse squared distances
 * max(0, |q|^2 + |c|^2 - 2 q.c), the nprobe nearest non-empty clusters, then per
 * probed cluster max(0, |q|^2 + |x|^2 - 2 q.x) (squared L2, float32), merged
 * into the k smallest.  The dot products are accumulated in double and rounded
 * once to float, a fixed order standing in for the unspecified BLAS order;
 * ties are broken by lower index.  labels[i] names the cluster of point i;
 * clusters with no point are skipped, as forest.py:51-53 drops them. */
int or_ivfl2_search(const float *db, int64_t n, int64_t d, const float *cent, int32_t nc, const int32_t *labels,
                    const float *q, int64_t nq, int64_t k, int32_t nprobe, int64_t *out_idx, float *out_dist,
                    int64_t *out_cnt, int nthreads) {
    set_threads(nthreads);
    std::vector<std::vector<int32_t>> inv((size_t)nc);
    for (int64_t i = 0; i < n; ++i) inv[(size_t)labels[i]].push_back((int32_t)i);
    std::vector<int32_t> live;
    for (int32_t c = 0; c < nc; ++c)
        if (!inv[(size_t)c].empty()) live.push_back(c);
    int32_t nl = (int32_t)live.size();
    int32_t np = std::min(nprobe, nl);
    auto dotf = [d](const float *a, const float *b) {
        double s = 0;
        for (int64_t j = 0; j < d; ++j) s += (double)a[j] * (double)b[j];
        return (float)s;
    };
    std::vector<float> xnorm((size_t)n);
    for (int64_t i = 0; i < n; ++i) xnorm[(size_t)i] = dotf(db + i * d, db + i * d);
#pragma omp parallel for schedule(dynamic)
    for (int64_t qi = 0; qi < nq; ++qi) {
        const float *qq = q + qi * d;
        float qn = dotf(qq, qq);
        std::vector<std::pair<float, int32_t>> cd((size_t)nl);
        for (int32_t j = 0; j < nl; ++j) {
            const float *cc = cent + (int64_t)live[(size_t)j] * d;
            float v = qn + dotf(cc, cc) - 2.0f * dotf(qq, cc);
            cd[(size_t)j] = {std::max(0.0f, v), live[(size_t)j]};
        }
        std::partial_sort(cd.begin(), cd.begin() + np, cd.end());
        std::vector<std::pair<float, int64_t>> res;
        for (int32_t p = 0; p < np; ++p)
            for (int32_t idx : inv[(size_t)cd[(size_t)p].second]) {
                float v = qn + xnorm[(size_t)idx] - 2.0f * dotf(qq, db + (int64_t)idx * d);
                res.push_back({std::max(0.0f, v), (int64_t)idx});
            }
        int64_t kk = std::min<int64_t>(k, (int64_t)res.size());
        std::partial_sort(res.begin(), res.begin() + kk, res.end());
        out_cnt[qi] = kk;
        for (int64_t j = 0; j < k; ++j) {
            if (j < kk) { out_idx[qi * k + j] = res[(size_t)j].second; out_dist[qi * k + j] = res[(size_t)j].first; }
            else { out_idx[qi * k + j] = -1; out_dist[qi * k + j] = 0.f; }
        }
    }
    return 0;
}

/* Exact squared-L2 k-NN in double precision (the FP64 host oracle for the
 * tensor-core shortlist and the IVF recall ground truth): nearest-first, ties
 * by lower index; out_dist holds the double squared distances. */
int or_knn_l2sq_f64(const float *db, int64_t n, int64_t d, const float *q, int64_t nq, int64_t k, int64_t *out_idx,
                    double *out_dist, int nthreads) {
    if (n <= 0 || k <= 0) return 1;
    int64_t kk = std::min(k, n);
    set_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
    for (int64_t qi = 0; qi < nq; ++qi) {
        const float *qq = q + qi * d;
        // bounded max-heap of (dist, idx)
        std::priority_queue<std::pair<double, int64_t>> heap;
        for (int64_t i = 0; i < n; ++i) {
            const float *x = db + i * d;
            double s = 0;
            for (int64_t j = 0; j < d; ++j) { double t = (double)qq[j] - (double)x[j]; s += t * t; }
            if ((int64_t)heap.size() < kk) heap.push({s, i});
            else if (std::make_pair(s, i) < heap.top()) { heap.pop(); heap.push({s, i}); }
        }
        for (int64_t j = kk - 1; j >= 0; --j) { out_idx[qi * k + j] = heap.top().second; out_dist[qi * k + j] = heap.top().first; heap.pop(); }
        for (int64_t j = kk; j < k; ++j) { out_idx[qi * k + j] = -1; out_dist[qi * k + j] = 0; }
    }
    return 0;
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
