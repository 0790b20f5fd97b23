// mih.cu — multi-index hashing for binary descriptors: candidate lookup on the
// host, candidate verification (exact Hamming + top-k) on the GPU.
//
// Semantics of MIHBinaryIndex (pynear/include/MIH.hpp:58-175): a descriptor of
// nbytes is cut into m sub-strings of nbytes/m <= 8 bytes; table t maps the
// t-th sub-string (little-endian key) to the rows holding it.  A query's
// candidates are the rows whose t-th sub-string lies within floor(radius / m)
// bits of the query's, for some t (pigeonhole: every row within radius bits
// is one).  The k nearest candidates by exact Hamming distance are returned,
// nearest first; ties go to the lower row index (the reference leaves them to
// its hash-set order).  Fewer than k results when fewer rows are candidates.
//
// GB300 split: the tables are host hash maps of CSR buckets (built once at
// set()); a search enumerates the neighbour keys and gathers each query's
// de-duplicated candidate ids on host threads, uploads them as one CSR, and
// one warp per query computes the candidates' distances from the device copy
// of the rows (128-bit loads, POPC) into a register top-k.
#include <algorithm>
#include <cstring>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "index.cuh"
#include "topk.cuh"

namespace gn {

struct MihState {
    int32_t m = 8;
    int64_t n = 0, nbytes = 0, sub_nbytes = 0, pitch16 = 0;
    std::vector<std::unordered_map<uint64_t, uint32_t>> bucket_of;  // per table: key -> bucket
    std::vector<std::vector<int64_t>> boff;                         // per table: bucket offsets
    std::vector<std::vector<int32_t>> ids;                          // per table: rows, ascending per bucket
    DBuf rows, q, coff, cand, oidx, odist, ocnt;
};

static MihState *mst(gn_index *ix) { return reinterpret_cast<MihState *>(ix->ext); }

static inline uint64_t sub_key(const uint8_t *row, int32_t t, int64_t sub_nbytes) {
    uint64_t key = 0;
    std::memcpy(&key, row + (size_t)t * sub_nbytes, (size_t)sub_nbytes);
    return key;
}

// every key within `radius` flipped bits of `key` among its low `nbits` bits
static void neighbour_keys(uint64_t key, int nbits, int radius, int start, std::vector<uint64_t> &out) {
    out.push_back(key);
    if (radius == 0) return;
    for (int b = start; b < nbits; ++b) neighbour_keys(key ^ ((uint64_t)1 << b), nbits, radius - 1, b + 1, out);
}

// One warp per query: exact Hamming distance to each candidate (lane-strided),
// register top-k of (distance, row) keys.
template <int R>
__global__ void mih_verify_kernel(const uint4 *__restrict__ rows, int w16, const uint4 *__restrict__ q,
                                  const int64_t *__restrict__ coff, const int32_t *__restrict__ cand, int64_t nq,
                                  int k, int64_t *__restrict__ out_idx, int64_t *__restrict__ out_dist,
                                  int64_t *__restrict__ out_cnt) {
    const int lane = threadIdx.x & 31;
    const int64_t qi = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (qi >= nq) return;
    const uint4 *qr = q + qi * w16;
    WarpTopK<R> L;
    L.init();
    uint64_t thr = KEY_EMPTY;
    const int64_t c0 = coff[qi], c1 = coff[qi + 1];
    for (int64_t base = c0; base < c1; base += 32) {
        const int64_t c = base + lane;
        uint64_t key = KEY_EMPTY;
        if (c < c1) {
            const int32_t id = cand[c];
            const uint4 *xr = rows + (int64_t)id * w16;
            uint32_t d = 0;
            for (int w = 0; w < w16; ++w) {
                const uint4 a = __ldg(xr + w), b = __ldg(qr + w);
                d += __popc(a.x ^ b.x) + __popc(a.y ^ b.y) + __popc(a.z ^ b.z) + __popc(a.w ^ b.w);
            }
            key = make_key(d, (uint32_t)id);
        }
        L.offer(key, thr, k);
    }
    int cnt = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int pos = r * 32 + lane;
        const uint64_t key = L.v[r];
        const bool e = key == KEY_EMPTY;
        if (pos < k) {
            out_idx[qi * k + pos] = e ? -1 : (int64_t)key_idx(key);
            out_dist[qi * k + pos] = e ? 0 : (int64_t)key_dist(key);
        }
        cnt += __popc(__ballot_sync(0xffffffffu, pos < k && !e));
    }
    if (lane == 0) out_cnt[qi] = cnt;
}

}  // namespace gn

using namespace gn;

extern "C" int gn_mih_create(int32_t m, gn_index **out) {
    if (!out) return fail(GN_ERR_INVALID, "null output");
    if (m <= 0) return fail(GN_ERR_INVALID, "MIH: m must be positive");
    gn_index *ix = new gn_index();
    ix->kind = K_MIH;
    MihState *S = new MihState();
    S->m = m;
    ix->ext = S;
    ix->ext_free = [](void *p) { delete reinterpret_cast<MihState *>(p); };
    *out = ix;
    return GN_OK;
}

extern "C" int gn_mih_set(gn_index *ix, const uint8_t *data, int64_t n, int64_t nbytes) {
    if (!ix || ix->kind != K_MIH) return fail(GN_ERR_INVALID, "not an MIH index");
    MihState &S = *mst(ix);
    std::lock_guard<std::mutex> lk(ix->mu);
    S.n = 0;
    S.bucket_of.clear();
    S.boff.clear();
    S.ids.clear();
    if (n <= 0) return GN_OK;  // empty index: searches return no results
    if (!data || nbytes <= 0) return fail(GN_ERR_INVALID, "MIH: bad data");
    if (n >= 0x7fffffffLL) return fail(GN_ERR_UNSUPPORTED, "MIH: at most 2^31-2 rows");
    if (nbytes < S.m || nbytes % S.m != 0)
        return fail(GN_ERR_INVALID, "MIH: descriptor byte width must be divisible by m");
    if (nbytes / S.m > 8)
        return fail(GN_ERR_INVALID,
                    "MIH: sub-string width exceeds 8 bytes (uint64_t key capacity). Increase m so that nbytes/m <= 8.");
    S.nbytes = nbytes;
    S.sub_nbytes = nbytes / S.m;
    S.pitch16 = round_up(nbytes, 16);
    // tables: count per key, offsets, fill (rows ascending within a bucket)
    S.bucket_of.assign((size_t)S.m, {});
    S.boff.assign((size_t)S.m, {});
    S.ids.assign((size_t)S.m, {});
    for (int32_t t = 0; t < S.m; ++t) {
        auto &map = S.bucket_of[(size_t)t];
        std::vector<int64_t> count;
        std::vector<uint32_t> bkt((size_t)n);
        map.reserve((size_t)n);
        for (int64_t i = 0; i < n; ++i) {
            const uint64_t key = sub_key(data + i * nbytes, t, S.sub_nbytes);
            auto it = map.find(key);
            if (it == map.end()) {
                it = map.emplace(key, (uint32_t)count.size()).first;
                count.push_back(0);
            }
            bkt[(size_t)i] = it->second;
            ++count[it->second];
        }
        auto &off = S.boff[(size_t)t];
        off.assign(count.size() + 1, 0);
        for (size_t b = 0; b < count.size(); ++b) off[b + 1] = off[b] + count[b];
        auto &idv = S.ids[(size_t)t];
        idv.resize((size_t)n);
        std::vector<int64_t> fill(off.begin(), off.end() - 1);
        for (int64_t i = 0; i < n; ++i) idv[(size_t)fill[bkt[(size_t)i]]++] = (int32_t)i;
    }
    GN_TRY(make_stream(ix));
    GN_TRY(upload_rows(S.rows, data, n, nbytes, (int)(S.pitch16 / 16), ix->stream));
    GN_CUDA_TRY(cudaStreamSynchronize(ix->stream));
    S.n = n;
    ix->n = n;
    ix->dim = nbytes;
    return GN_OK;
}

extern "C" int gn_mih_search_knn(gn_index *ix, const uint8_t *queries, int64_t nq, int64_t k, int32_t radius,
                                 int64_t *out_idx, int64_t *out_dist, int64_t *out_cnt) {
    if (!ix || ix->kind != K_MIH) return fail(GN_ERR_INVALID, "not an MIH index");
    if (k <= 0 || k > 256) return fail(GN_ERR_INVALID, "MIH: k must be in [1, 256]");
    if (radius < 0) return fail(GN_ERR_INVALID, "MIH: radius must be >= 0");
    if (nq < 0 || (nq > 0 && (!queries || !out_idx || !out_dist || !out_cnt)))
        return fail(GN_ERR_INVALID, "bad query arguments");
    MihState &S = *mst(ix);
    std::lock_guard<std::mutex> lk(ix->mu);
    if (nq == 0) return GN_OK;
    if (S.n == 0) {  // empty index: no candidates
        for (int64_t i = 0; i < nq * k; ++i) {
            out_idx[i] = -1;
            out_dist[i] = 0;
        }
        for (int64_t i = 0; i < nq; ++i) out_cnt[i] = 0;
        return GN_OK;
    }
    // candidates of every query, on host threads (each query: its neighbour
    // keys in each table, the buckets' rows, sorted and de-duplicated)
    const int r_sub = radius / S.m;
    const int nbits = (int)(S.sub_nbytes * 8);
    std::vector<std::vector<int32_t>> cands((size_t)nq);
    const int nthreads = (int)std::max<unsigned>(1, std::min<unsigned>(std::thread::hardware_concurrency(), 64));
    auto work = [&](int tid) {
        std::vector<uint64_t> keys;
        for (int64_t qi = tid; qi < nq; qi += nthreads) {
            std::vector<int32_t> &c = cands[(size_t)qi];
            const uint8_t *qr = queries + qi * S.nbytes;
            for (int32_t t = 0; t < S.m; ++t) {
                keys.clear();
                neighbour_keys(sub_key(qr, t, S.sub_nbytes), nbits, r_sub, 0, keys);
                const auto &map = S.bucket_of[(size_t)t];
                const auto &off = S.boff[(size_t)t];
                const auto &idv = S.ids[(size_t)t];
                for (uint64_t key : keys) {
                    auto it = map.find(key);
                    if (it == map.end()) continue;
                    c.insert(c.end(), idv.begin() + off[it->second], idv.begin() + off[it->second + 1]);
                }
            }
            std::sort(c.begin(), c.end());
            c.erase(std::unique(c.begin(), c.end()), c.end());
        }
    };
    {
        std::vector<std::thread> pool;
        for (int t = 1; t < nthreads; ++t) pool.emplace_back(work, t);
        work(0);
        for (auto &th : pool) th.join();
    }
    std::vector<int64_t> coff((size_t)nq + 1, 0);
    for (int64_t qi = 0; qi < nq; ++qi) coff[(size_t)qi + 1] = coff[(size_t)qi] + (int64_t)cands[(size_t)qi].size();
    std::vector<int32_t> flat((size_t)std::max<int64_t>(coff[(size_t)nq], 1));
    for (int64_t qi = 0; qi < nq; ++qi)
        std::copy(cands[(size_t)qi].begin(), cands[(size_t)qi].end(), flat.begin() + coff[(size_t)qi]);
    cudaStream_t st = ix->stream;
    GN_TRY(upload_rows(S.q, queries, nq, S.nbytes, (int)(S.pitch16 / 16), st));
    GN_TRY(S.coff.ensure(coff.size() * 8));
    GN_TRY(S.cand.ensure(flat.size() * 4));
    GN_TRY(S.oidx.ensure((size_t)nq * k * 8));
    GN_TRY(S.odist.ensure((size_t)nq * k * 8));
    GN_TRY(S.ocnt.ensure((size_t)nq * 8));
    GN_CUDA_TRY(cudaMemcpyAsync(S.coff.p, coff.data(), coff.size() * 8, cudaMemcpyHostToDevice, st));
    GN_CUDA_TRY(cudaMemcpyAsync(S.cand.p, flat.data(), flat.size() * 4, cudaMemcpyHostToDevice, st));
    const unsigned blocks = (unsigned)ceil_div(nq, 4);
    const int w16 = (int)(S.pitch16 / 16);
    auto launch = [&](auto RC) -> int {
        constexpr int R = decltype(RC)::value;
        mih_verify_kernel<R><<<blocks, 128, 0, st>>>(S.rows.as<uint4>(), w16, S.q.as<uint4>(), S.coff.as<int64_t>(),
                                                     S.cand.as<int32_t>(), nq, (int)k, S.oidx.as<int64_t>(),
                                                     S.odist.as<int64_t>(), S.ocnt.as<int64_t>());
        return GN_OK;
    };
    if (k <= 32) GN_TRY(launch(std::integral_constant<int, 1>()));
    else if (k <= 64) GN_TRY(launch(std::integral_constant<int, 2>()));
    else if (k <= 128) GN_TRY(launch(std::integral_constant<int, 4>()));
    else GN_TRY(launch(std::integral_constant<int, 8>()));
    GN_CUDA_TRY(cudaGetLastError());
    GN_CUDA_TRY(cudaMemcpyAsync(out_idx, S.oidx.p, (size_t)nq * k * 8, cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaMemcpyAsync(out_dist, S.odist.p, (size_t)nq * k * 8, cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaMemcpyAsync(out_cnt, S.ocnt.p, (size_t)nq * 8, cudaMemcpyDeviceToHost, st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    return GN_OK;
}

extern "C" int gn_mih_info(gn_index *ix, int32_t *m, int64_t *n, int64_t *nbytes) {
    if (!ix || ix->kind != K_MIH) return fail(GN_ERR_INVALID, "not an MIH index");
    MihState &S = *mst(ix);
    if (m) *m = S.m;
    if (n) *n = S.n;
    if (nbytes) *nbytes = S.n ? S.nbytes : 0;
    return GN_OK;
}
