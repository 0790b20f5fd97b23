// ivf_graph.cu — CUDA-graph replay of the float IVF batch pipeline.
//
// A search batch is a chain of about a dozen short kernels (coarse scores,
// probe selection, bucketing, work items, list scan, select) whose launch gaps
// matter at small batches.  With graphs enabled the chain for a batch size is
// captured once into a CUDA graph on fixed staging buffers (queries in,
// indices / distances / counts out) and replayed for every later batch of that
// size: one graph launch per batch.
//
// Validity: a captured graph holds device pointers and kernel arguments of one
// search configuration.  It is dropped when the index's configuration version
// changes (set, set_assigned, n_probe, engine, prober) or when any device
// buffer was reallocated since it was captured.  A new batch size first runs
// the pipeline uncaptured — that sizes every scratch buffer for it and returns
// the batch's results — and is captured right after, so that capture itself
// never allocates.
#include "ivf.cuh"
#include "timing.cuh"

namespace gn {

void IvfGraphs::clear() {
    for (auto &e : execs) cudaGraphExecDestroy(e.second);
    execs.clear();
}

IvfGraphs::~IvfGraphs() {
    clear();
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
}

// Capture the pipeline for nq queries on st into an executable graph.
static int ivf_capture(gn_index *ix, int64_t nq, cudaStream_t st, cudaGraphExec_t *out) {
    IvfL2State &S = *ix->ivfl2;
    IvfGraphs &G = *S.graphs;
    *out = nullptr;
    GN_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int rc = ivfl2_search_core(ix, G.gq.as<float>(), nq, G.k, G.gidx.as<int64_t>(), G.gdist.as<float>(),
                                     G.gcnt.as<int64_t>(), st);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc != GN_OK || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc != GN_OK ? rc : fail(GN_ERR_CUDA, std::string("stream capture: ") + cudaGetErrorString(e));
    }
    const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return fail(GN_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    return GN_OK;
}

// Graphs are captured and replayed on the index's own (non-blocking) stream:
// the caller's stream may be the legacy default stream, which cannot be
// captured.  Events order the two streams both ways.
int ivfl2_search_graph(gn_index *ix, const float *q, bool q_host, int64_t nq, int k, int64_t *idx, float *dist,
                       int64_t *cnt, bool out_host, cudaStream_t user) {
    IvfL2State &S = *ix->ivfl2;
    IvfGraphs &G = *S.graphs;
    const cudaStream_t st = ix->stream;
    if (user != st) {
        GN_CUDA_TRY(cudaEventRecord(G.ev_in, user));
        GN_CUDA_TRY(cudaStreamWaitEvent(st, G.ev_in, 0));
    }
    if (G.dp != S.dp) {  // the data was replaced by rows of another width
        GN_TRY(G.gq.ensure((size_t)G.max_batch * S.dp * 4));
        GN_CUDA_TRY(cudaMemsetAsync(G.gq.p, 0, (size_t)G.max_batch * S.dp * 4, st));
        G.dp = S.dp;
    }
    if (G.cfg != S.cfg || G.gen != dbuf_generation()) {
        G.clear();
        G.cfg = S.cfg;
        G.gen = dbuf_generation();
    }
    // stage the queries at row pitch dp (the padding columns stay zero)
    const cudaMemcpyKind kin = q_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (q_host) {  // a small pageable batch goes through the index's pinned staging
        const void *qs = q;
        GN_TRY(stage_queries(ix, q, (size_t)nq * S.d * 4, st, &qs));
        q = static_cast<const float *>(qs);
    }
    if (S.d == S.dp)
        GN_CUDA_TRY(cudaMemcpyAsync(G.gq.p, q, (size_t)nq * S.d * 4, kin, st));
    else
        GN_CUDA_TRY(cudaMemcpy2DAsync(G.gq.p, (size_t)S.dp * 4, q, (size_t)S.d * 4, (size_t)S.d * 4, (size_t)nq, kin,
                                      st));
    cudaGraphExec_t exec = nullptr;
    for (auto &e : G.execs)
        if (e.first == nq) exec = e.second;
    if (exec) {
        GN_CUDA_TRY(cudaGraphLaunch(exec, st));
        G.replays++;
    } else {
        // first batch of this size: run it uncaptured (sizes the scratch, gives
        // the results), then capture the same pipeline for the next ones
        GN_TRY(ivfl2_search_core(ix, G.gq.as<float>(), nq, k, G.gidx.as<int64_t>(), G.gdist.as<float>(),
                                 G.gcnt.as<int64_t>(), st));
        GN_CUDA_TRY(cudaGetLastError());
        if (G.gen != dbuf_generation()) {  // a buffer grew: graphs of other sizes hold stale pointers
            G.clear();
            G.gen = dbuf_generation();
        }
        const int rc = ivf_capture(ix, nq, st, &exec);
        if (rc == GN_OK && G.gen == dbuf_generation()) {
            G.execs.emplace_back(nq, exec);
        } else {
            if (exec) cudaGraphExecDestroy(exec);
            G.capture_failures++;
        }
    }
    if (out_host) {
        GN_TRY(download_result(ix, idx, G.gidx.p, (size_t)nq * k * 8, st));
        GN_TRY(download_result(ix, dist, G.gdist.p, (size_t)nq * k * 4, st));
        GN_TRY(download_result(ix, cnt, G.gcnt.p, (size_t)nq * 8, st));
    } else {
        GN_CUDA_TRY(cudaMemcpyAsync(idx, G.gidx.p, (size_t)nq * k * 8, cudaMemcpyDeviceToDevice, st));
        GN_CUDA_TRY(cudaMemcpyAsync(dist, G.gdist.p, (size_t)nq * k * 4, cudaMemcpyDeviceToDevice, st));
        GN_CUDA_TRY(cudaMemcpyAsync(cnt, G.gcnt.p, (size_t)nq * 8, cudaMemcpyDeviceToDevice, st));
    }
    // host results: the caller synchronises the index's stream (with the
    // error word's copy behind the results')
    if (!out_host && user != st) {
        GN_CUDA_TRY(cudaEventRecord(G.ev_out, st));
        GN_CUDA_TRY(cudaStreamWaitEvent(user, G.ev_out, 0));
    }
    return GN_OK;
}

}  // namespace gn

using namespace gn;

extern "C" int gn_ivfl2_enable_graphs(gn_index *ix, int64_t max_batch, int32_t k) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    if (max_batch < 0 || (max_batch > 0 && k <= 0)) return fail(GN_ERR_INVALID, "max_batch >= 0 and k > 0 required");
    std::lock_guard<std::mutex> lk(ix->mu);
    IvfL2State &S = *ix->ivfl2;
    if (max_batch == 0) {
        if (S.graphs && ix->stream) cudaStreamSynchronize(ix->stream);
        delete S.graphs;
        S.graphs = nullptr;
        return GN_OK;
    }
    if (S.nc == 0) return fail(GN_ERR_EMPTY, "Index is empty — call set() first");
    GN_TRY(make_stream(ix));
    cudaStream_t st = ix->stream;
    if (!S.graphs) S.graphs = new IvfGraphs;
    IvfGraphs &G = *S.graphs;
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    G.clear();
    G.max_batch = max_batch;
    G.k = k;
    G.dp = S.dp;
    G.replays = G.capture_failures = 0;
    if (!G.ev_in) GN_CUDA_TRY(cudaEventCreateWithFlags(&G.ev_in, cudaEventDisableTiming));
    if (!G.ev_out) GN_CUDA_TRY(cudaEventCreateWithFlags(&G.ev_out, cudaEventDisableTiming));
    GN_TRY(G.gq.ensure((size_t)max_batch * S.dp * 4));
    GN_TRY(G.gidx.ensure((size_t)max_batch * k * 8));
    GN_TRY(G.gdist.ensure((size_t)max_batch * k * 4));
    GN_TRY(G.gcnt.ensure((size_t)max_batch * 8));
    GN_CUDA_TRY(cudaMemsetAsync(G.gq.p, 0, (size_t)max_batch * S.dp * 4, st));
    // size the scratch for the largest batch once, so that smaller batches
    // seldom grow a buffer (and drop the graphs captured so far)
    GN_TRY(ivfl2_search_core(ix, G.gq.as<float>(), max_batch, k, G.gidx.as<int64_t>(), G.gdist.as<float>(),
                             G.gcnt.as<int64_t>(), st));
    GN_CUDA_TRY(cudaStreamSynchronize(st));
    G.cfg = S.cfg;
    G.gen = dbuf_generation();
    return GN_OK;
}

extern "C" int gn_ivfl2_graph_info(gn_index *ix, int64_t *out) {
    if (!ix || ix->kind != K_IVFL2 || !ix->ivfl2 || !out) return fail(GN_ERR_INVALID, "not an IVFFlatL2 index");
    std::lock_guard<std::mutex> lk(ix->mu);
    const IvfGraphs *G = ix->ivfl2->graphs;
    out[0] = G ? G->max_batch : 0;
    out[1] = G ? (int64_t)G->execs.size() : 0;
    out[2] = G ? G->replays : 0;
    out[3] = G ? G->capture_failures : 0;
    return GN_OK;
}
