// CUDA-graph form of the device batch (gsx_searcher_search_batch_device).
//
// A caller that searches the same buffers again and again (a fixed-size query slot filled
// between launches) captures the whole batch once: the work-queue reset, the two batch-order
// kernels and the persistent search launch become one CUDA graph, replayed with a single
// cudaGraphLaunch.  Everything the replay touches besides the searcher's resident index and the
// caller's buffers is owned by the graph object (queue counters, per-query status, order keys,
// global visited tables), so later calls on the searcher, which may resize the searcher's own
// scratch, cannot leave the graph pointing at freed memory.  The visited tables' query tags
// advance on the device, so every replay starts on tables that read as empty.
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <new>

#include "gsx_host.h"

namespace gsx {
int server_make_cfg(gsx_searcher *s, int kmax, int efmax, int nq, LaunchCfg *cfg, int *spill_bits);
}  // namespace gsx

using namespace gsx;

struct gsx_batch_graph {
    gsx_searcher *s = nullptr;
    int device = 0;
    // the captured batch
    const float *q = nullptr;
    int nq = 0, k = 0, kmax = 0, ef = 0;
    const int32_t *ef_per = nullptr, *k_per = nullptr;
    int32_t *ids = nullptr, *cmps = nullptr, *exps = nullptr;
    float *dis = nullptr;
    LaunchCfg cfg{};
    int sbits = 0;
    bool ordered = false;
    // scratch owned by the graph
    DevBuf status, counters, qkeys, qorder;
    SpillTables spill;
    uint32_t *gtab = nullptr, *gtab_epoch = nullptr;
    // CUDA objects
    cudaStream_t cap = nullptr;   // private stream of the capture
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr;   // recorded after every launch

    ~gsx_batch_graph() {
        cudaSetDevice(device);
        if (done) cudaEventSynchronize(done);
        if (done) cudaEventDestroy(done);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
    }
};

namespace {

// Enqueues the batch on `st` with the graph's own scratch, the same work as the searcher's device
// batch: queue reset, batch order when the queries outnumber the resident warps, search launch.
int enqueue_owned(gsx_batch_graph *g, cudaStream_t st) {
    gsx_searcher *s = g->s;
    GSX_CUDA(cudaMemsetAsync(g->counters.p, 0, 8, st));
    BatchView bv{};
    bv.queries = g->q;
    bv.nq = g->nq;
    bv.k = g->k;
    bv.ef = g->ef;
    bv.k_per = g->k_per;
    bv.ef_per = g->ef_per;
    bv.order = nullptr;
    bv.single = 0;
    bv.out_stride = g->kmax;
    bv.out_ids = g->ids;
    bv.out_dis = g->dis;
    bv.cmps = g->cmps;
    bv.expansions = g->exps;
    bv.status = g->status.as<int32_t>();
    bv.counter = g->counters.as<unsigned>();
    bv.overflow = g->counters.as<unsigned>() + 1;
    if (g->ordered) {
        GSX_CUDA(launch_batch_order(g->q, g->nq, s->ix.d, s->pdir.as<float>(), s->order_lo, s->order_scale,
                                    g->qkeys.as<uint32_t>(), g->qorder.as<int32_t>(), st));
        bv.order = g->qorder.as<int32_t>();
    }
    bv.gtab = g->gtab;
    bv.gtab_epoch = g->gtab_epoch;
    bv.gtab_bits = g->sbits;
    bv.gtab_shift = visited_id_bits(s->ix.N);
    GSX_CUDA(launch_search(s->ix, bv, g->cfg, st));
    return GSX_OK;
}

int make_graph(gsx_batch_graph *g) {
    gsx_searcher *s = g->s;
    // the caller may have written the queries on any stream: the plain run below reads them
    GSX_CUDA(cudaDeviceSynchronize());
    int rc = server_make_cfg(s, g->kmax, g->ef, g->nq, &g->cfg, &g->sbits);
    if (rc) return rc;
    g->ordered = s->pdir.p && !(s->tuning.prefetch & kNoBatchOrder) &&
                 g->nq > g->cfg.max_blocks * g->cfg.warps_per_block;
    if ((rc = g->status.ensure((size_t)g->nq * 4))) return rc;
    if ((rc = g->counters.ensure(256))) return rc;
    if (g->ordered) {
        if ((rc = g->qkeys.ensure((size_t)g->nq * 4))) return rc;
        if ((rc = g->qorder.ensure((size_t)g->nq * 4))) return rc;
    }
    GSX_CUDA(cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking));
    GSX_CUDA(cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming));
    const size_t slots = (size_t)g->cfg.max_blocks * g->cfg.warps_per_block;
    if ((rc = g->spill.ensure(slots, g->sbits, visited_id_bits(s->ix.N), g->cap, &g->gtab, &g->gtab_epoch))) return rc;
    // one plain run first: it clears the new tables, loads the kernels and sets their shared-memory
    // attributes, so that the capture below records stream work only
    if ((rc = enqueue_owned(g, g->cap))) return rc;
    GSX_CUDA(cudaStreamSynchronize(g->cap));
    GSX_CUDA(cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeRelaxed));
    rc = enqueue_owned(g, g->cap);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(g->cap, &graph);  // ends the capture on every path
    g->graph = graph;
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    GSX_CUDA(cudaGraphInstantiate(&g->exec, g->graph, 0));
    GSX_CUDA(cudaEventRecord(g->done, g->cap));
    return GSX_OK;
}

}  // namespace

extern "C" int gsx_searcher_capture_batch(gsx_searcher *s, const float *d_queries, int32_t nq, int32_t k,
                                          const int32_t *d_ef, const int32_t *d_k, int32_t kmax, int32_t *d_ids,
                                          float *d_dis, int32_t *d_cmps, int32_t *d_expansions,
                                          gsx_batch_graph **out) {
    try {
        if (!out) return fail(GSX_ERR_INVALID, "null argument");
        *out = nullptr;
        if (!s || !d_queries || !d_ids || !d_dis) return fail(GSX_ERR_INVALID, "null argument");
        if (!s->has_data) return fail(GSX_ERR_STATE, "search before set_data");
        if (nq <= 0) return fail(GSX_ERR_INVALID, "a captured batch needs at least one query");
        if (k <= 0) return fail(GSX_ERR_INVALID, "k must be positive");
        if (kmax < k) kmax = k;
        cudaError_t e = cudaSetDevice(s->device);
        if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
        std::unique_ptr<gsx_batch_graph> g(new (std::nothrow) gsx_batch_graph);
        if (!g) return fail(GSX_ERR_NOMEM, "out of host memory");
        g->s = s;
        g->device = s->device;
        g->q = d_queries;
        g->nq = nq;
        g->k = k;
        g->kmax = kmax;
        g->ef = s->ef;  // with per-query ef on the device the searcher's ef is the upper bound
        g->ef_per = d_ef;
        g->k_per = d_k;
        g->ids = d_ids;
        g->dis = d_dis;
        g->cmps = d_cmps;
        g->exps = d_expansions;
        const int rc = make_graph(g.get());
        if (rc) return rc;  // the graph object and its scratch are freed here
        *out = g.release();
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_capture_batch")
}

extern "C" int gsx_batch_graph_launch(gsx_batch_graph *g, void *stream) {
    try {
        if (!g || !g->exec) return fail(GSX_ERR_INVALID, "null argument");
        cudaError_t e = cudaSetDevice(g->device);
        if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
        cudaStream_t st = stream ? (cudaStream_t)stream : g->s->stream;
        e = cudaGraphLaunch(g->exec, st);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
        e = cudaEventRecord(g->done, st);
        if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_batch_graph_launch")
}

extern "C" int gsx_batch_graph_overflow_count(gsx_batch_graph *g, uint32_t *count) {
    try {
        if (!g || !count) return fail(GSX_ERR_INVALID, "null argument");
        cudaError_t e = cudaSetDevice(g->device);
        if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
        if ((e = cudaEventSynchronize(g->done)) != cudaSuccess) return cuda_fail(e, "cudaEventSynchronize");
        if ((e = cudaMemcpy(count, g->counters.as<uint32_t>() + 1, 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail(e, "cudaMemcpy(overflow count)");
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_batch_graph_overflow_count")
}

extern "C" int gsx_batch_graph_destroy(gsx_batch_graph *g) {
    try {
        if (!g) return GSX_OK;
        delete g;  // waits for the latest launch first
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_batch_graph_destroy")
}
