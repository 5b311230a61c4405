/*
 * glass_gb300.h - C ABI of the GB300 graph-search path (libglass_gb300.so).
 *
 * Plain pointers, sizes and status codes; no C++ or framework types cross this boundary.  Every
 * entry point returns GSX_OK (0) or a GSX_ERR_* code; gsx_last_error() gives the message of the
 * calling thread's last failure.  Each declaration names the reference interface it replaces
 * (zilliztech/pyglass, path:line).
 *
 * Threading: a searcher handle owns one CUDA stream and its device buffers; calls on the same
 * handle must not overlap (the reference's Searcher.search is not re-entrant either,
 * glass/searcher/graph_searcher.hpp:133).  Different handles may be used from different threads.
 */
#ifndef GLASS_GB300_H
#define GLASS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GSX_OK = 0,
    GSX_ERR_INVALID = 1,     /* bad argument, unknown string, malformed file */
    GSX_ERR_CUDA = 2,        /* CUDA runtime error (message carries the CUDA error string) */
    GSX_ERR_NOMEM = 3,       /* device or host allocation failed / admission refused */
    GSX_ERR_STATE = 4,       /* call out of order (e.g. search before set_data) */
    GSX_ERR_IO = 5,          /* file could not be opened / read / written */
    GSX_ERR_TIMEOUT = 6,     /* a bounded wait gave up */
    GSX_ERR_UNSUPPORTED = 7  /* valid in the reference but outside this path (e.g. PQ8) */
};

typedef struct gsx_graph gsx_graph;
typedef struct gsx_searcher gsx_searcher;

/* Message of the calling thread's last failed call ("" if none). */
const char *gsx_last_error(void);
/* Library version string. */
const char *gsx_version(void);
/* Number of visible CUDA devices (0 when there is none; never fails). */
int gsx_device_count(void);

/* ---- graphs: glass::Graph<int32_t> (glass/graph.hpp:26-246) -------------------------------- */

/* Graph(filename, format) / Graph::load (python/bindings.cc:47-57, glass/graph.hpp:255-287).
 * format: "glass" (with optional HNSW upper levels, HNSWInitializer.hpp:64-75), "nsg",
 * "diskann" or "hnswlib" (graph.hpp:289-379).  The graph is validated: every id is -1 or in
 * [0, N), and every HNSW upper-level neighbour exists on that level. */
int gsx_graph_load(const char *filename, const char *format, gsx_graph **out);
/* Builds a graph from memory: adj is N*K int32 (-1 padded), eps the entry points. */
int gsx_graph_create(const int32_t *adj, int32_t N, int32_t K, const int32_t *eps, int32_t nep, gsx_graph **out);
/* Attaches HNSW upper levels (HNSWInitializer, glass/hnsw/HNSWInitializer.hpp:22-86) to a graph:
 * hK = upper-level degree, ep = entry point, levels[N] = number of upper levels of each node,
 * lists = the nodes' level lists concatenated in node order (levels[u]*hK int32 each, -1 padded).
 * The graph is re-validated. */
int gsx_graph_set_levels(gsx_graph *g, int32_t hK, int32_t ep, const int32_t *levels, const int32_t *lists);
/* Graph::save (graph.hpp:240-253) in the glass format. */
int gsx_graph_save(const gsx_graph *g, const char *filename);
/* N, K, number of entry points, and whether HNSW upper levels are present. */
int gsx_graph_info(const gsx_graph *g, int32_t *N, int32_t *K, int32_t *nep, int32_t *has_hnsw);
/* Copies the adjacency (N*K int32) out. */
int gsx_graph_adjacency(const gsx_graph *g, int32_t *adj_out);
/* Copies the entry points (nep int32, Graph::eps, graph.hpp:37) out. */
int gsx_graph_eps(const gsx_graph *g, int32_t *eps_out);
void gsx_graph_destroy(gsx_graph *g);

/* ---- searchers: GraphSearcherBase (glass/searcher/searcher_base.hpp:7-19) ---------------- */

/* create_searcher(graph, metric, quantizer, refine_quant) (graph_searcher.hpp:256-391).
 * metric "L2" | "IP"; quantizer "SQ8U" | "SQ8" | "SQ4U" | "SQ4UA" | "SQ2U" | "SQ1" (IP only, as
 * in the reference) | "E5M2" | "FP32" | "FP16" | "BF16" (an unknown name selects FP32, as the
 * reference's quantizer_map does; SQ6, SQ4, SQ8P and PQ8 return GSX_ERR_UNSUPPORTED); refine_quant as make_refiner reads it
 * (graph_searcher.hpp:227-254): "" none, "FP16" an FP16 store, "FP32" or a name the quantizer map
 * lacks an FP32 store, any other known name no refiner; "SQ8U" / "SQ8" with an SQ quantizer return
 * GSX_ERR_UNSUPPORTED.  The graph's contents move into the searcher (python/bindings.cc:98); *graph
 * is left empty but must still be destroyed.  device = CUDA ordinal. */
int gsx_searcher_create(gsx_graph *graph, const char *metric, const char *quantizer, const char *refine_quant,
                        int device, gsx_searcher **out);
void gsx_searcher_destroy(gsx_searcher *s);

/* SetData (graph_searcher.hpp:51-70, refiner.hpp:26-37): calibrates the quantizer, encodes the
 * n x dim fp32 rows on the device and keeps the codes (and the FP32 refine store) resident. */
int gsx_searcher_set_data(gsx_searcher *s, const float *data, int32_t n, int32_t dim);

/* SetEf / GetEf (graph_searcher.hpp:72-74). */
int gsx_searcher_set_ef(gsx_searcher *s, int32_t ef);
int gsx_searcher_get_ef(const gsx_searcher *s, int32_t *ef);

/* Search (graph_searcher.hpp:131-138, refiner.hpp:45-70): one query, host buffers; ids[k],
 * dis[k].  The plain per-query GPU form: one launch, one warp. */
int gsx_searcher_search(gsx_searcher *s, const float *query, int32_t k, int32_t *ids, float *dis);

/* SearchBatch (graph_searcher.hpp:143-159, refiner.hpp:72-90): nq queries from host memory,
 * results to host memory, one batched launch.  dis may be NULL. */
int gsx_searcher_search_batch(gsx_searcher *s, const float *queries, int32_t nq, int32_t k, int32_t *ids,
                              float *dis);

/* Batched search with per-query ef and k (either array may be NULL = uniform), buffers in
 * DEVICE memory, enqueued on `stream` (cudaStream_t, NULL = the searcher's stream) without a
 * host synchronisation.  Per-query ef values must not exceed the searcher's ef (set_ef) and
 * per-query k values must not exceed kmax; output rows have stride kmax.  d_cmps / d_expansions
 * (may be NULL) receive per-query distance and expansion counts.  A query whose shared-memory
 * visited table would overflow is left as -1/inf and counted (gsx_searcher_overflow_count); the
 * host-buffer entry points re-run such queries exactly.  No reference counterpart: the
 * batched/persistent form. */
int gsx_searcher_search_batch_device(gsx_searcher *s, const float *d_queries, int32_t nq, int32_t k,
                                     const int32_t *d_ef, const int32_t *d_k, int32_t kmax, int32_t *d_ids,
                                     float *d_dis, int32_t *d_cmps, int32_t *d_expansions, void *stream);

/* Queries of the last device batch left unanswered because their visited table overflowed
 * (synchronises the searcher's stream). */
int gsx_searcher_overflow_count(gsx_searcher *s, uint32_t *count);

/* ---- CUDA-graph form of the device batch (no reference counterpart) ----------------------- */
typedef struct gsx_batch_graph gsx_batch_graph;

/* Captures gsx_searcher_search_batch_device with these arguments (the searcher's current ef and
 * tuning) as one CUDA graph: work-queue reset, batch-order kernels and the persistent search.
 * Replays (gsx_batch_graph_launch) read the same device buffers, so a caller refills d_queries
 * (and d_ef / d_k) in place between launches.  The call synchronises the device, runs the batch
 * once without capture (the outputs then hold its results), and returns the graph.  The graph owns
 * its scratch (queue counters, status words, order keys, visited tables); it uses the searcher's
 * resident index, so it must be destroyed before the searcher and is invalid after a new
 * gsx_searcher_set_data.  As in the device batch, a query whose visited table overflows is left
 * as -1/inf and counted (gsx_batch_graph_overflow_count). */
int gsx_searcher_capture_batch(gsx_searcher *s, const float *d_queries, int32_t nq, int32_t k,
                               const int32_t *d_ef, const int32_t *d_k, int32_t kmax, int32_t *d_ids, float *d_dis,
                               int32_t *d_cmps, int32_t *d_expansions, gsx_batch_graph **out);
/* One replay on `stream` (cudaStream_t, NULL = the searcher's stream), without a host
 * synchronisation.  Replays of one graph run one after another, whichever streams they go to. */
int gsx_batch_graph_launch(gsx_batch_graph *g, void *stream);
/* Queries of the latest replay left unanswered (waits for that replay). */
int gsx_batch_graph_overflow_count(gsx_batch_graph *g, uint32_t *count);
/* Waits for the latest replay and frees the graph and its scratch; NULL is accepted. */
int gsx_batch_graph_destroy(gsx_batch_graph *g);

/* Allocation-free batched search; no counterpart in the reference.  For callers that may not
 * allocate device memory while they serve: engines that hand all GPU memory to their own pool at
 * start-up, and latency-bound paths that cannot take the device-wide synchronisation an allocation
 * or free can cause.  The call allocates nothing: d_queries (nq x dim fp32) and d_ids / d_dis
 * (nq x k) are the caller's device buffers, and the per-call scratch (work-queue counters and one
 * status word per query) is a fixed array inside the library, about 256 KB on every GPU that loads
 * it, held until the process exits.  Hence at most 65,536 queries per call; a larger nq is
 * rejected with GSX_ERR_INVALID.  The first call on a device looks up that array's device address;
 * make it before any stream capture.  All calls share the array and it keeps the last call's
 * contents: calls that overlap on the GPU (other streams or threads) race, so the caller must
 * serialise them.  Enqueued on `stream` (NULL = the searcher's stream) with the searcher's ef,
 * without synchronising.  A query whose visited set outgrows its shared-memory table is left
 * unanswered: all its k ids are -1 and its distances +inf (the allocating entry points answer every
 * query).  A query that ran to the end always returns at least one id, since its entry point enters
 * its pool, so ids[q*k] == -1 marks an unanswered query; gsx_searcher_noalloc_overflow_count gives
 * how many there were.  The current CUDA device of the calling thread is unchanged on return. */
int gsx_searcher_search_batch_noalloc(gsx_searcher *s, const float *d_queries, int32_t nq, int32_t k,
                                      int32_t *d_ids, float *d_dis, void *stream);
/* Number of queries the latest allocation-free search on the searcher's device left unanswered,
 * read from the same fixed array (no allocation).  Call it after synchronising the stream that
 * search ran on; it reads whatever the array holds at that moment, so a later allocation-free call
 * on the device replaces the count.  No counterpart in the reference. */
int gsx_searcher_noalloc_overflow_count(gsx_searcher *s, uint32_t *count);

/* Same as above with HOST buffers (copies inside), synchronous. */
int gsx_searcher_search_batch_mixed(gsx_searcher *s, const float *queries, int32_t nq, int32_t k,
                                    const int32_t *ef, const int32_t *kq, int32_t kmax, int32_t *ids, float *dis);

/* Optimize (graph_searcher.hpp:76-129): the reference tunes CPU prefetch depth on 1,000
 * sampled base rows; here the same sample tunes warps per CTA, visited-table size and lanes
 * per row.  num_threads is accepted for signature parity and ignored. */
int gsx_searcher_optimize(gsx_searcher *s, int32_t num_threads);

/* GetLastSearchAvgDistCmps (graph_searcher.hpp:140-141): average distance computations per
 * query of the last batched search. */
int gsx_searcher_get_last_search_avg_dist_cmps(const gsx_searcher *s, double *out);

/* Tuning knobs chosen by gsx_searcher_optimize (0 = automatic). */
typedef struct {
    int32_t warps_per_block;  /* queries per CTA */
    int32_t table_bits;       /* log2 of the per-query visited-table slots in shared memory
                                 (1 = none: the visited set lives in the warp's global table) */
    int32_t lanes_per_row;    /* lanes cooperating on one code row (SQ kinds) */
    int32_t prefetch;         /* bit 4: run batches larger than one wave of resident warps in index
                                 order instead of sorted along the base data's principal
                                 direction (the order never changes a result); bit 3: do not
                                 stage neighbour code rows in shared memory during the visited
                                 check (staging applies to the integer kinds' rows of at most 128
                                 bytes and E5M2 rows of at most 256); bit 2: prefetch each
                                 neighbour's code row into L1 before its visited check (unstaged
                                 rows); bit 1: load the next adjacency row during the merge (the
                                 merge settles the next pop before it moves pool entries); bit 0:
                                 also prefetch that row's code rows; bit 5: also prefetch the
                                 visited-table buckets of that row's neighbours */
    int32_t spill_bits;       /* log2 of the slots of each warp's global visited table (4 bytes a
                                 slot; 7..20, 0 = sized from the visit counts seen).  A size that
                                 gsx_searcher_optimize picked applies to launches whose automatic
                                 size is at most the one it tuned against; others get the
                                 automatic size. */
} gsx_tuning;
int gsx_searcher_get_tuning(const gsx_searcher *s, gsx_tuning *t);
int gsx_searcher_set_tuning(gsx_searcher *s, const gsx_tuning *t);

/* Device memory (bytes) the index holds resident, and the bytes one in-flight query needs. */
int gsx_searcher_memory(const gsx_searcher *s, size_t *index_bytes, size_t *per_query_bytes);

/* ---- distance computers: ComputerImpl::operator() (glass/quant/computer.hpp:42-75) -------- */

/* out[i*m+j] = distance(query i, base row ids[i*m+j]) with the searcher's quantizer (refine=0)
 * or its FP32 refine store (refine=1), computed by the same device code the search uses.
 * Host buffers.  SQ distances are exact integers returned as double. */
int gsx_searcher_distances(gsx_searcher *s, const float *queries, int32_t nq, const int32_t *ids, int32_t m,
                           int32_t refine, double *out);

/* Copies out the encoded base rows (n*code_size bytes) and calibrator parameters (2 floats: min and
 * dif, or max for the symmetric calibrator; for SQ8 the first dimension's min and dif, see below). */
int gsx_searcher_codes(const gsx_searcher *s, uint8_t *codes, float *params, int32_t *code_size);

/* All calibrator parameters of the search quantizer: *count = 2 (scalar calibrators), or 2*dalign for
 * SQ8's per-dimension calibrator (AffinePerDimCalibrator, calibrator.hpp:66-91: mins then difs).
 * params may be NULL to ask for the count. */
int gsx_searcher_params(const gsx_searcher *s, float *params, int32_t *count);

/* ---- exact ground truth (no reference counterpart; replaces brute force in examples/main.py) -- */

/* Exact k nearest neighbours of nq queries over N base rows by brute force on the tensor cores,
 * for recall checks: bf16 tensor-core scores (one pass when every input is exactly representable
 * in bf16, else a three-pass hi/lo split), 32 candidates per query per base chunk, then exact fp64
 * rescoring; ids/dis are nq x k sorted by (distance, id).  Device buffers (fp32, row-major);
 * d <= 128, k <= 16; ip = 1 for inner product (distance -q.x), else squared L2.  *exact_inputs (may
 * be NULL) reports whether the single exact pass was used.  Synchronises `stream`. */
int gsx_knn_exact(const float *d_base, int64_t N, int32_t d, const float *d_queries, int32_t nq, int32_t k,
                  int32_t ip, int32_t *d_ids, float *d_dis, int32_t *exact_inputs, void *stream);

/* ---- graph construction ------------------------------------------------------------------- */

/* Builds an NSG (use_ssg = 0) or SSG (use_ssg = 1) graph over N fp32 rows (host memory, row-major)
 * on the GPU; replaces NSG::Build (glass/nsg/nsg.hpp:55-104) behind Index("NSG" | "SSG", metric,
 * "FP32", R, L).build(data) (python/bindings.cc:60-87).  The graph is R wide with one entry point
 * (the row nearest to the centroid); L = 0 means R + 32 and C = R + 100, as in the reference
 * (nsg.hpp:46-53).  Its kNN graph holds the exact knn_k (<= 64; the reference uses 64) nearest rows
 * by fp32 squared L2 (tensor-core candidates, brute force where they may fall short) in place of
 * NN-Descent; reverse links are merged per node in one step instead of one lock-protected
 * insertion at a time, so the build is deterministic.  Squared
 * L2 over the fp32 rows (the reference's NSG is L2-only); d <= 128, R <= 256.  knng_out (may be
 * NULL) receives the N x min(knn_k, N - 1) kNN graph; seconds (may be NULL) receives 7 values: kNN
 * graph + entry point, link, reverse links, connectivity, total, the number of nodes attached by
 * the connectivity pass, and the number of kNN rows redone by brute force (rows whose tensor-core
 * candidate lists may have cut their neighbours short). */
int gsx_graph_build_nsg(const float *data, int64_t N, int32_t d, int32_t R, int32_t L, int32_t use_ssg,
                        int32_t knn_k, int32_t *knng_out, double *seconds, gsx_graph **out);

/* ---- serving: continuous batching over a resident index (no reference counterpart) -------- */

typedef struct gsx_server gsx_server;

/* Starts a request loop on searcher s: a dispatcher thread admits queued requests (oldest first)
 * into an arena of max_queries_in_flight device query slots, capped so that the arena takes at
 * most half of the free device memory, and launches each admitted group (the oldest requests, up
 * to max_queries_in_flight / (2 * streams) queries, on one contiguous slot range) on one of
 * `streams` (1..32) CUDA streams, so that groups overlap on the device.  kmax / efmax bound the
 * per-request k and ef.
 * While a server runs, the searcher must not be used directly. */
int gsx_server_create(gsx_searcher *s, int32_t max_queries_in_flight, int32_t kmax, int32_t efmax, int32_t streams,
                      gsx_server **out);
/* Number of query slots actually admitted by free device memory. */
int gsx_server_capacity(const gsx_server *sv, int32_t *slots);
/* Queues nq queries (host memory, copied) with their k and ef; returns a ticket at once. */
int gsx_server_submit(gsx_server *sv, const float *queries, int32_t nq, int32_t k, int32_t ef, uint64_t *ticket);
/* Waits at most timeout_ms for a ticket; on success writes ids/dis (nq*k each, may be NULL) and the
 * submit-to-completion latency, and forgets the ticket.  GSX_ERR_TIMEOUT leaves it pending. */
int gsx_server_wait(gsx_server *sv, uint64_t ticket, int32_t timeout_ms, int32_t *ids, float *dis, double *latency_ms);
/* Completed queries, queued requests, groups on the device. */
int gsx_server_stats(gsx_server *sv, int64_t *completed_queries, int32_t *queued_requests, int32_t *running_groups);
/* Open-loop Poisson load for measuring a server (no reference counterpart): n_requests requests
 * arrive at exponential gaps of mean 1/request_rate s; each has a log-uniform number of queries in
 * [size_min, size_max] (consecutive rows of `queries`, nq_pool rows), a k drawn from ks[0..nk) and
 * an ef from efs[0..nef).  Requests are submitted on schedule whether or not earlier ones have
 * finished.  Writes every request's submit-to-completion latency (ms), its size (may be NULL) and
 * the wall time of the whole run. */
int gsx_server_drive_poisson(gsx_server *sv, const float *queries, int32_t nq_pool, int32_t n_requests,
                             double request_rate, int32_t size_min, int32_t size_max, const int32_t *ks, int32_t nk,
                             const int32_t *efs, int32_t nef, uint64_t seed, double *latency_ms, int32_t *sizes,
                             double *wall_s);
/* Finishes every queued request, then stops the loop and frees its memory. */
void gsx_server_destroy(gsx_server *sv);

#ifdef __cplusplus
}
#endif

#endif /* GLASS_GB300_H */
