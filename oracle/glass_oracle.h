/*
 * glass_oracle.h - CPU restatement of the pyglass graph-search path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the parity suite compares the GPU path against,
 * and the CPU baseline that bench.py times on the host cores.  The product (pyglass_gb300) never
 * links, loads or calls it.
 *
 * Parity of this restatement is pinned against the unmodified reference (oracle/_ref, built from
 * the reference headers by oracle/Makefile) through the golden fixtures in tests/golden/.
 *
 * Every function cites the reference file:line whose behaviour it restates.
 */
#ifndef GLASS_ORACLE_H
#define GLASS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Quantizer kinds (names follow glass/quant/quant.hpp:25-43). */
enum { GO_FP32 = 0, GO_FP16 = 1, GO_BF16 = 2, GO_E5M2 = 3, GO_SQ8U = 4, GO_SQ8 = 5, GO_SQ4U = 7, GO_SQ4UA = 8,
       GO_SQ2U = 11, GO_SQ1 = 12 };
/* Metrics (glass/common.hpp:13-19). */
enum { GO_L2 = 0, GO_IP = 1 };

/* Row layout of a quantizer: dalign = ceil(d/align)*align, csize = dalign*nbits/8
 * (glass/storage/tensor.hpp:118-123 with the per-quantizer Quantizer<metric, align, nbits>). */
int go_layout(int kind, int d, int *dalign, int *csize);

/* Calibrator training as SetData runs it (sq8u_quant.hpp:240, sq4u_quant.hpp:307-309,
 * calibrator.hpp:481-514, quant/utils.hpp:584-603).  p[0],p[1] = (min, dif) for affine,
 * (max, 0) for symmetric, (0,0) for E5M2/FP32. */
void go_train(int kind, int metric, const float *data, int64_t n, int d, float *p);

/* Encodes n base rows into n*csize bytes (sq8u_quant.hpp:250-254, sq4u_quant.hpp:319-329,
 * e5m2_quant.hpp:390-394, fp32_quant.hpp:436-440).  Padding bytes are zero. */
void go_encode(int kind, int metric, const float *p, const float *data, int64_t n, int d, uint8_t *codes);

/* Encodes one query the way get_computer does (computer.hpp:54-63): SQ kinds write csize code
 * bytes; E5M2 and FP32 write dalign floats (query copied, zero padded).  Returns bytes written. */
int go_encode_query(int kind, int metric, const float *p, const float *q, int d, void *out);

/* Distance between an encoded query and one encoded row, as the reference's dist_func computes
 * it over dalign dimensions (helpa l2_s7_s7 / dot_s8_s8 / l2a_u4_u4 / l2_fp32_fp32 /
 * dot_fp32_fp32, glass L2SqrE5M2 / IPE5M2).  Integer kinds are exact; float kinds follow the
 * x86 AVX-512 accumulation order (16 lane accumulators, fused multiply-add, halving tree). */
double go_distance(int kind, int metric, const void *qenc, const uint8_t *code, int dalign);

/* out[qi*m+j] = go_distance(encoded query qi, row ids[qi*m+j]) for nq queries (OpenMP). */
void go_query_distances(int kind, int metric, const float *p, int d, const float *queries, int64_t nq,
                        const uint8_t *codes, const int32_t *ids, int m, double *out);

/* Glass-format graph (glass/graph.hpp:106-153, hnsw/HNSWInitializer.hpp:64-86). */
typedef struct {
    int32_t N, K;
    int32_t *adj;     /* N*K, -1 padded */
    int32_t nep;
    int32_t *eps;
    int32_t has_hnsw; /* upper levels present */
    int32_t hK, hep;  /* upper-level degree, entry point */
    int32_t *levels;  /* N */
    int64_t *loff;    /* N+1 offsets into lists (int32 units) */
    int32_t *lists;   /* concatenated level lists, levels[u]*hK entries for node u */
} go_graph;

int go_graph_load(const char *path, go_graph *g);
int go_graph_load_nsg(const char *path, go_graph *g);
void go_graph_free(go_graph *g);

/* Encoded index: graph + codes of the search quantizer (+ optional FP32 refine store). */
typedef struct {
    const go_graph *g;
    int kind, metric, d, dalign, csize;
    float p[2];
    const uint8_t *codes;
    int has_refine;         /* refiner present (refiner.hpp:15-111) */
    float refine_factor;    /* get_refine_factor (graph_searcher.hpp:227-238) */
    int r_dalign;
    const void *r_codes;    /* N*r_dalign rows of the refine quantizer: fp32, or fp16 when r_kind = GO_FP16 */
    int r_kind;             /* GO_FP32 or GO_FP16 (make_refiner, graph_searcher.hpp:240-254) */
    const float *pp;        /* SQ8: the calibrator's 2*dalign parameters (mins, then difs) */
} go_index;

/*
 * Batched search as Searcher.batch_search runs it (Refiner::SearchBatch refiner.hpp:72-90 ->
 * GraphSearcher::SearchBatch graph_searcher.hpp:143-159 -> SearchImpl2 :196-224).
 * single=1 selects Searcher.search semantics instead (refiner.hpp:45-70, graph_searcher.hpp:131-138:
 * the expansion limit becomes max(k, ef)).  ef_per_query / k_per_query may be NULL (uniform).
 * Outputs ids[nq*kmax], dis[nq*kmax] with row stride kmax = max k; entries past a query's k or
 * past the pool size are -1 / +inf.  cmps[nq] (may be NULL) gets per-query distance counts.
 * nthreads<=0 uses all OpenMP threads.
 */
void go_search(const go_index *ix, const float *queries, int64_t nq, int k, int ef, const int32_t *ef_per_query,
               const int32_t *k_per_query, int single, int32_t *ids, float *dis, int64_t *cmps, int nthreads);

/* NSG / SSG graph build (oracle/nsg_oracle.c).  knng_in (may be NULL: computed) is N x min(knn_k,
 * N - 1); ep_in < 0 computes the entry point.  Writes knng_out (same shape), graph_out (N x R, -1
 * padded), the entry point and the number of nodes attached for connectivity, and, when link_out is
 * not NULL, the pruned forward graph of the link step before reverse links (N x R, -1 padded).
 * 0 on success. */
int go_nsg_build(const float *x, int64_t N, int d, int R, int L, int ssg, int knn_k, const int32_t *knng_in,
                 int32_t ep_in, int32_t *knng_out, int32_t *graph_out, int32_t *ep_out, int32_t *n_attached,
                 int32_t *link_out);

#ifdef __cplusplus
}
#endif

#endif
