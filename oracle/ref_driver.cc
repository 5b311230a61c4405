// Test-infrastructure driver for the UNMODIFIED reference (zilliztech/pyglass).
//
// This file is ours; it only #includes the reference's header-only sources where they lie
// (include path given by oracle/Makefile) and re-exports the pieces the parity suite needs as a
// plain C ABI, so that Python (ctypes) can run the reference searcher, quantizers and graph
// builders on the same inputs as the GPU path.  It is never linked into the product.
//
// Reference entry points wrapped here:
//   glass::create_searcher            glass/searcher/graph_searcher.hpp:256-391
//   GraphSearcherBase::SetData/Search/SearchBatch/SetEf/GetLastSearchAvgDistCmps
//                                      glass/searcher/searcher_base.hpp:7-19
//   glass::create_hnsw / create_nsg    glass/hnsw/hnsw.hpp:74-133, glass/nsg/nsg.hpp:411-434
//   Graph<int>::load/save             glass/graph.hpp:106-153 (load in every format, :121-245)
//   Quantizer train/add/get_computer   glass/quant/*.hpp
#include <omp.h>

#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "glass/hnsw/hnsw.hpp"
#include "glass/nsg/nsg.hpp"
#include "glass/searcher/graph_searcher.hpp"

namespace {

struct RefSearcher {
    std::unique_ptr<glass::GraphSearcherBase> s;
};

// Runs `fn` with a freshly trained quantizer of the requested kind.
template <typename Fn>
int with_quant(const std::string &quant, const std::string &metric, int d, Fn &&fn) {
    using glass::Metric;
    bool l2 = metric != "IP";
    if (quant == "SQ8U") {
        if (l2) { glass::SQ8QuantizerUniform<Metric::L2> q(d); return fn(q); }
        glass::SQ8QuantizerUniform<Metric::IP> q(d); return fn(q);
    }
    if (quant == "SQ8") {
        if (l2) { glass::SQ8Quantizer<Metric::L2> q(d); return fn(q); }
        glass::SQ8Quantizer<Metric::IP> q(d); return fn(q);
    }
    if (quant == "SQ4UA") {
        if (l2) { glass::SQ4QuantizerUniformAsym<Metric::L2> q(d); return fn(q); }
        glass::SQ4QuantizerUniformAsym<Metric::IP> q(d); return fn(q);
    }
    if (quant == "SQ1") {
        if (l2) { glass::SQ1Quantizer<Metric::L2> q(d); return fn(q); }
        glass::SQ1Quantizer<Metric::IP> q(d); return fn(q);
    }
    if (quant == "SQ2U") {
        if (l2) { glass::SQ2QuantizerUniform<Metric::L2> q(d); return fn(q); }
        glass::SQ2QuantizerUniform<Metric::IP> q(d); return fn(q);
    }
    if (quant == "SQ4U") {
        if (l2) { glass::SQ4QuantizerUniform<Metric::L2> q(d); return fn(q); }
        glass::SQ4QuantizerUniform<Metric::IP> q(d); return fn(q);
    }
    if (quant == "E5M2") {
        if (l2) { glass::E5M2Quantizer<Metric::L2> q(d); return fn(q); }
        glass::E5M2Quantizer<Metric::IP> q(d); return fn(q);
    }
    if (quant == "FP32") {
        if (l2) { glass::FP32Quantizer<Metric::L2> q(d); return fn(q); }
        glass::FP32Quantizer<Metric::IP> q(d); return fn(q);
    }
    if (quant == "FP16") {
        if (l2) { glass::FP16Quantizer<Metric::L2> q(d); return fn(q); }
        glass::FP16Quantizer<Metric::IP> q(d); return fn(q);
    }
    if (quant == "BF16") {
        if (l2) { glass::BF16Quantizer<Metric::L2> q(d); return fn(q); }
        glass::BF16Quantizer<Metric::IP> q(d); return fn(q);
    }
    return -1;
}

template <typename Q>
void calib_params(const Q &q, float *params) {
    params[0] = params[1] = 0.0f;
    if constexpr (requires { q.calibrator.dif; }) {
        params[0] = q.calibrator.min;
        params[1] = q.calibrator.dif;
    } else if constexpr (requires { q.calibrator.max; }) {
        params[0] = q.calibrator.max;
    } else if constexpr (requires { q.calibrator.difs; }) {  // per-dimension: mins, then difs (dalign each)
        const size_t n = q.calibrator.mins.size();
        std::memcpy(params, q.calibrator.mins.data(), n * sizeof(float));
        std::memcpy(params + n, q.calibrator.difs.data(), n * sizeof(float));
    }
}

}  // namespace

extern "C" {

void ref_set_num_threads(int n) { omp_set_num_threads(n); }

// Builds a graph with the reference CPU builder and saves it in the glass format.
double ref_build_graph(const char *index_type, const float *data, int n, int d, const char *metric,
                       const char *quant, int R, int L, const char *out_path) {
    std::unique_ptr<glass::Builder> b;
    std::string t(index_type);
    if (t == "HNSW") b = glass::create_hnsw(metric, quant, R, L);
    else if (t == "NSG") b = glass::create_nsg(quant, R, L, false);
    else if (t == "SSG") b = glass::create_nsg(quant, R, L, true);
    if (!b) return -1.0;
    auto g = b->Build(data, n, d);
    g.save(out_path);
    return b->GetConstructionTime();
}

void *ref_searcher_create(const char *graph_path, const float *data, int n, int d, const char *metric,
                          const char *quant, const char *refine) {
    glass::Graph<int> g;
    g.load(graph_path, "glass");
    auto *r = new RefSearcher;
    r->s = glass::create_searcher(std::move(g), metric, quant, refine);
    if (!r->s) { delete r; return nullptr; }
    r->s->SetData(data, n, d);
    return r;
}

void ref_searcher_set_ef(void *h, int ef) { ((RefSearcher *)h)->s->SetEf(ef); }

void ref_searcher_search(void *h, const float *q, int k, int *ids, float *dis) {
    ((RefSearcher *)h)->s->Search(q, k, ids, dis);
}

void ref_searcher_search_batch(void *h, const float *qs, int nq, int k, int *ids, float *dis) {
    ((RefSearcher *)h)->s->SearchBatch(qs, nq, k, ids, dis);
}

double ref_searcher_dist_cmps(void *h) { return ((RefSearcher *)h)->s->GetLastSearchAvgDistCmps(); }

void ref_searcher_destroy(void *h) { delete (RefSearcher *)h; }

// The reference NSG's link step for every node (the first loop of NSG::link, nsg.hpp:166-176:
// search_on_graph, then sync_prune) over a given kNN graph and entry point, with the FP32
// quantizer's symmetric distances; writes the pruned forward graph (before add_reverse_links).
int ref_nsg_link(const float *data, int n, int d, int R, int L, int ssg, const int *knng, int K, int ep, int *out) {
    using Q = glass::FP32Quantizer<glass::Metric::L2>;
    glass::NSG<Q> nsg(R, L, ssg != 0);
    nsg.nb = n;
    nsg.d = d;
    nsg.ep = ep;
    Q quant(d);
    quant.train(data, n);
    quant.add(data, n);
    auto computer = quant.get_sym_computer();
    glass::Graph<int> kg(n, K);
    std::memcpy(kg.data, knng, (size_t)n * K * 4);
    glass::Graph<glass::Node> tmp(n, R);
#pragma omp parallel for schedule(dynamic)
    for (int i = 0; i < n; ++i) {
        std::vector<glass::Node> fullset;
        glass::LinearPool<float> pool(n, nsg.L, nsg.L);
        nsg.search_on_graph(computer, i, kg, ep, pool, fullset);
        nsg.sync_prune(computer, i, pool, fullset, kg, tmp);
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < R; ++j) out[(size_t)i * R + j] = tmp.at(i, j).id;
    return 0;
}

// The reference NSG's entry point (NSG::Init, nsg.hpp:106-127: the row nearest the float centroid
// by the FP32 quantizer's distance).
int ref_nsg_init(const float *data, int n, int d) {
    using Q = glass::FP32Quantizer<glass::Metric::L2>;
    glass::NSG<Q> nsg(32, 0, false);
    nsg.nb = n;
    nsg.d = d;
    Q quant(d);
    quant.train(data, n);
    quant.add(data, n);
    nsg.Init(quant, data);
    return nsg.ep;
}

// A graph read by the reference's own loader (Graph<int>::load, glass/graph.hpp:121-135, with its
// glass / diskann / hnswlib / nsg readers), for comparison with the product's loaders.
void *ref_graph_open(const char *path, const char *format) {
    auto *g = new glass::Graph<int>;
    g->load(path, format);
    return g;
}

void ref_graph_info(void *h, int *N, int *K, int *nep) {
    auto *g = (glass::Graph<int> *)h;
    *N = g->N;
    *K = g->K;
    *nep = (int)g->eps.size();
}

void ref_graph_copy(void *h, int *eps, int *adj) {
    auto *g = (glass::Graph<int> *)h;
    std::memcpy(eps, g->eps.data(), g->eps.size() * 4);
    std::memcpy(adj, g->data, (size_t)g->N * g->K * 4);
}

void ref_graph_close(void *h) { delete (glass::Graph<int> *)h; }

// Code size in bytes of one encoded row for quantizer `quant` at dimension d.
int ref_code_size(const char *quant, const char *metric, int d) {
    return with_quant(quant, metric, d, [](auto &q) { return (int)q.code_size(); });
}

// Trains the quantizer on data[n*d] exactly as SetData does, writes all n codes (n*code_size bytes)
// and the calibrator parameters (min,dif for affine; max for symmetric).
int ref_encode(const char *quant, const char *metric, const float *data, int n, int d, char *codes,
               float *params) {
    return with_quant(quant, metric, d, [&](auto &q) {
        q.train(data, n);
        q.add(data, n);
        for (int i = 0; i < n; ++i) std::memcpy(codes + (int64_t)i * q.code_size(), q.get_code(i), q.code_size());
        calib_params(q, params);
        return 0;
    });
}

// Trains on data like SetData, then evaluates the per-query distance computer of `quant` for
// every (query, id) pair: out[qi*m + j] = computer_qi(ids[qi*m + j]).  Also returns the encoded
// query rows (the computer's private query buffer, code_size bytes each; float queries for
// E5M2/FP32 are returned as their dim_align*4 bytes).
int ref_query_distances(const char *quant, const char *metric, const float *data, int n, int d,
                        const float *queries, int nq, const int *ids, int m, double *out, char *qcodes,
                        int qcode_stride) {
    return with_quant(quant, metric, d, [&](auto &q) {
        q.train(data, n);
        q.add(data, n);
        for (int qi = 0; qi < nq; ++qi) {
            auto comp = q.get_computer(queries + (int64_t)qi * d);
            for (int j = 0; j < m; ++j) out[(int64_t)qi * m + j] = (double)comp(ids[(int64_t)qi * m + j]);
            if (qcodes) {
                using X = typename std::decay_t<decltype(comp)>::X;
                int nbytes = (int)(q.dim_align() * sizeof(X));
                // 1-byte query codes are code_size() bytes, except SQ4UA's, which are one byte per
                // dimension (sq4ua_quant.hpp:52-58)
                using Q = std::decay_t<decltype(q)>;
                constexpr bool asym = std::is_same_v<Q, glass::SQ4QuantizerUniformAsym<glass::Metric::L2>> ||
                                      std::is_same_v<Q, glass::SQ4QuantizerUniformAsym<glass::Metric::IP>>;
                if constexpr (sizeof(X) == 1 && !asym) nbytes = q.code_size();
                std::memcpy(qcodes + (int64_t)qi * qcode_stride, comp.q, std::min(nbytes, qcode_stride));
            }
        }
        return 0;
    });
}

}  // extern "C"
