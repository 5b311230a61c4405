// Reference-side adapter: the glass::GraphSearcherBase and glass::Builder implementations a pyglass
// tree adds to route its Searcher and NSG builds to libglass_gb300.  Header-only; compile it inside
// the pyglass tree (its glass/ headers on the include path) and link against libglass_gb300.so.
//
//   GpuGraphSearcher  implements GraphSearcherBase (glass/searcher/searcher_base.hpp:7-19) with the
//                     gsx_searcher_* C ABI; its constructor takes what create_searcher takes
//                     (glass/searcher/graph_searcher.hpp:256-391) and moves the graph in, HNSW
//                     upper levels included (glass/hnsw/HNSWInitializer.hpp:22-86).
//   GpuNSG            implements Builder (glass/builder.hpp) with gsx_graph_build_nsg, the GPU form
//                     of NSG::Build (glass/nsg/nsg.hpp:55-104) over FP32 rows.
//
// Errors throw std::runtime_error with the library's message (the reference prints and returns
// null instead).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "glass/builder.hpp"
#include "glass/graph.hpp"
#include "glass/searcher/searcher_base.hpp"
#include "glass_gb300.h"

namespace glass {

struct GpuGraphSearcher : GraphSearcherBase {
    gsx_searcher *s = nullptr;

    static void check(int rc) {
        if (rc != GSX_OK) throw std::runtime_error(gsx_last_error());
    }

    GpuGraphSearcher(Graph<int32_t> graph, const std::string &metric, const std::string &quant,
                     const std::string &refine, int device = 0) {
        gsx_graph *g = nullptr;
        check(gsx_graph_create(graph.data, graph.N, graph.K, graph.eps.data(), (int32_t)graph.eps.size(), &g));
        if (graph.initializer) {
            auto &in = *graph.initializer;
            std::vector<int32_t> lists;
            for (int32_t u = 0; u < graph.N; ++u)
                lists.insert(lists.end(), in.lists[u], in.lists[u] + (size_t)in.levels[u] * in.K);
            const int rc = gsx_graph_set_levels(g, in.K, in.ep, in.levels.data(), lists.data());
            if (rc != GSX_OK) {
                gsx_graph_destroy(g);
                check(rc);
            }
        }
        const int rc = gsx_searcher_create(g, metric.c_str(), quant.c_str(), refine.c_str(), device, &s);
        gsx_graph_destroy(g);
        check(rc);
    }
    ~GpuGraphSearcher() override { gsx_searcher_destroy(s); }
    GpuGraphSearcher(const GpuGraphSearcher &) = delete;
    GpuGraphSearcher &operator=(const GpuGraphSearcher &) = delete;

    void SetData(const float *data, int32_t n, int32_t dim) override { check(gsx_searcher_set_data(s, data, n, dim)); }
    void SetEf(int32_t ef) override { check(gsx_searcher_set_ef(s, ef)); }
    int32_t GetEf() const override {
        int32_t e = 0;
        check(gsx_searcher_get_ef(s, &e));
        return e;
    }
    void Optimize(int32_t num_threads = 0) override { check(gsx_searcher_optimize(s, num_threads)); }
    double GetLastSearchAvgDistCmps() const override {
        double v = 0;
        check(gsx_searcher_get_last_search_avg_dist_cmps(s, &v));
        return v;
    }
    void Search(const float *q, int32_t k, int32_t *dst, float *scores = nullptr) const override {
        check(gsx_searcher_search(s, q, k, dst, scores));
    }
    void SearchBatch(const float *qs, int32_t nq, int32_t k, int32_t *dst, float *scores = nullptr) const override {
        check(gsx_searcher_search_batch(s, qs, nq, k, dst, scores));
    }
};

struct GpuNSG : Builder {
    int R, L, ssg;
    double secs[7] = {0, 0, 0, 0, 0, 0, 0};
    GpuNSG(int R, int L, bool ssg) : R(R), L(L), ssg(ssg ? 1 : 0) {}
    Graph<int32_t> Build(const float *data, int32_t n, int32_t dim) override {
        gsx_graph *g = nullptr;
        if (gsx_graph_build_nsg(data, n, dim, R, L, ssg, 64, nullptr, secs, &g) != GSX_OK)
            throw std::runtime_error(gsx_last_error());
        int32_t N = 0, K = 0, nep = 0, h = 0;
        gsx_graph_info(g, &N, &K, &nep, &h);
        Graph<int32_t> out(N, K);
        gsx_graph_adjacency(g, out.data);
        out.eps.resize(nep);
        gsx_graph_eps(g, out.eps.data());
        gsx_graph_destroy(g);
        return out;
    }
    double GetConstructionTime() const override { return secs[4]; }
};

}  // namespace glass
