// Python module `pyglass_gb300._glass`: the reference's glass.Graph / glass.Searcher surface
// (python/bindings.cc:40-154, 239-269) over the C ABI of libglass_gb300 (include/glass_gb300.h).
// Argument names, defaults and return shapes are the reference's; failures raise RuntimeError
// with the library's message instead of printing and continuing.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>

#include "../../../include/glass_gb300.h"

namespace py = pybind11;

namespace {

void check(int rc) {
    if (rc != GSX_OK) throw std::runtime_error(std::string("glass-gb300: ") + gsx_last_error());
}

using f32arr = py::array_t<float, py::array::c_style | py::array::forcecast>;
using i32arr = py::array_t<int32_t, py::array::c_style | py::array::forcecast>;

// get_input_array_shapes (python/bindings.cc:20-36), with the shape error actually raised.
void shape_of(const py::buffer_info &b, size_t *rows, size_t *features) {
    if (b.ndim == 2) {
        *rows = (size_t)b.shape[0];
        *features = (size_t)b.shape[1];
    } else if (b.ndim == 1) {
        *rows = 1;
        *features = (size_t)b.shape[0];
    } else {
        throw std::runtime_error("Input vector data wrong shape. Data must be a 1D or 2D array.");
    }
}

struct Graph {
    gsx_graph *g = nullptr;

    Graph() = default;
    Graph(const std::string &filename, const std::string &format) { check(gsx_graph_load(filename.c_str(), format.c_str(), &g)); }
    ~Graph() {
        if (g) gsx_graph_destroy(g);
    }
    Graph(const Graph &) = delete;
    Graph &operator=(const Graph &) = delete;

    void save(const std::string &filename) {
        if (!g) throw std::runtime_error("glass-gb300: empty graph");
        check(gsx_graph_save(g, filename.c_str()));
    }
    void load(const std::string &filename, const std::string &format) {
        gsx_graph *n = nullptr;
        check(gsx_graph_load(filename.c_str(), format.c_str(), &n));
        if (g) gsx_graph_destroy(g);
        g = n;
    }
    py::tuple info() const {
        int32_t N = 0, K = 0, nep = 0, h = 0;
        if (g) check(gsx_graph_info(g, &N, &K, &nep, &h));
        return py::make_tuple(N, K, nep, (bool)h);
    }
};

Graph *graph_from_adjacency(i32arr adj, i32arr eps) {
    auto b = adj.request();
    if (b.ndim != 2) throw std::runtime_error("adjacency must be N x K");
    auto *G = new Graph;
    check(gsx_graph_create(adj.data(), (int32_t)b.shape[0], (int32_t)b.shape[1], eps.data(), (int32_t)eps.size(), &G->g));
    return G;
}

// A captured device batch (gsx_searcher_capture_batch); the Python object keeps its searcher alive.
struct BatchGraph {
    gsx_batch_graph *g = nullptr;
    explicit BatchGraph(gsx_batch_graph *h) : g(h) {}
    ~BatchGraph() { close(); }
    BatchGraph(const BatchGraph &) = delete;
    BatchGraph &operator=(const BatchGraph &) = delete;
    gsx_batch_graph *live() const {
        if (!g) throw std::runtime_error("glass-gb300: the batch graph is closed");
        return g;
    }
    void launch(uintptr_t stream) {
        gsx_batch_graph *h = live();
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_batch_graph_launch(h, (void *)stream);
        }
        check(rc);
    }
    unsigned overflow_count() {
        gsx_batch_graph *h = live();
        uint32_t c = 0;
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_batch_graph_overflow_count(h, &c);
        }
        check(rc);
        return c;
    }
    void close() {
        if (g) {
            py::gil_scoped_release l;
            gsx_batch_graph_destroy(g);
        }
        g = nullptr;
    }
};

struct Searcher {
    gsx_searcher *s = nullptr;
    int32_t dim = 0;

    Searcher(Graph &graph, py::object input, const std::string &metric, const std::string &quantizer,
             const std::string &refine_quant, int device) {
        if (!graph.g) throw std::runtime_error("glass-gb300: graph is empty");
        check(gsx_searcher_create(graph.g, metric.c_str(), quantizer.c_str(), refine_quant.c_str(), device, &s));
        f32arr items(input);
        size_t rows, features;
        shape_of(items.request(), &rows, &features);
        dim = (int32_t)features;
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_set_data(s, items.data(), (int32_t)rows, (int32_t)features);
        }
        check(rc);
    }
    ~Searcher() {
        if (s) gsx_searcher_destroy(s);
    }
    Searcher(const Searcher &) = delete;
    Searcher &operator=(const Searcher &) = delete;

    void check_dim(size_t features) const {
        if ((int32_t)features != dim)
            throw std::runtime_error("glass-gb300: query dimension " + std::to_string(features) + " != data dimension " +
                                     std::to_string(dim));
    }

    py::tuple search(py::object query, int k) {
        f32arr items(query);
        size_t rows, features;
        shape_of(items.request(), &rows, &features);
        check_dim(features);
        if (k <= 0) throw std::runtime_error("glass-gb300: k must be positive");
        py::array_t<int32_t> ids((py::ssize_t)k);
        py::array_t<float> dis((py::ssize_t)k);
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_search(s, items.data(), k, ids.mutable_data(), dis.mutable_data());
        }
        check(rc);
        return py::make_tuple(ids, dis);
    }

    py::tuple batch_search(py::object query, int k, int num_threads) {
        (void)num_threads;  // the OpenMP thread count has no GPU meaning
        f32arr items(query);
        size_t nq, features;
        shape_of(items.request(), &nq, &features);
        check_dim(features);
        if (k <= 0) throw std::runtime_error("glass-gb300: k must be positive");
        py::array_t<int32_t> ids({(py::ssize_t)nq, (py::ssize_t)k});
        py::array_t<float> dis({(py::ssize_t)nq, (py::ssize_t)k});
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_search_batch(s, items.data(), (int32_t)nq, k, ids.mutable_data(), dis.mutable_data());
        }
        check(rc);
        return py::make_tuple(ids, dis);
    }

    // Batched search with per-query ef and k (the batched/persistent form); rows of the outputs
    // have max(k) entries, padded with -1 / inf past each query's k.
    py::tuple batch_search_mixed(py::object query, py::object ef, py::object ks) {
        f32arr items(query);
        size_t nq, features;
        shape_of(items.request(), &nq, &features);
        check_dim(features);
        i32arr efa(ef), ka(ks);
        if ((size_t)efa.size() != nq || (size_t)ka.size() != nq)
            throw std::runtime_error("glass-gb300: ef and k need one entry per query");
        int32_t kmax = 1;
        for (size_t i = 0; i < nq; ++i) kmax = std::max(kmax, ka.data()[i]);
        py::array_t<int32_t> ids({(py::ssize_t)nq, (py::ssize_t)kmax});
        py::array_t<float> dis({(py::ssize_t)nq, (py::ssize_t)kmax});
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_search_batch_mixed(s, items.data(), (int32_t)nq, kmax, efa.data(), ka.data(), kmax,
                                                 ids.mutable_data(), dis.mutable_data());
        }
        check(rc);
        return py::make_tuple(ids, dis);
    }

    // Device-resident batch: pointers are integers (e.g. torch tensor data_ptr()); enqueued on
    // `stream` (0 = the searcher's own stream) without synchronising.
    void batch_search_device(uintptr_t queries, int nq, int k, uintptr_t ids, uintptr_t dis, uintptr_t ef_per,
                             uintptr_t k_per, int kmax, uintptr_t cmps, uintptr_t expansions, uintptr_t stream) {
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_search_batch_device(s, (const float *)queries, nq, k, (const int32_t *)ef_per,
                                                  (const int32_t *)k_per, kmax, (int32_t *)ids, (float *)dis,
                                                  (int32_t *)cmps, (int32_t *)expansions, (void *)stream);
        }
        check(rc);
    }

    unsigned overflow_count() {
        uint32_t c = 0;
        check(gsx_searcher_overflow_count(s, &c));
        return c;
    }

    BatchGraph *capture_batch_device(uintptr_t queries, int nq, int k, uintptr_t ids, uintptr_t dis, uintptr_t ef_per,
                                     uintptr_t k_per, int kmax, uintptr_t cmps, uintptr_t expansions) {
        gsx_batch_graph *h = nullptr;
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_capture_batch(s, (const float *)queries, nq, k, (const int32_t *)ef_per,
                                            (const int32_t *)k_per, kmax, (int32_t *)ids, (float *)dis,
                                            (int32_t *)cmps, (int32_t *)expansions, &h);
        }
        check(rc);
        return new BatchGraph(h);
    }

    py::array_t<double> distances(py::object query, py::object ids, bool refine) {
        f32arr q(query);
        i32arr id(ids);
        size_t nq, features;
        shape_of(q.request(), &nq, &features);
        check_dim(features);
        auto ib = id.request();
        const size_t m = ib.ndim == 2 ? (size_t)ib.shape[1] : (size_t)ib.shape[0];
        if ((size_t)id.size() != nq * m) throw std::runtime_error("glass-gb300: ids must be nq x m");
        py::array_t<double> out({(py::ssize_t)nq, (py::ssize_t)m});
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_distances(s, q.data(), (int32_t)nq, id.data(), (int32_t)m, refine ? 1 : 0, out.mutable_data());
        }
        check(rc);
        return out;
    }

    // (code size in bytes, calibrator parameters) of the search quantizer
    py::tuple calibration() {
        int32_t cs = 0, np_ = 0;
        float p[2];
        check(gsx_searcher_codes(s, nullptr, p, &cs));
        check(gsx_searcher_params(s, nullptr, &np_));
        std::vector<float> v((size_t)np_);
        check(gsx_searcher_params(s, v.data(), &np_));
        py::tuple t((size_t)np_);
        for (int32_t i = 0; i < np_; ++i) t[(size_t)i] = v[(size_t)i];
        return py::make_tuple(cs, t);
    }

    py::array_t<uint8_t> code_rows(int n) {
        int32_t cs = 0;
        float p[2];
        check(gsx_searcher_codes(s, nullptr, p, &cs));
        py::array_t<uint8_t> out({(py::ssize_t)n, (py::ssize_t)cs});
        check(gsx_searcher_codes(s, out.mutable_data(), p, &cs));
        return out;
    }

    void set_ef(int ef) { check(gsx_searcher_set_ef(s, ef)); }
    int get_ef() const {
        int32_t e = 0;
        check(gsx_searcher_get_ef(s, &e));
        return e;
    }
    void optimize(int num_threads) {
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_searcher_optimize(s, num_threads);
        }
        check(rc);
    }
    double get_last_search_avg_dist_cmps() const {
        double v = 0;
        check(gsx_searcher_get_last_search_avg_dist_cmps(s, &v));
        return v;
    }
    py::dict get_tuning() const {
        gsx_tuning t;
        check(gsx_searcher_get_tuning(s, &t));
        py::dict d;
        d["warps_per_block"] = t.warps_per_block;
        d["table_bits"] = t.table_bits;
        d["lanes_per_row"] = t.lanes_per_row;
        d["prefetch"] = t.prefetch;
        d["spill_bits"] = t.spill_bits;
        return d;
    }
    void set_tuning(int warps_per_block, int table_bits, int lanes_per_row, int prefetch, int spill_bits) {
        gsx_tuning t{warps_per_block, table_bits, lanes_per_row, prefetch, spill_bits};
        check(gsx_searcher_set_tuning(s, &t));
    }
    py::tuple memory() const {
        size_t ib = 0, pq = 0;
        check(gsx_searcher_memory(s, &ib, &pq));
        return py::make_tuple(ib, pq);
    }
};

// The serving loop (gsx_server_*): submit returns a ticket, wait returns (ids, dis, latency_ms).
// Index (python/bindings.cc:60-87): "NSG" and "SSG" over FP32 rows build on the GPU
// (gsx_graph_build_nsg); other index types and build quantizers raise.
struct Index {
    std::string type;
    int R = 32, L = 0;
    double secs[7] = {0, 0, 0, 0, 0, 0, 0};
    py::object knng = py::none();

    Index(const std::string &index_type, const std::string &metric, const std::string &quant, int R_, int L_)
        : type(index_type), R(R_), L(L_) {
        if (index_type != "NSG" && index_type != "SSG")
            throw std::runtime_error("glass-gb300: index type " + index_type +
                                     " is not built on the GPU (NSG and SSG are)");
        if (metric != "L2" && metric != "IP")
            throw std::runtime_error("glass-gb300: unknown metric " + metric);
        if (quant != "FP32")
            throw std::runtime_error("glass-gb300: the GPU graph build computes FP32 distances (quant \"FP32\")");
    }
    Graph *build(py::object input, int knn_k, bool keep_knn) {
        f32arr items(input);
        size_t rows = 0, features = 0;
        shape_of(items.request(), &rows, &features);
        const int kk = (int)std::min<size_t>((size_t)knn_k, rows > 1 ? rows - 1 : 1);
        py::array_t<int32_t> kn;
        int32_t *kp = nullptr;
        if (keep_knn) {
            kn = py::array_t<int32_t>({(py::ssize_t)rows, (py::ssize_t)kk});
            kp = kn.mutable_data();
        }
        auto *G = new Graph;
        int rc;
        {
            py::gil_scoped_release rel;
            rc = gsx_graph_build_nsg(items.data(), (int64_t)rows, (int32_t)features, R, L, type == "SSG" ? 1 : 0, knn_k, kp,
                                     secs, &G->g);
        }
        if (rc != GSX_OK) {
            delete G;
            check(rc);
        }
        knng = keep_knn ? py::object(kn) : py::object(py::none());
        return G;
    }
    double get_construction_time() const { return secs[4]; }
    py::dict stages() const {
        py::dict d;
        d["knn_graph_s"] = secs[0];
        d["link_s"] = secs[1];
        d["reverse_s"] = secs[2];
        d["connect_s"] = secs[3];
        d["total_s"] = secs[4];
        d["attached"] = (int64_t)secs[5];
        d["knn_rows_rechecked"] = (int64_t)secs[6];
        return d;
    }
};

// build_graph (python/bindings.cc:231-237)
double build_graph(const std::string &index_type, py::object input, const std::string &graph_file,
                   const std::string &metric, const std::string &quant, int R, int L) {
    Index index(index_type, metric, quant, R, L);
    std::unique_ptr<Graph> g(index.build(input, 64, false));
    g->save(graph_file);
    return index.get_construction_time();
}

struct Server {
    gsx_server *sv = nullptr;
    int32_t dim = 0;
    py::object keep;  // the Searcher must outlive the server

    Server(py::object searcher, int capacity, int kmax, int efmax, int streams) {
        Searcher &s = searcher.cast<Searcher &>();
        keep = searcher;
        dim = s.dim;
        check(gsx_server_create(s.s, capacity, kmax, efmax, streams, &sv));
    }
    ~Server() { close(); }
    void close() {
        if (sv) {
            py::gil_scoped_release l;
            gsx_server_destroy(sv);
            sv = nullptr;
        }
    }
    uint64_t submit(py::object query, int k, int ef) {
        if (!sv) throw std::runtime_error("glass-gb300: server closed");
        f32arr items(query);
        size_t nq, features;
        shape_of(items.request(), &nq, &features);
        if ((int32_t)features != dim) throw std::runtime_error("glass-gb300: query dimension mismatch");
        uint64_t t = 0;
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_server_submit(sv, items.data(), (int32_t)nq, k, ef, &t);
        }
        check(rc);
        return t;
    }
    py::tuple wait(uint64_t ticket, int nq, int k, int timeout_ms) {
        if (!sv) throw std::runtime_error("glass-gb300: server closed");
        py::array_t<int32_t> ids({(py::ssize_t)nq, (py::ssize_t)k});
        py::array_t<float> dis({(py::ssize_t)nq, (py::ssize_t)k});
        double lat = 0;
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_server_wait(sv, ticket, timeout_ms, ids.mutable_data(), dis.mutable_data(), &lat);
        }
        check(rc);
        return py::make_tuple(ids, dis, lat);
    }
    int capacity() const {
        int32_t c = 0;
        check(gsx_server_capacity(sv, &c));
        return c;
    }
    // Open-loop Poisson load; returns (latency_ms[n], sizes[n], wall_s).
    py::tuple drive_poisson(py::object queries, int n_requests, double request_rate, int size_min, int size_max,
                            py::object ks, py::object efs, uint64_t seed) {
        f32arr q(queries);
        i32arr k(ks), e(efs);
        size_t nq, features;
        shape_of(q.request(), &nq, &features);
        if ((int32_t)features != dim) throw std::runtime_error("glass-gb300: query dimension mismatch");
        py::array_t<double> lat((py::ssize_t)n_requests);
        py::array_t<int32_t> sz((py::ssize_t)n_requests);
        double wall = 0;
        int rc;
        {
            py::gil_scoped_release l;
            rc = gsx_server_drive_poisson(sv, q.data(), (int32_t)nq, n_requests, request_rate, size_min, size_max,
                                          k.data(), (int32_t)k.size(), e.data(), (int32_t)e.size(), seed,
                                          lat.mutable_data(), sz.mutable_data(), &wall);
        }
        check(rc);
        return py::make_tuple(lat, sz, wall);
    }
    py::tuple stats() {
        int64_t done = 0;
        int32_t q = 0, r = 0;
        check(gsx_server_stats(sv, &done, &q, &r));
        return py::make_tuple(done, q, r);
    }
};

}  // namespace

PYBIND11_MODULE(_glass, m) {
    m.doc() = "GB300 graph search with the glass.Searcher / glass.Graph API";
    // set_num_threads (bindings.cc:38): OpenMP has no role on the GPU path; accepted for parity.
    m.def("set_num_threads", [](int) {}, py::arg("num_threads"));
    m.def("version", []() { return std::string(gsx_version()); });
    m.def("device_count", []() { return gsx_device_count(); });
    // Exact kNN ground truth on device buffers (integer pointers, e.g. torch data_ptr()); returns
    // True when the single exact bf16 pass was used.
    m.def(
        "knn_exact",
        [](uintptr_t base, int64_t N, int d, uintptr_t queries, int nq, int k, bool ip, uintptr_t ids, uintptr_t dis,
           uintptr_t stream) {
            int32_t exact = 0;
            int rc;
            {
                py::gil_scoped_release l;
                rc = gsx_knn_exact((const float *)base, N, d, (const float *)queries, nq, k, ip ? 1 : 0, (int32_t *)ids,
                                   (float *)dis, &exact, (void *)stream);
            }
            check(rc);
            return exact != 0;
        },
        py::arg("base"), py::arg("N"), py::arg("d"), py::arg("queries"), py::arg("nq"), py::arg("k"),
        py::arg("ip") = false, py::arg("ids"), py::arg("dis"), py::arg("stream") = 0);

    py::class_<Graph>(m, "Graph")
        .def(py::init<>())
        .def(py::init<const std::string &, const std::string &>(), py::arg("filename"), py::arg("format") = "glass")
        .def("save", &Graph::save, py::arg("filename"))
        .def("load", &Graph::load, py::arg("filename"), py::arg("format") = "glass")
        .def("info", &Graph::info)
        .def_static("from_adjacency", &graph_from_adjacency, py::arg("adjacency"), py::arg("eps"),
                    py::return_value_policy::take_ownership);

    py::class_<Searcher>(m, "Searcher")
        .def(py::init<Graph &, py::object, const std::string &, const std::string &, const std::string &, int>(),
             py::arg("graph"), py::arg("data"), py::arg("metric"), py::arg("quantizer"), py::arg("refine_quant") = "",
             py::arg("device") = 0)
        .def("set_ef", &Searcher::set_ef, py::arg("ef"))
        .def("get_ef", &Searcher::get_ef)
        .def("search", &Searcher::search, py::arg("query"), py::arg("k"))
        .def("batch_search", &Searcher::batch_search, py::arg("query"), py::arg("k"), py::arg("num_threads") = 0)
        .def("batch_search_mixed", &Searcher::batch_search_mixed, py::arg("query"), py::arg("ef"), py::arg("k"))
        .def("batch_search_device", &Searcher::batch_search_device, py::arg("queries"), py::arg("nq"), py::arg("k"),
             py::arg("ids"), py::arg("dis"), py::arg("ef_per") = 0, py::arg("k_per") = 0, py::arg("kmax") = 0,
             py::arg("cmps") = 0, py::arg("expansions") = 0, py::arg("stream") = 0)
        .def("overflow_count", &Searcher::overflow_count)
        .def("capture_batch_device", &Searcher::capture_batch_device, py::arg("queries"), py::arg("nq"), py::arg("k"),
             py::arg("ids"), py::arg("dis"), py::arg("ef_per") = 0, py::arg("k_per") = 0, py::arg("kmax") = 0,
             py::arg("cmps") = 0, py::arg("expansions") = 0, py::return_value_policy::take_ownership,
             py::keep_alive<0, 1>())
        .def("optimize", &Searcher::optimize, py::arg("num_threads") = 0)
        .def("get_last_search_dist_cmps", &Searcher::get_last_search_avg_dist_cmps)
        .def("distances", &Searcher::distances, py::arg("query"), py::arg("ids"), py::arg("refine") = false)
        .def("code_rows", &Searcher::code_rows, py::arg("n"))
        .def("calibration", &Searcher::calibration)
        .def("get_tuning", &Searcher::get_tuning)
        .def("set_tuning", &Searcher::set_tuning, py::arg("warps_per_block") = 0, py::arg("table_bits") = 0,
             py::arg("lanes_per_row") = 0, py::arg("prefetch") = 2, py::arg("spill_bits") = 0)
        .def("memory", &Searcher::memory);

    py::class_<BatchGraph>(m, "BatchGraph")
        .def("launch", &BatchGraph::launch, py::arg("stream") = 0)
        .def("overflow_count", &BatchGraph::overflow_count)
        .def("close", &BatchGraph::close);

    py::class_<Index>(m, "Index")
        .def(py::init<const std::string &, const std::string &, const std::string &, int, int>(), py::arg("index_type"),
             py::arg("metric"), py::arg("quant") = "FP32", py::arg("R") = 32, py::arg("L") = 0)
        .def("build", &Index::build, py::arg("data"), py::arg("knn_k") = 64, py::arg("keep_knn") = false,
             py::return_value_policy::take_ownership)
        .def("get_construction_time", &Index::get_construction_time)
        .def("stages", &Index::stages)
        .def_readonly("knn_graph", &Index::knng);

    m.def("build_graph", &build_graph, py::arg("index_type"), py::arg("input"), py::arg("graph_file"),
          py::arg("metric"), py::arg("quant") = "FP32", py::arg("R") = 32, py::arg("L") = 0);

    py::class_<Server>(m, "Server")
        .def(py::init<py::object, int, int, int, int>(), py::arg("searcher"), py::arg("capacity") = 65536,
             py::arg("kmax") = 100, py::arg("efmax") = 256, py::arg("streams") = 16)
        .def("submit", &Server::submit, py::arg("query"), py::arg("k"), py::arg("ef"))
        .def("wait", &Server::wait, py::arg("ticket"), py::arg("nq"), py::arg("k"), py::arg("timeout_ms") = 60000)
        .def("capacity", &Server::capacity)
        .def("drive_poisson", &Server::drive_poisson, py::arg("queries"), py::arg("n_requests"),
             py::arg("request_rate"), py::arg("size_min"), py::arg("size_max"), py::arg("ks"), py::arg("efs"),
             py::arg("seed") = 1)
        .def("stats", &Server::stats)
        .def("close", &Server::close);
}
