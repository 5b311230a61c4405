// Graph files and in-memory graphs: glass::Graph<int32_t> (glass/graph.hpp:26-379) and the HNSW
// upper levels (glass/hnsw/HNSWInitializer.hpp:64-86), held on the host until a searcher takes
// them to the device.
#include "gsx_host.h"

#include <cstdio>
#include <cstring>
#include <fstream>

namespace gsx {

namespace {

template <typename T>
bool rd(std::ifstream &f, T *p, size_t n = 1) {
    f.read(reinterpret_cast<char *>(p), (std::streamsize)(sizeof(T) * n));
    return (bool)f;
}

// Bytes from the read position to the end of the file.  Every size a header claims is checked
// against it before anything is allocated for it, so a malformed file is an error, never a huge
// allocation.
uint64_t bytes_left(std::ifstream &f) {
    const std::streamoff at = f.tellg();
    f.seekg(0, std::ios::end);
    const std::streamoff end = f.tellg();
    f.seekg(at);
    return (at >= 0 && end >= at) ? (uint64_t)(end - at) : 0;
}

int degree_unsupported(int32_t K) { return fail(GSX_ERR_UNSUPPORTED, "graph degree %d exceeds %d", K, kMaxDegree); }

int load_glass(const char *path, HostGraph &g) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(GSX_ERR_IO, "cannot open graph file '%s'", path);
    uint64_t left = bytes_left(f);
    int32_t nep = 0;
    if (!rd(f, &nep) || nep < 0 || (uint64_t)nep * 4 > left - 4)
        return fail(GSX_ERR_INVALID, "bad entry-point count in '%s'", path);
    g.eps.resize((size_t)nep);
    if (nep && !rd(f, g.eps.data(), (size_t)nep)) return fail(GSX_ERR_INVALID, "truncated graph file '%s'", path);
    if (!rd(f, &g.N) || !rd(f, &g.K) || g.N <= 0 || g.K <= 0)
        return fail(GSX_ERR_INVALID, "bad graph header in '%s'", path);
    if (g.K > kMaxDegree) return degree_unsupported(g.K);
    left = bytes_left(f);
    if ((uint64_t)g.N * (uint64_t)g.K * 4 > left) return fail(GSX_ERR_INVALID, "truncated adjacency in '%s'", path);
    g.adj.resize((size_t)g.N * (size_t)g.K);
    if (!rd(f, g.adj.data(), g.adj.size())) return fail(GSX_ERR_INVALID, "truncated adjacency in '%s'", path);
    left -= (uint64_t)g.adj.size() * 4;
    // optional HNSW upper levels (graph.hpp:282-285, HNSWInitializer.hpp:64-75)
    int32_t hn = 0;
    if (rd(f, &hn)) {
        if (!rd(f, &g.hK) || !rd(f, &g.hep) || hn != g.N || g.hK <= 0 || left < 12)
            return fail(GSX_ERR_INVALID, "bad HNSW level header in '%s'", path);
        left -= 12;
        g.has_hnsw = 1;
        g.levels.assign((size_t)g.N, 0);
        g.loff.assign((size_t)g.N + 1, 0);
        g.lists.clear();
        for (int32_t i = 0; i < g.N; ++i) {
            int32_t cur = 0;
            if (!rd(f, &cur) || cur < 0 || cur % g.hK != 0 || left < 4 || (uint64_t)cur * 4 > left - 4)
                return fail(GSX_ERR_INVALID, "bad HNSW list of node %d in '%s'", i, path);
            left -= 4 + (uint64_t)cur * 4;
            g.levels[i] = cur / g.hK;
            g.loff[i] = (int64_t)g.lists.size();
            size_t at = g.lists.size();
            g.lists.resize(at + (size_t)cur);
            if (cur && !rd(f, g.lists.data() + at, (size_t)cur))
                return fail(GSX_ERR_INVALID, "truncated HNSW lists in '%s'", path);
        }
        g.loff[g.N] = (int64_t)g.lists.size();
    }
    return GSX_OK;
}

// NSG format (graph.hpp:354-379): K, ep, then per node (count, ids).
int load_nsg(const char *path, HostGraph &g) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) return fail(GSX_ERR_IO, "cannot open graph file '%s'", path);
    const std::streamoff size = f.tellg();
    f.seekg(0);
    int32_t ep = 0;
    if (!rd(f, &g.K) || !rd(f, &ep) || g.K <= 0) return fail(GSX_ERR_INVALID, "bad NSG header in '%s'", path);
    if (g.K > kMaxDegree) return degree_unsupported(g.K);
    g.eps.assign(1, ep);
    std::vector<int32_t> buf;
    std::vector<std::vector<int32_t>> rows;
    while (f.tellg() < size) {
        int32_t c = 0;
        if (!rd(f, &c) || c < 0 || c > g.K) return fail(GSX_ERR_INVALID, "bad NSG row in '%s'", path);
        buf.resize((size_t)c);
        if (c && !rd(f, buf.data(), (size_t)c)) return fail(GSX_ERR_INVALID, "truncated NSG file '%s'", path);
        rows.push_back(buf);
    }
    g.N = (int32_t)rows.size();
    g.adj.assign((size_t)g.N * g.K, -1);
    for (int32_t i = 0; i < g.N; ++i) std::memcpy(&g.adj[(size_t)i * g.K], rows[i].data(), rows[i].size() * 4);
    return GSX_OK;
}

// DiskANN format (graph.hpp:289-316): u64 file size, K, ep, u64 frozen, then (count, ids) rows.
int load_diskann(const char *path, HostGraph &g) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(GSX_ERR_IO, "cannot open graph file '%s'", path);
    uint64_t size = 0, frozen = 0;
    int32_t ep = 0;
    if (!rd(f, &size) || !rd(f, &g.K) || !rd(f, &ep) || !rd(f, &frozen) || g.K <= 0)
        return fail(GSX_ERR_INVALID, "bad DiskANN header in '%s'", path);
    if (g.K > kMaxDegree) return degree_unsupported(g.K);
    g.eps.assign(1, ep);
    std::vector<std::vector<int32_t>> rows;
    std::vector<int32_t> buf;
    while ((uint64_t)f.tellg() < size) {
        int32_t c = 0;
        if (!rd(f, &c) || c < 0 || c > g.K) return fail(GSX_ERR_INVALID, "bad DiskANN row in '%s'", path);
        buf.resize((size_t)c);
        if (c && !rd(f, buf.data(), (size_t)c)) return fail(GSX_ERR_INVALID, "truncated DiskANN file '%s'", path);
        rows.push_back(buf);
    }
    g.N = (int32_t)rows.size();
    g.adj.assign((size_t)g.N * g.K, -1);
    for (int32_t i = 0; i < g.N; ++i) std::memcpy(&g.adj[(size_t)i * g.K], rows[i].data(), rows[i].size() * 4);
    return GSX_OK;
}

// hnswlib level-0 file (graph.hpp:318-352); multi-level files are refused as in the reference.
int load_hnswlib(const char *path, HostGraph &g) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(GSX_ERR_IO, "cannot open graph file '%s'", path);
    uint64_t max_el = 0, size_per = 0, maxM0 = 0;
    int32_t max_level = 0, ep = 0;
    f.seekg(8, std::ios::cur);
    rd(f, &max_el);
    f.seekg(8, std::ios::cur);
    rd(f, &size_per);
    f.seekg(16, std::ios::cur);
    rd(f, &max_level);
    if (max_level > 1) return fail(GSX_ERR_UNSUPPORTED, "multi-level hnswlib files are not supported");
    rd(f, &ep);
    f.seekg(8, std::ios::cur);
    rd(f, &maxM0);
    f.seekg(24, std::ios::cur);
    if (!f || max_el == 0 || max_el > (1u << 31) - 1 || maxM0 == 0 || size_per < 4 * (maxM0 + 1))
        return fail(GSX_ERR_INVALID, "bad hnswlib header in '%s'", path);
    if (maxM0 > (uint64_t)kMaxDegree) return degree_unsupported(maxM0 > (1u << 30) ? (1 << 30) : (int32_t)maxM0);
    if (size_per > bytes_left(f) / max_el) return fail(GSX_ERR_INVALID, "truncated hnswlib file '%s'", path);
    g.N = (int32_t)max_el;
    g.K = (int32_t)maxM0;
    g.eps.assign(1, ep);
    g.adj.assign((size_t)g.N * g.K, -1);
    std::vector<char> buf(size_per);
    for (int32_t i = 0; i < g.N; ++i) {
        if (!rd(f, buf.data(), size_per)) return fail(GSX_ERR_INVALID, "truncated hnswlib file '%s'", path);
        int32_t c = 0;
        std::memcpy(&c, buf.data(), 4);
        if (c < 0 || c > g.K) return fail(GSX_ERR_INVALID, "bad hnswlib row %d in '%s'", i, path);
        std::memcpy(&g.adj[(size_t)i * g.K], buf.data() + 4, (size_t)c * 4);
    }
    return GSX_OK;
}

}  // namespace

int validate_graph(const HostGraph &g) {
    if (g.N <= 0 || g.K <= 0) return fail(GSX_ERR_INVALID, "empty graph");
    if (g.K > kMaxDegree) return fail(GSX_ERR_UNSUPPORTED, "graph degree %d exceeds %d", g.K, kMaxDegree);
    if (g.adj.size() != (size_t)g.N * g.K) return fail(GSX_ERR_INVALID, "adjacency size mismatch");
    for (size_t i = 0; i < g.adj.size(); ++i) {
        const int32_t v = g.adj[i];
        if (v < -1 || v >= g.N) return fail(GSX_ERR_INVALID, "neighbour id %d of node %zu out of range", v, i / g.K);
    }
    if (!g.has_hnsw && g.eps.empty()) return fail(GSX_ERR_INVALID, "graph has no entry point");
    for (int32_t e : g.eps)
        if (e < 0 || e >= g.N) return fail(GSX_ERR_INVALID, "entry point %d out of range", e);
    if (g.has_hnsw) {
        if (g.hK <= 0 || g.hK > kMaxDegree) return fail(GSX_ERR_UNSUPPORTED, "HNSW level degree %d unsupported", g.hK);
        if (g.hep < 0 || g.hep >= g.N) return fail(GSX_ERR_INVALID, "HNSW entry point out of range");
        if (g.levels.size() != (size_t)g.N || g.loff.size() != (size_t)g.N + 1)
            return fail(GSX_ERR_INVALID, "HNSW level tables malformed");
        for (int32_t u = 0; u < g.N; ++u) {
            const int32_t lv = g.levels[u];
            if (lv < 0 || g.loff[u + 1] - g.loff[u] != (int64_t)lv * g.hK)
                return fail(GSX_ERR_INVALID, "HNSW lists of node %d malformed", u);
            for (int32_t l = 1; l <= lv; ++l) {
                const int32_t *list = g.lists.data() + g.loff[u] + (int64_t)(l - 1) * g.hK;
                for (int32_t i = 0; i < g.hK; ++i) {
                    const int32_t v = list[i];
                    if (v == -1) break;
                    // the descent reads v's list on level l, so v must exist on that level
                    if (v < 0 || v >= g.N || g.levels[v] < l)
                        return fail(GSX_ERR_INVALID, "HNSW neighbour %d of node %d not on level %d", v, u, l);
                }
            }
        }
    }
    return GSX_OK;
}

int graph_load(const char *path, const char *format, HostGraph &g) {
    g = HostGraph();
    const std::string fmt = format ? format : "glass";
    int rc;
    if (fmt == "glass") rc = load_glass(path, g);
    else if (fmt == "nsg") rc = load_nsg(path, g);
    else if (fmt == "diskann") rc = load_diskann(path, g);
    else if (fmt == "hnswlib") rc = load_hnswlib(path, g);
    else return fail(GSX_ERR_INVALID, "unknown graph format '%s'", fmt.c_str());
    if (rc != GSX_OK) return rc;
    return validate_graph(g);
}

int graph_save(const HostGraph &g, const char *path) {
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(GSX_ERR_IO, "cannot write graph file '%s'", path);
    const int32_t nep = (int32_t)g.eps.size();
    f.write(reinterpret_cast<const char *>(&nep), 4);
    f.write(reinterpret_cast<const char *>(g.eps.data()), (std::streamsize)nep * 4);
    f.write(reinterpret_cast<const char *>(&g.N), 4);
    f.write(reinterpret_cast<const char *>(&g.K), 4);
    f.write(reinterpret_cast<const char *>(g.adj.data()), (std::streamsize)g.adj.size() * 4);
    if (g.has_hnsw) {
        f.write(reinterpret_cast<const char *>(&g.N), 4);
        f.write(reinterpret_cast<const char *>(&g.hK), 4);
        f.write(reinterpret_cast<const char *>(&g.hep), 4);
        for (int32_t i = 0; i < g.N; ++i) {
            const int32_t cur = g.levels[i] * g.hK;
            f.write(reinterpret_cast<const char *>(&cur), 4);
            f.write(reinterpret_cast<const char *>(g.lists.data() + g.loff[i]), (std::streamsize)cur * 4);
        }
    }
    if (!f) return fail(GSX_ERR_IO, "write failed for '%s'", path);
    return GSX_OK;
}

}  // namespace gsx
