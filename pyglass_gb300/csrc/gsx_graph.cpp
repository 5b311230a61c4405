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

// The whole file in memory (one read).  The row formats below (NSG, DiskANN) are parsed from it in
// two passes: the first walks the (count, ids) records to count the rows and check every count, the
// second copies each record into its -1-padded row.
int read_all(const char *path, std::vector<char> &buf) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(GSX_ERR_IO, "cannot open graph file '%s'", path);
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (size < 0) {
        std::fclose(f);
        return fail(GSX_ERR_IO, "cannot size graph file '%s'", path);
    }
    buf.resize((size_t)size);
    const size_t got = size ? std::fread(buf.data(), 1, (size_t)size, f) : 0;
    std::fclose(f);
    if (got != (size_t)size) return fail(GSX_ERR_IO, "short read of graph file '%s'", path);
    return GSX_OK;
}

// (count, ids) records starting before byte `end` of buf, from byte `at`, into g.adj (g.K set); as in
// the reference's readers a record that starts before `end` is read whole.
int parse_rows(const std::vector<char> &buf, size_t at, size_t end, HostGraph &g, const char *what, const char *path) {
    if (end > buf.size()) end = buf.size();
    const size_t total = buf.size();
    size_t n = 0;
    for (size_t p = at; p < end; ++n) {
        int32_t c = 0;
        if (total - p < 4) return fail(GSX_ERR_INVALID, "truncated %s file '%s'", what, path);
        std::memcpy(&c, buf.data() + p, 4);
        if (c < 0 || c > g.K) return fail(GSX_ERR_INVALID, "bad %s row %zu in '%s'", what, n, path);
        if ((uint64_t)(total - p - 4) < (uint64_t)c * 4) return fail(GSX_ERR_INVALID, "truncated %s file '%s'", what, path);
        p += 4 + (size_t)c * 4;
    }
    if (n == 0 || n > 0x7fffffffu) return fail(GSX_ERR_INVALID, "%s file '%s' holds %zu rows", what, path, n);
    g.N = (int32_t)n;
    g.adj.assign(n * (size_t)g.K, -1);
    size_t p = at;
    for (size_t i = 0; i < n; ++i) {
        int32_t c = 0;
        std::memcpy(&c, buf.data() + p, 4);
        std::memcpy(&g.adj[i * (size_t)g.K], buf.data() + p + 4, (size_t)c * 4);
        p += 4 + (size_t)c * 4;
    }
    return GSX_OK;
}

// NSG format (graph.hpp:354-379): K, ep, then per node (count, ids).
int load_nsg(const char *path, HostGraph &g) {
    std::vector<char> buf;
    int rc = read_all(path, buf);
    if (rc) return rc;
    int32_t hdr[2] = {0, 0};
    if (buf.size() < 8) return fail(GSX_ERR_INVALID, "bad NSG header in '%s'", path);
    std::memcpy(hdr, buf.data(), 8);
    g.K = hdr[0];
    if (g.K <= 0) return fail(GSX_ERR_INVALID, "bad NSG header in '%s'", path);
    if (g.K > kMaxDegree) return degree_unsupported(g.K);
    g.eps.assign(1, hdr[1]);
    return parse_rows(buf, 8, buf.size(), g, "NSG", path);
}

// DiskANN format (graph.hpp:289-316): u64 file size, K, ep, u64 frozen, then (count, ids) rows up to
// the size the header states.
int load_diskann(const char *path, HostGraph &g) {
    std::vector<char> buf;
    int rc = read_all(path, buf);
    if (rc) return rc;
    if (buf.size() < 24) return fail(GSX_ERR_INVALID, "bad DiskANN header in '%s'", path);
    uint64_t size = 0;
    int32_t ep = 0;
    std::memcpy(&size, buf.data(), 8);
    std::memcpy(&g.K, buf.data() + 8, 4);
    std::memcpy(&ep, buf.data() + 12, 4);
    if (g.K <= 0) return fail(GSX_ERR_INVALID, "bad DiskANN header in '%s'", path);
    if (g.K > kMaxDegree) return degree_unsupported(g.K);
    g.eps.assign(1, ep);
    return parse_rows(buf, 24, size < buf.size() ? (size_t)size : buf.size(), g, "DiskANN", path);
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
