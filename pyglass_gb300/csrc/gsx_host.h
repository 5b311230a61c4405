// Host-side runtime of libglass_gb300: graphs, searchers, errors.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <exception>
#include <new>
#include <string>
#include <vector>

#include "../../include/glass_gb300.h"
#include "gsx_internal.h"

namespace gsx {

// Records the calling thread's error message and returns `code`.
int fail(int code, const char *fmt, ...);
// Maps a CUDA error to GSX_ERR_CUDA / GSX_ERR_NOMEM with a message.
int cuda_fail(cudaError_t e, const char *what);

// Closes the try block that encloses the body of every int-returning C-ABI entry point, so that
// no C++ exception crosses the ABI: a failed host allocation becomes GSX_ERR_NOMEM, any other
// exception GSX_ERR_INVALID, each with a message.
#define GSX_ABI_GUARD(name)                                                       \
    catch (const std::bad_alloc &) {                                              \
        return ::gsx::fail(GSX_ERR_NOMEM, "%s: out of host memory", name);       \
    }                                                                             \
    catch (const std::exception &e_) {                                            \
        return ::gsx::fail(GSX_ERR_INVALID, "%s: %s", name, e_.what());          \
    }

#define GSX_CUDA(call)                                              \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return ::gsx::cuda_fail(e_, #call); \
    } while (0)

// Makes `device` current for the scope and gives the caller's current device back on exit, so an
// entry point leaves the calling thread's CUDA state as it found it.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != device) err = cudaSetDevice(device);
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
};

struct HostGraph {
    int32_t N = 0, K = 0;
    std::vector<int32_t> adj;
    std::vector<int32_t> eps;
    int32_t has_hnsw = 0, hK = 0, hep = 0;
    std::vector<int32_t> levels;
    std::vector<int64_t> loff;
    std::vector<int32_t> lists;
};

int graph_load(const char *path, const char *format, HostGraph &g);
int graph_save(const HostGraph &g, const char *path);
int validate_graph(const HostGraph &g);

// A device allocation that grows on demand.
struct DevBuf;
// Global visited tables of `slots` warps (2^bits 32-bit entries each) followed by their query
// counters; zeroed whenever the layout (slots, bits, id bits) changes, so every slot reads as
// empty and the counters restart.
struct SpillTables;
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    int ensure(size_t n);
    void release();
    ~DevBuf() { release(); }
    template <typename T>
    T *as() const { return reinterpret_cast<T *>(p); }
};

struct SpillTables {
    DevBuf buf;
    size_t slots = 0;
    int bits = 0;
    int shift = 0;
    int ensure(size_t slots, int bits, int shift, cudaStream_t st, uint32_t **tab, uint32_t **epoch);
};

}  // namespace gsx

// The opaque handles of the C ABI.
struct gsx_graph {
    gsx::HostGraph g;
};

struct gsx_searcher {
    // create_searcher arguments
    int kind = gsx::K_FP32, metric = gsx::M_L2;
    int has_refine = 0;
    int r_kind = gsx::K_FP32;  // refine store: FP32 or FP16 rows
    float refine_factor = 1.0f;
    int device = 0;
    int ef = 32;
    gsx::HostGraph graph;  // host copy kept for save/inspection

    // device index
    bool has_data = false;
    gsx::IndexView ix{};
    gsx::DevBuf adj, eps, levels, loff, lists, codes, r_codes, sq8p;
    std::vector<float> h_sq8p;  // host copy of SQ8's per-dimension parameters (mins, then difs)
    cudaStream_t stream = nullptr;
    int num_sms = 0;

    // per-call scratch (device)
    gsx::DevBuf q, ids, dis, status, cmps, efp, kp, order, counters, dist_out, dist_ids;
    gsx::SpillTables spill, gtab;  // per-warp spill tables; whole-graph tables of the exact re-run
    gsx::DevBuf pdir, qkeys, qorder;  // batch order: direction + mean (2d floats), per-batch keys/order
    float order_lo = 0.0f, order_scale = 0.0f;
    // host copies for reporting
    std::vector<int32_t> h_cmps, h_status;
    double last_avg_cmps = 0.0;
    int32_t visit_hint = 0;  // largest per-query distance count seen
    double visit_avg = 0.0;  // mean per-query distance count of the last large batch
    int32_t last_batch_nq = 0;  // queries of the last host batch (the size optimize tunes for)

    // sample of base rows kept for optimize (graph_searcher.hpp:62-69)
    std::vector<float> sample;
    int32_t sample_n = 0;

    gsx_tuning tuning{0, 0, 0, 0, 0};
    bool spill_from_optimize = false;  // tuning.spill_bits was picked by optimize for its ef (launches
                                       // with larger pools get the automatic size)
    int spill_auto_at_opt = 0;         // the automatic size when optimize picked it
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};
