// Allocation-free batched search.
//
// Some callers of this library must not allocate device memory once they are serving: engines
// that reserve the GPU's memory for their own pool at start-up and treat any later driver
// allocation as a fault, and latency-bound paths that cannot afford the device-wide
// synchronisation cudaMalloc / cudaFree may bring.  For them, gsx_searcher_search_batch_noalloc
// runs the batched search with no allocation at all: the caller passes the queries and the output
// buffers, and the kernel's scratch (the work-queue counters and one status word per query) lives
// in the fixed array below, which every GPU that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "gsx_host.h"

namespace gsx {

// Largest number of queries one allocation-free call accepts.
constexpr int kNoAllocMaxQueries = 65536;

namespace {

// [0] work-queue head, [1] overflow count, [2 .. 2+kNoAllocMaxQueries) per-query status.
// In host code this name is only a stand-in for the device copy; its device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) uint32_t g_noalloc_scratch[2 + kNoAllocMaxQueries];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint32_t *g_scratch[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device.
int scratch_of(int device, uint32_t **out) {
    if (device < 0 || device >= kMaxDevices) return fail(GSX_ERR_INVALID, "device %d out of range", device);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_scratch[device] = static_cast<uint32_t *>(p);
    }
    *out = g_scratch[device];
    return GSX_OK;
}

}  // namespace

int noalloc_make_cfg(gsx_searcher *s, int kmax, int efmax, int nq, LaunchCfg *cfg);

}  // namespace gsx

using namespace gsx;

extern "C" int gsx_searcher_search_batch_noalloc(gsx_searcher *s, const float *d_queries, int32_t nq, int32_t k,
                                                 int32_t *d_ids, float *d_dis, void *stream) {
    try {
        if (!s || (nq > 0 && (!d_queries || !d_ids))) return fail(GSX_ERR_INVALID, "null argument");
        if (!s->has_data) return fail(GSX_ERR_STATE, "search before set_data");
        if (k <= 0) return fail(GSX_ERR_INVALID, "k must be positive");
        if (nq < 0 || nq > kNoAllocMaxQueries)
            return fail(GSX_ERR_INVALID, "nq=%d exceeds the %d-query limit of the allocation-free search", nq,
                        kNoAllocMaxQueries);
        if (nq == 0) return GSX_OK;
        DeviceScope dev(s->device);
        if (dev.err != cudaSuccess) return cuda_fail(dev.err, "cudaSetDevice");
        uint32_t *scratch = nullptr;
        int rc = scratch_of(s->device, &scratch);
        if (rc) return rc;
        LaunchCfg cfg;
        if ((rc = noalloc_make_cfg(s, k, s->ef, nq, &cfg))) return rc;
        cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
        // the array keeps the previous call's contents: the queue head and overflow count restart at
        // zero; every status word of this call is written by its query
        cudaError_t e = cudaMemsetAsync(scratch, 0, 2 * sizeof(uint32_t), st);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(no-alloc scratch)");
        BatchView bv{};
        bv.queries = d_queries;
        bv.nq = nq;
        bv.k = k;
        bv.ef = s->ef;
        bv.out_stride = k;
        bv.out_ids = d_ids;
        bv.out_dis = d_dis;
        bv.status = reinterpret_cast<int32_t *>(scratch + 2);
        bv.counter = scratch;
        bv.overflow = scratch + 1;
        e = launch_search(s->ix, bv, cfg, st);
        if (e != cudaSuccess) return cuda_fail(e, "search launch (no-alloc)");
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_search_batch_noalloc")
}

extern "C" int gsx_searcher_noalloc_overflow_count(gsx_searcher *s, uint32_t *count) {
    try {
        if (!s || !count) return fail(GSX_ERR_INVALID, "null argument");
        DeviceScope dev(s->device);
        if (dev.err != cudaSuccess) return cuda_fail(dev.err, "cudaSetDevice");
        uint32_t *scratch = nullptr;
        int rc = scratch_of(s->device, &scratch);
        if (rc) return rc;
        // word 1 of the array: the overflow count of the latest allocation-free search on this device
        cudaError_t e = cudaMemcpy(count, scratch + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(no-alloc overflow count)");
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_noalloc_overflow_count")
}
