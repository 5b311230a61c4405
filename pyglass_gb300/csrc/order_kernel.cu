// Work order of a large batch: the queries sorted by their projection on one principal direction of
// the base data, so that the queries resident on the GPU at the same time search nearby parts of the
// graph and share L2 lines (the reference's SearchBatch hands queries to OpenMP threads in index
// order, graph_searcher.hpp:143-159; the order decides only which queries run together, never a
// result, because every query's search is independent).
#include <cuda_runtime.h>

#include <cstdint>

#include "gsx_internal.h"

namespace gsx {

namespace {

constexpr int kSortThreads = 1024;

// One warp per query: bin of (q - mean) . dir on [lo, lo + kOrderBins / scale).
__global__ void order_keys(const float *__restrict__ q, int nq, int d, const float *__restrict__ dirmean, float lo,
                           float scale, uint32_t *__restrict__ keys) {
    const int lane = threadIdx.x & 31;
    const int qi = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (qi >= nq) return;
    const float *x = q + (size_t)qi * d;
    float s = 0.0f;
    for (int j = lane; j < d; j += 32) s += (x[j] - dirmean[d + j]) * dirmean[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        float b = (s - lo) * scale;
        b = b < 0.0f ? 0.0f : b;  // also maps NaN to bin 0
        keys[qi] = b >= (float)(kOrderBins - 1) ? (uint32_t)(kOrderBins - 1) : (uint32_t)b;
    }
}

// Counting sort of the bins in one block: histogram, exclusive scan, scatter.  Queries of one bin
// land in any order among themselves.
__global__ void __launch_bounds__(kSortThreads) order_sort(const uint32_t *__restrict__ keys, int nq,
                                                            int32_t *__restrict__ order) {
    __shared__ int cnt[kOrderBins];
    __shared__ int wsum[kSortThreads / 32];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    for (int b = t; b < kOrderBins; b += kSortThreads) cnt[b] = 0;
    __syncthreads();
    for (int i = t; i < nq; i += kSortThreads) atomicAdd(&cnt[keys[i]], 1);
    __syncthreads();
    // each thread owns kOrderBins / kSortThreads consecutive bins
    constexpr int per = kOrderBins / kSortThreads;
    int local[per];
    int tot = 0;
#pragma unroll
    for (int j = 0; j < per; ++j) {
        local[j] = cnt[t * per + j];
        tot += local[j];
    }
    int inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int w = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        wsum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    int run = inc - tot + (wid > 0 ? wsum[wid - 1] : 0);
#pragma unroll
    for (int j = 0; j < per; ++j) {
        cnt[t * per + j] = run;
        run += local[j];
    }
    __syncthreads();
    for (int i = t; i < nq; i += kSortThreads) order[atomicAdd(&cnt[keys[i]], 1)] = i;
}

}  // namespace

cudaError_t launch_batch_order(const float *q, int nq, int d, const float *dirmean, float lo, float scale,
                               uint32_t *keys, int32_t *order, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    const int warps_per_block = 8;
    order_keys<<<(nq + warps_per_block - 1) / warps_per_block, 32 * warps_per_block, 0, st>>>(q, nq, d, dirmean, lo,
                                                                                            scale, keys);
    order_sort<<<1, kSortThreads, 0, st>>>(keys, nq, order);
    return cudaGetLastError();
}

}  // namespace gsx
