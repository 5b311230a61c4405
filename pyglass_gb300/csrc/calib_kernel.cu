// Device-side calibration of SetData (graph_searcher.hpp:51-58, quant.train): the affine and
// symmetric calibrators' ranges (calibrator.hpp:14-63) and SQ4U's quantile range (find_minmax,
// quant/utils.hpp:31-40, on the first 10% of the flattened data, sq4u_quant.hpp:18-30), taken from
// the base data already resident on the device.  Values are compared through order-preserving
// 32-bit keys, so minima, maxima and order statistics are exact: the same floats the host
// reference selects.
#include <cuda_runtime.h>

#include <cstdint>

#include "gsx_internal.h"

namespace gsx {

namespace {

// Order-preserving key of a float (negative values reversed below the positive ones).
__device__ __forceinline__ uint32_t fkey(float x) {
    const uint32_t u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

constexpr int kThreads = 256;

int grid_of(int64_t n) {
    int64_t g = (n + kThreads * 8 - 1) / (kThreads * 8);
    if (g > 152 * 16) g = 152 * 16;
    return g < 1 ? 1 : (int)g;
}

// out[0] = min key, out[1] = max key (out preset to 0xffffffff / 0); absolute values when `absval`.
__global__ void minmax_keys(const float *__restrict__ x, int64_t n, int absval, unsigned *__restrict__ out) {
    uint32_t mn = 0xffffffffu, mx = 0u;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = absval ? fabsf(x[i]) : x[i];
        const uint32_t k = fkey(v);
        mn = k < mn ? k : mn;
        mx = k > mx ? k : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint32_t a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(out, mn);
        atomicMax(out + 1, mx);
    }
}

// One radix-select pass for two ranks at once: hist[s][digit] counts the items whose key matches
// prefix[s] on mask, by the 8-bit digit at `shift`.
__global__ void radix_hist2(const float *__restrict__ x, int64_t n, uint2 prefix, uint32_t mask, int shift,
                            unsigned *__restrict__ hist) {
    __shared__ unsigned h[2][256];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t k = fkey(x[i]);
        const uint32_t dgt = (k >> shift) & 255u;
        if ((k & mask) == prefix.x) atomicAdd(&h[0][dgt], 1u);
        if ((k & mask) == prefix.y) atomicAdd(&h[1][dgt], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x) {
        const unsigned c = (&h[0][0])[i];
        if (c) atomicAdd(hist + i, c);
    }
}

// SQ8's AffinePerDimCalibrator (calibrator.hpp:66-91) with drop ratio 0: find_minmax_perdim
// (quant/utils.hpp:52-70) files float i of the row-major data under "dimension" i / n, so entry j
// is the min / max of the j-th block of n consecutive floats.  One block of threads per entry.
__global__ void block_minmax(const float *__restrict__ x, int64_t n, int d, int dalign, float *__restrict__ out) {
    const int j = blockIdx.x;
    if (j >= dalign) return;
    if (j >= d) {
        if (threadIdx.x == 0) out[j] = out[dalign + j] = 0.0f;
        return;
    }
    const float *b = x + (int64_t)j * n;
    uint32_t mn = 0xffffffffu, mx = 0u;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t k = fkey(b[i]);
        mn = k < mn ? k : mn;
        mx = k > mx ? k : mx;
    }
    __shared__ uint32_t smn[32], smx[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint32_t a = __shfl_xor_sync(0xffffffffu, mn, o), c = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = a < mn ? a : mn;
        mx = c > mx ? c : mx;
    }
    if ((threadIdx.x & 31) == 0) {
        smn[threadIdx.x >> 5] = mn;
        smx[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mn = smn[w] < mn ? smn[w] : mn;
            mx = smx[w] > mx ? smx[w] : mx;
        }
        const uint32_t umn = (mn & 0x80000000u) ? (mn & 0x7fffffffu) : ~mn;
        const uint32_t umx = (mx & 0x80000000u) ? (mx & 0x7fffffffu) : ~mx;
        const float fmn = __uint_as_float(umn), fmx = __uint_as_float(umx);
        out[j] = fmn;
        out[dalign + j] = fmx - fmn;
    }
}

}  // namespace

cudaError_t launch_block_minmax(const float *x, int64_t n, int d, int dalign, float *out, cudaStream_t st) {
    block_minmax<<<dalign, kThreads, 0, st>>>(x, n, d, dalign, out);
    return cudaGetLastError();
}

cudaError_t launch_minmax_keys(const float *x, int64_t n, int absval, unsigned *out, cudaStream_t st) {
    const unsigned init[2] = {0xffffffffu, 0u};
    cudaError_t e = cudaMemcpyAsync(out, init, sizeof(init), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    minmax_keys<<<grid_of(n), kThreads, 0, st>>>(x, n, absval, out);
    return cudaGetLastError();
}

cudaError_t launch_radix_hist2(const float *x, int64_t n, uint32_t prefix0, uint32_t prefix1, uint32_t mask, int shift,
                               unsigned *hist, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(hist, 0, 512 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    radix_hist2<<<grid_of(n), kThreads, 0, st>>>(x, n, make_uint2(prefix0, prefix1), mask, shift, hist);
    return cudaGetLastError();
}

float float_of_key(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    static_assert(sizeof(f) == sizeof(u), "float is 32 bits");
    __builtin_memcpy(&f, &u, 4);
    return f;
}

}  // namespace gsx
