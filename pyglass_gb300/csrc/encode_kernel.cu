// Device-side encoding of base rows (SetData's quant.add, glass/searcher/graph_searcher.hpp:51-58):
// SQ8U (sq8u_quant.hpp:242-254), SQ4U (sq4u_quant.hpp:311-329), E5M2 (e5m2_quant.hpp:382-394) and
// the zero-padded FP32 rows of FP32Quantizer / the refine store (fp32_quant.hpp:428-440).
// The arithmetic is the query encoder's (gsx_device.cuh), so base and query codes agree with
// the reference bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "gsx_device.cuh"
#include "gsx_internal.h"

namespace gsx {

namespace {

template <int KIND, int METRIC>
__global__ void encode_rows(const float *__restrict__ data, int64_t n, int d, int csize, float p0, float p1,
                            uint32_t *__restrict__ out) {
    const int nw = csize >> 2;
    const int64_t total = n * (int64_t)nw;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / nw;
        const int wi = (int)(t - row * nw);
        const float *x = data + row * (int64_t)d;
        uint32_t word = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int b = 4 * wi + k;
            uint32_t byte;
            if (KIND == K_E5M2) byte = b < d ? e5m2_of(x[b]) : 0u;
            else byte = sq_code_byte<KIND, METRIC>(x, d, b, p0, p1);
            word |= byte << (8 * k);
        }
        out[t] = word;
    }
}

// FP16 / BF16 rows (fp16_quant.hpp:26-35, bf16_quant.hpp:26-37), two codes per 32-bit word.
// FP16 is helpa::fp32_to_fp16 on x86 (x86/data_convert.hpp:17-38): round to nearest even in 16-wide
// blocks while i < d, so the row's padding holds the conversions of the floats that follow the row
// in the data array (the next row's first values; zero past the end of the array).  BF16 converts
// element by element with round-to-nearest on the bit pattern, (bits + 0x8000) >> 16
// (helpa/types.hpp:20,34-35,72-75), and leaves the padding zero.
template <int KIND>
__global__ void encode_half_rows(const float *__restrict__ data, int64_t n, int d, int dalign,
                                 uint32_t *__restrict__ out) {
    const int nw = dalign >> 1;
    const int64_t total = n * (int64_t)nw, nitems = n * (int64_t)d;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / nw;
        const int wi = (int)(t - row * nw);
        uint32_t word = 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int j = 2 * wi + k;
            const int64_t e = row * (int64_t)d + j;
            uint32_t h = 0;
            if (KIND == K_FP16) {
                if (e < nitems) h = __half_as_ushort(__float2half_rn(data[e]));
            } else if (j < d) {
                h = (__float_as_uint(data[e]) + 0x8000u) >> 16;
            }
            word |= (h & 0xffffu) << (16 * k);
        }
        out[t] = word;
    }
}

// SQ8 rows (sq8_quant.hpp:43-47): code = transform(x, j) with the per-dimension calibrator, mul 255;
// the padding stays zero.  p = mins[dalign] then difs[dalign].
__global__ void encode_sq8_rows(const float *__restrict__ data, int64_t n, int d, int dalign,
                                const float *__restrict__ p, uint8_t *__restrict__ out) {
    const int64_t total = n * (int64_t)dalign;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / dalign;
        const int j = (int)(t - row * dalign);
        out[t] = j < d ? (uint8_t)affine_code(data[row * (int64_t)d + j], p[j], p[dalign + j], 255.0f) : (uint8_t)0;
    }
}

__global__ void pad_rows(const float *__restrict__ data, int64_t n, int d, int dalign, float *__restrict__ out) {
    const int64_t total = n * (int64_t)dalign;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = t / dalign;
        const int j = (int)(t - row * dalign);
        out[t] = j < d ? data[row * (int64_t)d + j] : 0.0f;
    }
}

int grid_for(int64_t work) {
    int64_t g = (work + 255) / 256;
    if (g > 152 * 32) g = 152 * 32;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

cudaError_t launch_encode(int kind, int metric, const float *data, int64_t n, int d, int dalign, int csize, float p0,
                          float p1, uint8_t *out, cudaStream_t st) {
    const int g = grid_for(n * (csize >> 2));
    uint32_t *o = reinterpret_cast<uint32_t *>(out);
    if (kind == K_SQ4U) encode_rows<K_SQ4U, M_L2><<<g, 256, 0, st>>>(data, n, d, csize, p0, p1, o);
    else if (kind == K_SQ2U) encode_rows<K_SQ2U, M_L2><<<g, 256, 0, st>>>(data, n, d, csize, p0, p1, o);
    else if (kind == K_SQ4UA) encode_rows<K_SQ4UA, M_L2><<<g, 256, 0, st>>>(data, n, d, csize, p0, p1, o);
    else if (kind == K_SQ1) encode_rows<K_SQ1, M_L2><<<g, 256, 0, st>>>(data, n, d, csize, p0, p1, o);
    else if (kind == K_SQ8U && metric == M_IP) encode_rows<K_SQ8U, M_IP><<<g, 256, 0, st>>>(data, n, d, csize, p0, p1, o);
    else if (kind == K_SQ8U) encode_rows<K_SQ8U, M_L2><<<g, 256, 0, st>>>(data, n, d, csize, p0, p1, o);
    else if (kind == K_E5M2) encode_rows<K_E5M2, M_L2><<<g, 256, 0, st>>>(data, n, d, csize, p0, p1, o);
    else if (kind == K_FP16) encode_half_rows<K_FP16><<<g, 256, 0, st>>>(data, n, d, dalign, o);
    else if (kind == K_BF16) encode_half_rows<K_BF16><<<g, 256, 0, st>>>(data, n, d, dalign, o);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_encode_sq8(const float *data, int64_t n, int d, int dalign, const float *p, uint8_t *out,
                              cudaStream_t st) {
    encode_sq8_rows<<<grid_for(n * dalign), 256, 0, st>>>(data, n, d, dalign, p, out);
    return cudaGetLastError();
}

cudaError_t launch_pad_rows(const float *data, int64_t n, int d, int dalign, float *out, cudaStream_t st) {
    pad_rows<<<grid_for(n * dalign), 256, 0, st>>>(data, n, d, dalign, out);
    return cudaGetLastError();
}

}  // namespace gsx
