// Device building blocks of the graph-search path: order keys, query encoding and the
// distance engines of the four quantizers.  Shared by search_kernel.cu and encode_kernel.cu.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gsx_internal.h"

namespace gsx {

constexpr unsigned kFull = 0xffffffffu;

// ---- order keys ------------------------------------------------------------------------------
// Pool entries carry an unsigned key whose order is the order of the distance: int32 for the
// SQ quantizers, fp32 for E5M2/FP32 (with -0 folded onto +0, which compare equal).
__device__ __forceinline__ uint32_t key_of(int32_t d) { return (uint32_t)d ^ 0x80000000u; }
__device__ __forceinline__ uint32_t key_of(float f) {
    uint32_t b = __float_as_uint(f);
    if (b == 0x80000000u) b = 0u;
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float dist_of_key_int(uint32_t k) { return (float)(int32_t)(k ^ 0x80000000u); }
__device__ __forceinline__ float dist_of_key_float(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

template <int KIND>
struct IsIntKind {
    static constexpr bool value =
        (KIND == K_SQ8U || KIND == K_SQ4U || KIND == K_SQ2U || KIND == K_SQ4UA || KIND == K_SQ1);
};

// ---- query encoding ---------------------------------------------------------------------------
// AffineCalibrator::transform (glass/quant/calibrator.hpp:488-492): IEEE division by dif, clamp
// to [0,1], scale, round half away from zero.  The reference build divides (it does not
// multiply by a reciprocal), and CUDA's '/' is the correctly rounded division, so the codes are
// identical.
__device__ __forceinline__ int affine_code(float x, float mn, float dif, float mul) {
    float t = (x - mn) / dif;
    if (t < 0.0f) t = 0.0f;
    if (t > 1.0f) t = 1.0f;
    return (int)roundf(t * mul);
}
// SymCalibrator::transform (calibrator.hpp:516-520).
__device__ __forceinline__ int sym_code(float x, float mx, float mul) {
    float t = x / mx;
    if (t < -1.0f) t = -1.0f;
    if (t > 1.0f) t = 1.0f;
    return (int)roundf(t * mul);
}

// Code byte `b` of an encoded row (base or query) for the SQ kinds; x = fp32 row, zero past d.
template <int KIND, int METRIC>
__device__ __forceinline__ uint32_t sq_code_byte(const float *x, int d, int b, float p0, float p1) {
    if (KIND == K_SQ2U) {  // sq2u_quant.hpp:39-52: dim 4b+k -> bits 2k of byte b
        uint32_t byte = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int j = 4 * b + k;
            if (j < d) byte |= (uint32_t)affine_code(x[j], p0, p1, 3.0f) << (2 * k);
        }
        return byte;
    } else if (KIND == K_SQ1) {  // sq1_quant.hpp:36-42: bit j%8 of byte j/8 = (x > 0)
        uint32_t byte = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = 8 * b + k;
            if (j < d && x[j] > 0.0f) byte |= 1u << k;
        }
        return byte;
    } else if (KIND == K_SQ4U || KIND == K_SQ4UA) {  // sq4u_quant.hpp:319-329: even dim -> low nibble
        int j0 = 2 * b, j1 = 2 * b + 1;
        uint32_t lo = j0 < d ? (uint32_t)affine_code(x[j0], p0, p1, 15.0f) : 0u;
        uint32_t hi = j1 < d ? (uint32_t)affine_code(x[j1], p0, p1, 15.0f) : 0u;
        return lo | (hi << 4);
    } else {  // SQ8U, sq8u_quant.hpp:250-254
        if (b >= d) return 0u;
        int c = METRIC == M_L2 ? affine_code(x[b], p0, p1, 127.0f) : sym_code(x[b], p0, 127.0f);
        return (uint32_t)(uint8_t)(int8_t)c;
    }
}

// e5m2 = high byte of the fp16 value (round to nearest even), glass/types.hpp:19-32.
__device__ __forceinline__ uint32_t e5m2_of(float x) {
    return (uint32_t)(__half_as_ushort(__float2half_rn(x)) >> 8);
}
__device__ __forceinline__ float f32_of_e5m2(uint32_t b) {
    return __half2float(__ushort_as_half((unsigned short)((b & 0xffu) << 8)));
}

// ---- warp helpers -------------------------------------------------------------------------------
template <int W>
__device__ __forceinline__ int32_t team_sum(int32_t v) {
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// ---- integer distance engines -----------------------------------------------------------------
// A row of csize bytes is read as 16-byte chunks; with LPR lanes per row, lane `sub` of a team
// takes chunks sub, sub+LPR, ...  The sums are exact integers, so any split gives the reference's
// value (helpa l2_s7_s7 / dot_s8_s8 / l2a_u4_u4, ref/l2_ref.hpp:57-77, ref/dot_ref.hpp:131-138).
//
// Query layout in shared memory (qc):
//   SQ4U: words [0, nw) = low nibbles of the query code (0x0F0F0F0F lanes), [nw, 2nw) = high
//         nibbles; nw = csize/4.  Sum of squares of all nibbles in qsq.
//   SQ8U: words [0, nw) = the code bytes.  L2 also uses qsq.
//   SQ4UA: the query is coded on 0..127 (transform(x, 127)); words [0, nw) hold its even dimensions
//         and [nw, 2nw) its odd ones, in the byte order of the base words' low / high nibbles.
//   SQ1:  words [0, nw) = the query's sign bits.
//   SQ2U: words [k*nw, (k+1)*nw), k = 0..3 = the query's 2-bit codes at bits 2k of each byte, one per
//         byte (0x03030303 lanes); qsq as for SQ4U.
// SQ2U word: the four 2-bit planes against the query's planes (l2a_u2_u2, helpa x86/l2_impl.hpp:301-333).
__device__ __forceinline__ void sq2_word(uint32_t w, const uint32_t *qp, int nw, uint32_t &aa, uint32_t &ab) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t x = (w >> (2 * k)) & 0x03030303u;
        aa = __dp4a(x, x, aa);
        ab = __dp4a(x, qp[k * nw], ab);
    }
}

// SQ4UA word (L2SqrSQ8SQ4, glass/simd/avx512.hpp:146-158): code c read as 8c+4 on the 0..127 scale.
__device__ __forceinline__ void sq4a_word(uint32_t w, uint32_t qe, uint32_t qo, uint32_t &aa, uint32_t &ab) {
    const uint32_t ylo = ((w & 0x0F0F0F0Fu) << 3) + 0x04040404u, yhi = (((w >> 4) & 0x0F0F0F0Fu) << 3) + 0x04040404u;
    aa = __dp4a(ylo, ylo, aa);
    aa = __dp4a(yhi, yhi, aa);
    ab = __dp4a(ylo, qe, ab);
    ab = __dp4a(yhi, qo, ab);
}

__device__ __forceinline__ void sq4_word(uint32_t w, uint32_t ql, uint32_t qh, uint32_t &aa, uint32_t &ab) {
    uint32_t lo = w & 0x0F0F0F0Fu, hi = (w >> 4) & 0x0F0F0F0Fu;
    aa = __dp4a(lo, lo, aa);
    aa = __dp4a(hi, hi, aa);
    ab = __dp4a(lo, ql, ab);
    ab = __dp4a(hi, qh, ab);
}

template <int KIND, int METRIC, int LPR>
__device__ __forceinline__ int32_t sq_partial(const uint8_t *__restrict__ codes, int csize, int id, int sub,
                                             const uint32_t *qc) {
    const uint4 *row = reinterpret_cast<const uint4 *>(codes + (size_t)id * (size_t)csize);
    const int nch = csize >> 4;
    if (KIND == K_SQ4UA) {
        const uint4 *qe = reinterpret_cast<const uint4 *>(qc);
        const uint4 *qo = reinterpret_cast<const uint4 *>(qc + (csize >> 2));
        uint32_t aa = 0, ab = 0;
#pragma unroll 4
        for (int c = sub; c < nch; c += LPR) {
            const uint4 v = __ldg(row + c);
            const uint4 e = qe[c], o = qo[c];
            sq4a_word(v.x, e.x, o.x, aa, ab);
            sq4a_word(v.y, e.y, o.y, aa, ab);
            sq4a_word(v.z, e.z, o.z, aa, ab);
            sq4a_word(v.w, e.w, o.w, aa, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (KIND == K_SQ1) {
        const uint4 *qv = reinterpret_cast<const uint4 *>(qc);
        int32_t s = 0;
        for (int c = sub; c < nch; c += LPR) {
            const uint4 v = __ldg(row + c), q = qv[c];
            s += __popc(v.x ^ q.x) + __popc(v.y ^ q.y) + __popc(v.z ^ q.z) + __popc(v.w ^ q.w);
        }
        return s;
    } else if (KIND == K_SQ2U) {
        const int nw = csize >> 2;
        uint32_t aa = 0, ab = 0;
#pragma unroll 2
        for (int c = sub; c < nch; c += LPR) {
            const uint4 v = __ldg(row + c);
            const uint32_t *q = qc + 4 * c;
            sq2_word(v.x, q + 0, nw, aa, ab);
            sq2_word(v.y, q + 1, nw, aa, ab);
            sq2_word(v.z, q + 2, nw, aa, ab);
            sq2_word(v.w, q + 3, nw, aa, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (KIND == K_SQ4U) {
        const uint4 *ql = reinterpret_cast<const uint4 *>(qc);
        const uint4 *qh = reinterpret_cast<const uint4 *>(qc + (csize >> 2));
        uint32_t aa = 0, ab = 0;
#pragma unroll 4
        for (int c = sub; c < nch; c += LPR) {
            uint4 v = __ldg(row + c);
            uint4 l = ql[c], h = qh[c];
            sq4_word(v.x, l.x, h.x, aa, ab);
            sq4_word(v.y, l.y, h.y, aa, ab);
            sq4_word(v.z, l.z, h.z, aa, ab);
            sq4_word(v.w, l.w, h.w, aa, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (METRIC == M_L2) {  // SQ8U L2: codes are 0..127
        const uint4 *qv = reinterpret_cast<const uint4 *>(qc);
        uint32_t aa = 0, ab = 0;
#pragma unroll 4
        for (int c = sub; c < nch; c += LPR) {
            uint4 v = __ldg(row + c);
            uint4 q = qv[c];
            aa = __dp4a(v.x, v.x, aa); ab = __dp4a(v.x, q.x, ab);
            aa = __dp4a(v.y, v.y, aa); ab = __dp4a(v.y, q.y, ab);
            aa = __dp4a(v.z, v.z, aa); ab = __dp4a(v.z, q.z, ab);
            aa = __dp4a(v.w, v.w, aa); ab = __dp4a(v.w, q.w, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else {  // SQ8U IP: signed codes -127..127, distance = -sum(x*y)
        const uint4 *qv = reinterpret_cast<const uint4 *>(qc);
        int32_t s = 0;
#pragma unroll 4
        for (int c = sub; c < nch; c += LPR) {
            uint4 v = __ldg(row + c);
            uint4 q = qv[c];
            s = __dp4a((int)v.x, (int)q.x, s);
            s = __dp4a((int)v.y, (int)q.y, s);
            s = __dp4a((int)v.z, (int)q.z, s);
            s = __dp4a((int)v.w, (int)q.w, s);
        }
        return s;
    }
}

// Whole-row integer partial distance (one lane per row) from a row in shared memory: the same
// arithmetic as sq_partial with one lane.
template <int KIND, int METRIC>
__device__ __forceinline__ int32_t sq_partial_row(const uint4 *row, int nch, const uint32_t *qc) {
    if (KIND == K_SQ4UA) {
        const uint4 *qe = reinterpret_cast<const uint4 *>(qc);
        const uint4 *qo = reinterpret_cast<const uint4 *>(qc + 4 * nch);
        uint32_t aa = 0, ab = 0;
#pragma unroll 4
        for (int c = 0; c < nch; ++c) {
            const uint4 v = row[c];
            const uint4 e = qe[c], o = qo[c];
            sq4a_word(v.x, e.x, o.x, aa, ab);
            sq4a_word(v.y, e.y, o.y, aa, ab);
            sq4a_word(v.z, e.z, o.z, aa, ab);
            sq4a_word(v.w, e.w, o.w, aa, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (KIND == K_SQ1) {
        const uint4 *qv = reinterpret_cast<const uint4 *>(qc);
        int32_t s = 0;
        for (int c = 0; c < nch; ++c) {
            const uint4 v = row[c], q = qv[c];
            s += __popc(v.x ^ q.x) + __popc(v.y ^ q.y) + __popc(v.z ^ q.z) + __popc(v.w ^ q.w);
        }
        return s;
    } else if (KIND == K_SQ2U) {
        const int nw = 4 * nch;
        uint32_t aa = 0, ab = 0;
#pragma unroll 2
        for (int c = 0; c < nch; ++c) {
            const uint4 v = row[c];
            const uint32_t *q = qc + 4 * c;
            sq2_word(v.x, q + 0, nw, aa, ab);
            sq2_word(v.y, q + 1, nw, aa, ab);
            sq2_word(v.z, q + 2, nw, aa, ab);
            sq2_word(v.w, q + 3, nw, aa, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (KIND == K_SQ4U) {
        const uint4 *ql = reinterpret_cast<const uint4 *>(qc);
        const uint4 *qh = reinterpret_cast<const uint4 *>(qc + 4 * nch);
        uint32_t aa = 0, ab = 0;
#pragma unroll 4
        for (int c = 0; c < nch; ++c) {
            const uint4 v = row[c];
            const uint4 l = ql[c], h = qh[c];
            sq4_word(v.x, l.x, h.x, aa, ab);
            sq4_word(v.y, l.y, h.y, aa, ab);
            sq4_word(v.z, l.z, h.z, aa, ab);
            sq4_word(v.w, l.w, h.w, aa, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (METRIC == M_L2) {
        const uint4 *qv = reinterpret_cast<const uint4 *>(qc);
        uint32_t aa = 0, ab = 0;
#pragma unroll 4
        for (int c = 0; c < nch; ++c) {
            const uint4 v = row[c];
            const uint4 q = qv[c];
            aa = __dp4a(v.x, v.x, aa); ab = __dp4a(v.x, q.x, ab);
            aa = __dp4a(v.y, v.y, aa); ab = __dp4a(v.y, q.y, ab);
            aa = __dp4a(v.z, v.z, aa); ab = __dp4a(v.z, q.z, ab);
            aa = __dp4a(v.w, v.w, aa); ab = __dp4a(v.w, q.w, ab);
        }
        return (int32_t)aa - 2 * (int32_t)ab;
    } else {
        const uint4 *qv = reinterpret_cast<const uint4 *>(qc);
        int32_t s = 0;
#pragma unroll 4
        for (int c = 0; c < nch; ++c) {
            const uint4 v = row[c];
            const uint4 q = qv[c];
            s = __dp4a((int)v.x, (int)q.x, s);
            s = __dp4a((int)v.y, (int)q.y, s);
            s = __dp4a((int)v.z, (int)q.z, s);
            s = __dp4a((int)v.w, (int)q.w, s);
        }
        return s;
    }
}

// Partial integer distance of chunk c (16 bytes, of nch) of a code row held in registers, against
// the query layout in shared memory: the same words sq_partial reads for that chunk.  Summed over the
// chunks of a row in any split, the partials give sq_partial's exact integer.
template <int KIND, int METRIC>
__device__ __forceinline__ int32_t sq_partial_chunk(const uint4 v, int c, int nch, const uint32_t *qc) {
    if (KIND == K_SQ4UA) {
        const uint4 e = reinterpret_cast<const uint4 *>(qc)[c];
        const uint4 o = reinterpret_cast<const uint4 *>(qc + 4 * nch)[c];
        uint32_t aa = 0, ab = 0;
        sq4a_word(v.x, e.x, o.x, aa, ab);
        sq4a_word(v.y, e.y, o.y, aa, ab);
        sq4a_word(v.z, e.z, o.z, aa, ab);
        sq4a_word(v.w, e.w, o.w, aa, ab);
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (KIND == K_SQ1) {
        const uint4 q = reinterpret_cast<const uint4 *>(qc)[c];
        return __popc(v.x ^ q.x) + __popc(v.y ^ q.y) + __popc(v.z ^ q.z) + __popc(v.w ^ q.w);
    } else if (KIND == K_SQ2U) {
        const int nw = 4 * nch;
        const uint32_t *q = qc + 4 * c;
        uint32_t aa = 0, ab = 0;
        sq2_word(v.x, q + 0, nw, aa, ab);
        sq2_word(v.y, q + 1, nw, aa, ab);
        sq2_word(v.z, q + 2, nw, aa, ab);
        sq2_word(v.w, q + 3, nw, aa, ab);
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (KIND == K_SQ4U) {
        const uint4 l = reinterpret_cast<const uint4 *>(qc)[c];
        const uint4 h = reinterpret_cast<const uint4 *>(qc + 4 * nch)[c];
        uint32_t aa = 0, ab = 0;
        sq4_word(v.x, l.x, h.x, aa, ab);
        sq4_word(v.y, l.y, h.y, aa, ab);
        sq4_word(v.z, l.z, h.z, aa, ab);
        sq4_word(v.w, l.w, h.w, aa, ab);
        return (int32_t)aa - 2 * (int32_t)ab;
    } else if (METRIC == M_L2) {
        const uint4 q = reinterpret_cast<const uint4 *>(qc)[c];
        uint32_t aa = 0, ab = 0;
        aa = __dp4a(v.x, v.x, aa); ab = __dp4a(v.x, q.x, ab);
        aa = __dp4a(v.y, v.y, aa); ab = __dp4a(v.y, q.y, ab);
        aa = __dp4a(v.z, v.z, aa); ab = __dp4a(v.z, q.z, ab);
        aa = __dp4a(v.w, v.w, aa); ab = __dp4a(v.w, q.w, ab);
        return (int32_t)aa - 2 * (int32_t)ab;
    } else {
        const uint4 q = reinterpret_cast<const uint4 *>(qc)[c];
        int32_t s = 0;
        s = __dp4a((int)v.x, (int)q.x, s);
        s = __dp4a((int)v.y, (int)q.y, s);
        s = __dp4a((int)v.z, (int)q.z, s);
        s = __dp4a((int)v.w, (int)q.w, s);
        return s;
    }
}

// Finishes a team's integer distance (all lanes of the warp must call it).
template <int KIND, int METRIC, int LPR>
__device__ __forceinline__ int32_t sq_finish(int32_t partial, int32_t qsq) {
    int32_t s = team_sum<LPR>(partial);
    if (KIND == K_SQ8U && METRIC == M_IP) return -s;
    if (KIND == K_SQ1) return s;  // Hamming distance, no query term
    return qsq + s;
}

// ---- float distance engines ---------------------------------------------------------------------
// The reference's AVX-512 kernels keep 16 lane accumulators (dimension i goes to accumulator
// i mod 16), fuse each multiply-add, and reduce the 16 lanes in a fixed tree:
//   helpa (FP32, helpa x86/l2_impl.hpp:50-71, dot_impl.hpp:52-71): a[i]+=a[i+8], +4, +2, +1;
//   glass (E5M2, glass/simd/avx512.hpp:15-38 with avx512_utils.hpp:12-15): +8, +4, then
//   (a0+a1)+(a2+a3).
// Reproducing that order gives the same bits as the x86 reference.  With LPR lanes per row each
// lane owns NA = 16/LPR consecutive accumulators; the first tree levels cross lanes by shuffles.
// FP16 and BF16 codes (helpa x86 l2a/dota_fp32_fp16, _fp32_bf16: the same 16 fused accumulators and
// helpa reduction as FP32) widen exactly to fp32 before the arithmetic.
// SQ8 (L2SqrSQ8_ext / IPSQ8_ext, glass/simd/avx512.hpp:40-75): y = fma(code + 0.5, dif, 256 min)
// against 256 q (L2: (256q - y)^2, IP: q*y), glass's reduction; `ext` = mins[16*nsteps] then difs.
// Row loads of the float engines: read-only global loads, or plain loads of a row staged in
// shared memory (SMEM).
template <bool SMEM, typename T>
__device__ __forceinline__ T ld_row(const T *p) {
    if constexpr (SMEM) return *p;
    else return __ldg(p);
}

template <int KIND, int METRIC, int LPR, bool SMEM = false>
__device__ __forceinline__ float float_dist(const uint8_t *__restrict__ row_bytes, int nsteps, int sub,
                                            const float *fq, bool active, const float *__restrict__ ext = nullptr) {
    constexpr int NA = 16 / LPR;
    constexpr bool E5M2 = KIND == K_E5M2 || KIND == K_SQ8;  // glass's reduction tree
    float a[NA];
#pragma unroll
    for (int i = 0; i < NA; ++i) a[i] = 0.0f;
    if (active) {
        for (int m = 0; m < nsteps; ++m) {
            const int base = 16 * m + NA * sub;
            float y[NA];
            if constexpr (KIND == K_FP16 || KIND == K_BF16) {
                static_assert(NA == 4 || NA == 16, "16-bit engines support 1 or 4 lanes per row");
                uint32_t ws[NA / 2];
                if constexpr (NA == 16) {
                    const uint4 *r = reinterpret_cast<const uint4 *>(row_bytes + 2 * base);
                    const uint4 w0 = ld_row<SMEM>(r), w1 = ld_row<SMEM>(r + 1);
                    ws[0] = w0.x; ws[1] = w0.y; ws[2] = w0.z; ws[3] = w0.w;
                    ws[4] = w1.x; ws[5] = w1.y; ws[6] = w1.z; ws[7] = w1.w;
                } else {
                    const uint2 w = ld_row<SMEM>(reinterpret_cast<const uint2 *>(row_bytes + 2 * base));
                    ws[0] = w.x; ws[1] = w.y;
                }
#pragma unroll
                for (int i = 0; i < NA; ++i) {
                    const uint32_t h = (ws[i >> 1] >> (16 * (i & 1))) & 0xffffu;
                    if constexpr (KIND == K_FP16) y[i] = __half2float(__ushort_as_half((unsigned short)h));
                    else y[i] = __uint_as_float(h << 16);
                }
            } else if constexpr (KIND == K_SQ8) {
                static_assert(NA == 4 || NA == 16, "SQ8 engine supports 1 or 4 lanes per row");
                uint32_t ws[NA / 4];
                if constexpr (NA == 16) {
                    const uint4 w = ld_row<SMEM>(reinterpret_cast<const uint4 *>(row_bytes + base));
                    ws[0] = w.x; ws[1] = w.y; ws[2] = w.z; ws[3] = w.w;
                } else {
                    ws[0] = ld_row<SMEM>(reinterpret_cast<const uint32_t *>(row_bytes + base));
                }
                const float *mi = ext + base, *dif = ext + 16 * nsteps + base;
#pragma unroll
                for (int i = 0; i < NA; ++i) {
                    const float c5 = (float)((ws[i >> 2] >> (8 * (i & 3))) & 0xffu) + 0.5f;
                    y[i] = fmaf(c5, __ldg(dif + i), __ldg(mi + i) * 256.0f);
                }
            } else if constexpr (KIND == K_E5M2) {
                if constexpr (NA == 16) {
                    uint4 w = ld_row<SMEM>(reinterpret_cast<const uint4 *>(row_bytes + base));
                    uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                    for (int i = 0; i < NA; ++i) y[i] = f32_of_e5m2(ws[i >> 2] >> (8 * (i & 3)));
                } else {
                    static_assert(NA == 4 || NA == 16, "E5M2 engine supports 1 or 4 lanes per row");
                    uint32_t w = ld_row<SMEM>(reinterpret_cast<const uint32_t *>(row_bytes + base));
#pragma unroll
                    for (int i = 0; i < NA; ++i) y[i] = f32_of_e5m2(w >> (8 * i));
                }
            } else {
                const float4 *r4 = reinterpret_cast<const float4 *>(row_bytes) + (base >> 2);
#pragma unroll
                for (int i = 0; i < NA / 4; ++i) {
                    float4 v = ld_row<SMEM>(r4 + i);
                    y[4 * i] = v.x; y[4 * i + 1] = v.y; y[4 * i + 2] = v.z; y[4 * i + 3] = v.w;
                }
            }
            const float4 *q4 = reinterpret_cast<const float4 *>(fq + base);
#pragma unroll
            for (int i = 0; i < NA / 4; ++i) {
                float4 q = q4[i];
                float qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    if (METRIC == M_L2) {
                        const float qv = KIND == K_SQ8 ? qq[t] * 256.0f : qq[t];
                        float df = qv - y[4 * i + t];
                        a[4 * i + t] = fmaf(df, df, a[4 * i + t]);
                    } else {
                        a[4 * i + t] = fmaf(qq[t], y[4 * i + t], a[4 * i + t]);
                    }
                }
            }
        }
    }
    // tree levels w = 8 and 4 (shared by both orders)
#pragma unroll
    for (int w = 8; w >= 4; w >>= 1) {
        if (w >= NA) {  // partner accumulator lives in another lane of the team
            const int lane_off = w / NA;
#pragma unroll
            for (int i = 0; i < NA; ++i) a[i] = a[i] + __shfl_xor_sync(kFull, a[i], lane_off);
        } else {
#pragma unroll
            for (int i = 0; i < w; ++i) a[i] = a[i] + a[i + w];
        }
    }
    // a[0..3] now hold the four partial sums s4[0..3] in every lane of the team
    float r;
    if (E5M2) {
        float x = a[0] + a[1], z = a[2] + a[3];
        r = x + z;
    } else {
        float x = a[0] + a[2], z = a[1] + a[3];
        r = x + z;
    }
    return METRIC == M_L2 ? r : -r;
}

}  // namespace gsx
