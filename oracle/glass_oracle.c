/*
 * glass_oracle.c - CPU restatement of the pyglass graph-search path (TEST INFRASTRUCTURE ONLY).
 *
 * The parity suite checks the GPU path against this file, and bench.py times it as the CPU
 * baseline.  The product never links it.  Its own parity against the unmodified reference is
 * pinned by tests/golden/ fixtures produced with oracle/_ref (see oracle/Makefile).
 *
 * Written from the reference's behaviour, in plain C: no reference source is reproduced.
 */
#include "glass_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------------ */
/* layout                                                                                      */

int go_layout(int kind, int d, int *dalign, int *csize) {
    int align, nbits;
    switch (kind) {
        case GO_SQ8U: align = 64; nbits = 8; break;   /* sq8u_quant.hpp:14  Quantizer<metric,64,8> */
        case GO_SQ4U: align = 128; nbits = 4; break;  /* sq4u_quant.hpp:13  Quantizer<metric,128,4> */
        case GO_SQ2U: align = 256; nbits = 2; break;  /* sq2u_quant.hpp:11  Quantizer<metric,256,2> */
        case GO_SQ8: align = 16; nbits = 8; break;    /* sq8_quant.hpp:15-16 Quantizer<metric,16,8> */
        case GO_SQ4UA: align = 128; nbits = 4; break; /* sq4ua_quant.hpp:13  Quantizer<metric,128,4> */
        case GO_SQ1: align = 512; nbits = 1; break;   /* sq1_quant.hpp:16   Quantizer<metric,512,1> */
        case GO_E5M2: align = 16; nbits = 8; break;   /* e5m2_quant.hpp:11  Quantizer<metric,16,8> */
        case GO_FP16: align = 16; nbits = 16; break;  /* fp16_quant.hpp:10-16 (no AVX512-FP16 build macro) */
        case GO_BF16: align = 16; nbits = 16; break;  /* bf16_quant.hpp:9-15 (no AVX512-BF16 build macro) */
        case GO_FP32: align = 16; nbits = 32; break;  /* fp32_quant.hpp:8   Quantizer<metric,16,32> */
        default: return -1;
    }
    int da = (d + align - 1) / align * align;       /* tensor.hpp:122 */
    if (dalign) *dalign = da;
    if (csize) *csize = da * nbits / 8;             /* tensor.hpp:123 */
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* calibration (quant/utils.hpp:584-603, calibrator.hpp:481-514)                               */

static int cmp_float(const void *a, const void *b) {
    float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

/* r-th smallest (0-based) of v[0..n) - quickselect on a private copy. */
static float kth_smallest(float *v, int64_t n, int64_t r) {
    int64_t lo = 0, hi = n - 1;
    while (hi > lo) {
        if (hi - lo < 32) {
            qsort(v + lo, (size_t)(hi - lo + 1), sizeof(float), cmp_float);
            return v[r];
        }
        float a = v[lo], b = v[(lo + hi) / 2], c = v[hi];
        float piv = a < b ? (b < c ? b : (a < c ? c : a)) : (a < c ? a : (b < c ? c : b));
        int64_t i = lo, j = hi;
        while (i <= j) {
            while (v[i] < piv) i++;
            while (v[j] > piv) j--;
            if (i <= j) {
                float t = v[i]; v[i] = v[j]; v[j] = t;
                i++; j--;
            }
        }
        if (r <= j) hi = j;
        else if (r >= i) lo = i;
        else return v[r];
    }
    return v[r];
}

/* find_minmax (quant/utils.hpp:584-593): with top = int64(nitems*ratio)+1, returns the top-th
 * smallest and the top-th largest value.  The product nitems*ratio is a float product. */
static void find_minmax(const float *data, int64_t nitems, float ratio, float *mn, float *mx) {
    int64_t top = (int64_t)((float)nitems * ratio) + 1;
    if (top > nitems) top = nitems;
    float *v = (float *)malloc(sizeof(float) * (size_t)nitems);
    memcpy(v, data, sizeof(float) * (size_t)nitems);
    *mn = kth_smallest(v, nitems, top - 1);
    memcpy(v, data, sizeof(float) * (size_t)nitems);
    *mx = kth_smallest(v, nitems, nitems - top);
    free(v);
}

/* find_absmax (quant/utils.hpp:595-603) with ratio 0: the largest |x|. */
static float find_absmax(const float *data, int64_t nitems) {
    float m = -INFINITY;
    for (int64_t i = 0; i < nitems; ++i) {
        float x = fabsf(data[i]);
        if (x > m) m = x;
    }
    return m;
}

/* SQ8's AffinePerDimCalibrator (calibrator.hpp:66-91) with drop ratio 0 (sq8_quant.hpp:22,29-33):
 * find_minmax_perdim (quant/utils.hpp:52-70) walks the n*d floats in order and files float i under
 * "dimension" i / n, so entry j holds the min and max of the j-th block of n consecutive floats (not
 * of column j); the arrays are then extended with zeros to dalign.  p = mins[dalign], difs[dalign]. */
static void train_sq8(const float *data, int64_t n, int d, float *p) {
    int dalign, csize;
    go_layout(GO_SQ8, d, &dalign, &csize);
    for (int j = 0; j < 2 * dalign; ++j) p[j] = 0.0f;
    for (int j = 0; j < d; ++j) {
        const float *b = data + (int64_t)j * n;
        float mn = b[0], mx = b[0];
        for (int64_t i = 1; i < n; ++i) {
            if (b[i] < mn) mn = b[i];
            if (b[i] > mx) mx = b[i];
        }
        p[j] = mn;
        p[dalign + j] = mx - mn;
    }
}

void go_train(int kind, int metric, const float *data, int64_t n, int d, float *p) {
    if (kind == GO_SQ8) { train_sq8(data, n, d, p); return; }
    p[0] = p[1] = 0.0f;
    if (kind == GO_SQ8U) {
        int64_t nitems = n * (int64_t)d;          /* sq8u_quant.hpp:240, drop_ratio 0 */
        if (metric == GO_L2) {
            float mn, mx;
            find_minmax(data, nitems, 0.0f, &mn, &mx);
            p[0] = mn;
            p[1] = mx - mn;                       /* calibrator.hpp:481-486 */
        } else {
            p[0] = find_absmax(data, nitems);     /* calibrator.hpp:511-514 */
        }
    } else if (kind == GO_SQ4UA) {
        /* sq4ua_quant.hpp:18,26: all n*d floats, drop 1% at each end */
        float mn, mx;
        find_minmax(data, n * (int64_t)d, 0.01f, &mn, &mx);
        p[0] = mn;
        p[1] = mx - mn;
    } else if (kind == GO_SQ4U || kind == GO_SQ2U) {
        /* sq4u_quant.hpp:307-309, sq2u_quant.hpp:27-29: nitems = (int64)(n*d*0.1f) - an int64*float
         * product - then drop 1% (SQ4U) or 5% (SQ2U) at each end */
        int64_t nitems = (int64_t)((float)(n * (int64_t)d) * 0.1f);
        if (nitems < 1) nitems = 1;
        float mn, mx;
        find_minmax(data, nitems, kind == GO_SQ4U ? 0.01f : 0.05f, &mn, &mx);
        p[0] = mn;
        p[1] = mx - mn;
    }
}

/* AffineCalibrator::transform (calibrator.hpp:488-492) / SymCalibrator::transform (:516-520):
 * IEEE division by dif (or max), clamp, scale, round half away from zero.  Checked against the
 * compiled reference: a reciprocal multiply differs on values that land on .5 boundaries. */
static inline int affine_code(float x, float mn, float dif, int mul) {
    x = (x - mn) / dif;
    if (x < 0.0f) x = 0.0f;
    if (x > 1.0f) x = 1.0f;
    return (int)roundf(x * (float)mul);
}

static inline int sym_code(float x, float mx, int mul) {
    x = x / mx;
    if (x < -1.0f) x = -1.0f;
    if (x > 1.0f) x = 1.0f;
    return (int)roundf(x * (float)mul);
}

/* float -> IEEE half, round to nearest even (the F16C conversion helpa::fp16 uses,
 * helpa/types.hpp:92-95), written from the IEEE-754 binary16 definition. */
static uint16_t f32_to_f16_rne(float f) {
    uint32_t x;
    memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) {                         /* inf or nan */
        return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u | ((ax >> 13) & 0x3ffu) : 0));
    }
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); /* rounds to >= 65520 -> inf */
    int32_t e = (int32_t)(ax >> 23) - 127;
    uint32_t m = ax & 0x7fffffu;
    if (e >= -14) {                                  /* normal half */
        uint32_t h = ((uint32_t)(e + 15) << 10) | (m >> 13);
        uint32_t rem = m & 0x1fffu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    if (e < -25) return (uint16_t)sign;              /* below half of the smallest subnormal */
    /* subnormal half: value = m' * 2^-24 */
    uint32_t full = m | 0x800000u;                   /* 24-bit significand, value = full*2^(e-23) */
    int shift = 13 + (-14 - e);                      /* bits dropped: value = full * 2^(e-23) = h * 2^-24 */
    uint32_t h = full >> shift;
    uint32_t rem = full & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1);
    if (rem > half || (rem == half && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

static float f16_to_f32(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    uint32_t x;
    if (e == 0) {
        if (m == 0) {
            x = sign;
        } else {                                     /* subnormal: m * 2^-24 */
            float v = (float)m * 5.9604644775390625e-08f;
            memcpy(&x, &v, 4);
            x |= sign;
        }
    } else if (e == 31) {
        x = sign | 0x7f800000u | (m << 13);
    } else {
        x = sign | ((e + 112u) << 23) | (m << 13);
    }
    float f;
    memcpy(&f, &x, 4);
    return f;
}

/* bf16 on x86: round to nearest with ties away from zero on the bit pattern, (bits + 0x8000) >> 16
 * (helpa/types.hpp:20,34-35,72-75); decode = bits << 16 (types.hpp:50-58). */
static inline uint16_t bf16_encode(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return (uint16_t)((u + 0x8000u) >> 16);
}
static inline float bf16_decode(uint16_t h) {
    uint32_t u = (uint32_t)h << 16;
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* e5m2 code = high byte of the fp16 value (glass/types.hpp:19-32); decode = byte<<8 as fp16. */
static inline uint8_t e5m2_encode(float x) { return (uint8_t)(f32_to_f16_rne(x) >> 8); }
static inline float e5m2_decode(uint8_t b) { return f16_to_f32((uint16_t)((uint16_t)b << 8)); }

/* `avail` = floats readable from x (the rest of the data array): FP16 rows read past their end, below. */
static void encode_row(int kind, int metric, const float *p, const float *x, int d, int csize, int64_t avail,
                       uint8_t *out) {
    memset(out, 0, (size_t)csize);
    if (kind == GO_SQ8U) {
        if (metric == GO_L2) {
            for (int j = 0; j < d; ++j) out[j] = (uint8_t)(int8_t)affine_code(x[j], p[0], p[1], 127);
        } else {
            for (int j = 0; j < d; ++j) out[j] = (uint8_t)(int8_t)sym_code(x[j], p[0], 127);
        }
    } else if (kind == GO_SQ1) {                     /* sq1_quant.hpp:36-42: bit j%8 of byte j/8 = (x > 0) */
        for (int j = 0; j < d; ++j)
            if (x[j] > 0) out[j / 8] |= (uint8_t)(1u << (j % 8));
    } else if (kind == GO_SQ4U || kind == GO_SQ4UA) { /* sq4u_quant.hpp:319-329: even dim -> low nibble */
        for (int j = 0; j < d; ++j) {
            uint8_t y = (uint8_t)affine_code(x[j], p[0], p[1], 15);
            out[j / 2] |= (j & 1) ? (uint8_t)(y << 4) : y;
        }
    } else if (kind == GO_SQ8) {                     /* sq8_quant.hpp:43-47: transform(x, j), mul 255 */
        const int dalign = csize;
        for (int j = 0; j < d; ++j) out[j] = (uint8_t)affine_code(x[j], p[j], p[dalign + j], 255);
    } else if (kind == GO_SQ2U) {                    /* sq2u_quant.hpp:39-52: dim j -> bits 2*(j%4) of byte j/4 */
        for (int j = 0; j < d; ++j) out[j / 4] |= (uint8_t)(affine_code(x[j], p[0], p[1], 3) << (2 * (j & 3)));
    } else if (kind == GO_E5M2) {
        for (int j = 0; j < d; ++j) out[j] = e5m2_encode(x[j]);
    } else if (kind == GO_FP16) {
        /* helpa::fp32_to_fp16 (x86/data_convert.hpp:17-38): vcvtps2ph (nearest-even) over 16-wide blocks
         * while i < d, so the block that holds the row's tail also converts the floats that follow it
         * in the data array into the padding (the next row's first dalign-d values); the last row's
         * padding would read past the array and is left zero here */
        const int dalign = csize / 2;
        for (int j = 0; j < dalign; ++j) {
            const float v = j < d ? x[j] : ((int64_t)j < avail ? x[j] : 0.0f);
            uint16_t h = (j < d || (int64_t)j < avail) ? f32_to_f16_rne(v) : 0;
            memcpy(out + 2 * j, &h, 2);
        }
    } else if (kind == GO_BF16) {                    /* BF16Quantizer::encode: bf16(float) per element */
        for (int j = 0; j < d; ++j) { uint16_t h = bf16_encode(x[j]); memcpy(out + 2 * j, &h, 2); }
    } else {
        memcpy(out, x, sizeof(float) * (size_t)d);
    }
}

void go_encode(int kind, int metric, const float *p, const float *data, int64_t n, int d, uint8_t *codes) {
    int dalign, csize;
    go_layout(kind, d, &dalign, &csize);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        encode_row(kind, metric, p, data + i * d, d, csize, (n - i) * (int64_t)d, codes + i * csize);
}

int go_encode_query(int kind, int metric, const float *p, const float *q, int d, void *out) {
    int dalign, csize;
    go_layout(kind, d, &dalign, &csize);
    if (kind == GO_SQ4UA) {                          /* sq4ua_quant.hpp:52-58 encode8: transform(x, 127), bytes */
        memset(out, 0, (size_t)dalign);
        for (int j = 0; j < d; ++j) ((uint8_t *)out)[j] = (uint8_t)affine_code(q[j], p[0], p[1], 127);
        return dalign;
    }
    if (kind == GO_SQ8U || kind == GO_SQ4U || kind == GO_SQ2U || kind == GO_SQ1) {
        encode_row(kind, metric, p, q, d, csize, d, (uint8_t *)out);
        return csize;
    }
    memset(out, 0, sizeof(float) * (size_t)dalign);  /* computer.hpp:56-59 (zero-filled align_alloc) */
    memcpy(out, q, sizeof(float) * (size_t)d);
    if (kind == GO_SQ8) {                            /* the computer's extra arguments: mins, difs */
        memcpy((float *)out + dalign, p, sizeof(float) * 2 * (size_t)dalign);
        return (int)sizeof(float) * 3 * dalign;
    }
    return (int)sizeof(float) * dalign;
}

/* ------------------------------------------------------------------------------------------ */
/* distances                                                                                   */

/* 16 lane accumulators reduced by halving (lanes i and i+8, then +4, +2, +1): the order of the
 * AVX-512 kernels l2a_fp32_fp32 (helpa x86/l2_impl.hpp:50-71), dota_fp32_fp32 (dot_impl.hpp:52-71)
 * and L2SqrE5M2/IPE5M2 (glass/simd/avx512.hpp:15-38). */
static float reduce16(float *acc) {
    for (int w = 8; w >= 1; w >>= 1)
        for (int i = 0; i < w; ++i) acc[i] = acc[i] + acc[i + w];
    return acc[0];
}

/* glass's own reduce_add_f32x16 (glass/simd/avx512_utils.hpp:12-15), used by the E5M2 kernels:
 * halve twice (i+8, i+4), then add adjacent pairs (0+1, 2+3) and the two pair sums. */
static float reduce16_glass(float *acc) {
    for (int w = 8; w >= 4; w >>= 1)
        for (int i = 0; i < w; ++i) acc[i] = acc[i] + acc[i + w];
    float a = acc[0] + acc[1], b = acc[2] + acc[3];
    return a + b;
}

double go_distance(int kind, int metric, const void *qenc, const uint8_t *code, int dalign) {
    if (kind == GO_SQ8U) {
        const int8_t *x = (const int8_t *)qenc, *y = (const int8_t *)code;
        int32_t s = 0;
        if (metric == GO_L2) {                        /* l2_s7_s7_ref (helpa ref/l2_ref.hpp:57-65) */
            for (int i = 0; i < dalign; ++i) { int32_t t = (int32_t)x[i] - (int32_t)y[i]; s += t * t; }
            return (double)s;
        }
        for (int i = 0; i < dalign; ++i) s += (int32_t)x[i] * (int32_t)y[i];   /* dot_s8_s8_ref */
        return (double)(-s);
    }
    if (kind == GO_SQ4UA) {                           /* L2SqrSQ8SQ4 (glass/simd/avx512.hpp:146-158): the 4-bit code
                                                         * c read as 8c+4 on the query's 0..127 scale */
        const uint8_t *x = (const uint8_t *)qenc, *y = code;
        int32_t s = 0;
        for (int j = 0; j < dalign / 2; ++j) {   /* dims 2j (low nibble) and 2j+1 (high nibble) */
            const int32_t t0 = (int32_t)x[2 * j] - (8 * (y[j] & 15) + 4);
            const int32_t t1 = (int32_t)x[2 * j + 1] - (8 * (y[j] >> 4) + 4);
            s += t0 * t0 + t1 * t1;
        }
        return (double)s;
    }
    if (kind == GO_SQ1) {                             /* SQ1Quantizer::distf (sq1_quant.hpp:43-62): Hamming */
        const uint8_t *x = (const uint8_t *)qenc, *y = code;
        int32_t s = 0;
        for (int i = 0; i < dalign / 8; ++i) s += __builtin_popcount((unsigned)(x[i] ^ y[i]));
        return (double)s;
    }
    if (kind == GO_SQ2U) {                            /* l2a_u2_u2 (x86/l2_impl.hpp:301-333): L2 on 2-bit codes, both metrics */
        const uint8_t *x = (const uint8_t *)qenc, *y = code;
        int32_t s = 0;
        for (int j = 0; j < dalign / 4; ++j) {   /* dims 4j+k at bits 2k of byte j */
            const int32_t a = x[j], b = y[j];
            const int32_t d0 = (a & 3) - (b & 3), d1 = ((a >> 2) & 3) - ((b >> 2) & 3);
            const int32_t d2 = ((a >> 4) & 3) - ((b >> 4) & 3), d3 = (a >> 6) - (b >> 6);
            s += d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
        }
        return (double)s;
    }
    if (kind == GO_SQ4U) {                            /* l2_u4_u4_ref (ref/l2_ref.hpp:67-77); L2 for both metrics */
        const uint8_t *x = (const uint8_t *)qenc, *y = code;
        int32_t s = 0;
        for (int j = 0; j < dalign / 2; ++j) {   /* dims 2j (low nibble) and 2j+1 (high nibble) */
            const int32_t d0 = (x[j] & 15) - (y[j] & 15), d1 = (x[j] >> 4) - (y[j] >> 4);
            s += d0 * d0 + d1 * d1;
        }
        return (double)s;
    }
    const float *q = (const float *)qenc;
    float acc[16] = {0};
    if (kind == GO_SQ8) {
        /* L2SqrSQ8_ext / IPSQ8_ext (glass/simd/avx512.hpp:40-75): y = (code + 0.5) * dif + 256 * min, in
         * 256ths of the data scale, against 256 * x, with y = fma(code + 0.5, dif, 256 * min): the
         * contraction the reference's -Ofast build applies inside its search loop (checked against the
         * compiled reference's search results).  A stand-alone compiled copy of the L2 kernel
         * reassociates 256x - y differently and lands 1-2 ulp away.  Glass's reduction. */
        const float *mi = q + dalign, *dif = q + 2 * dalign;
        for (int i = 0; i < dalign; ++i) {
            const float c5 = (float)code[i] + 0.5f;
            if (metric == GO_L2) {
                float t = q[i] * 256.0f - fmaf(c5, dif[i], mi[i] * 256.0f);
                acc[i & 15] = fmaf(t, t, acc[i & 15]);
            } else {
                acc[i & 15] = fmaf(q[i], fmaf(c5, dif[i], mi[i] * 256.0f), acc[i & 15]);
            }
        }
        float r = reduce16_glass(acc);
        return metric == GO_L2 ? (double)r : (double)(-r);
    }
    if (kind == GO_E5M2) {
        for (int i = 0; i < dalign; ++i) {
            float y = e5m2_decode(code[i]);
            /* glass/simd/avx512.hpp:15-38; -Ofast contracts the multiply and add into one fma */
            if (metric == GO_L2) { float t = q[i] - y; acc[i & 15] = fmaf(t, t, acc[i & 15]); }
            else acc[i & 15] = fmaf(q[i], y, acc[i & 15]);
        }
        float r = reduce16_glass(acc);
        return metric == GO_L2 ? (double)r : (double)(-r);
    } else if (kind == GO_FP16 || kind == GO_BF16) {
        /* l2a_fp32_fp16 / dota_fp32_fp16 and the bf16 twins (helpa x86/l2_impl.hpp:74-107, 145-181,
         * dot_impl.hpp:74-83, 139-150): the fp32 query against the exactly widened code, 16 fused
         * accumulators, helpa's reduction */
        for (int i = 0; i < dalign; ++i) {
            uint16_t h;
            memcpy(&h, code + 2 * i, 2);
            float y = kind == GO_FP16 ? f16_to_f32(h) : bf16_decode(h);
            if (metric == GO_L2) { float t = q[i] - y; acc[i & 15] = fmaf(t, t, acc[i & 15]); }
            else acc[i & 15] = fmaf(q[i], y, acc[i & 15]);
        }
    } else {
        const float *y = (const float *)code;
        for (int i = 0; i < dalign; ++i) {
            if (metric == GO_L2) { float t = q[i] - y[i]; acc[i & 15] = fmaf(t, t, acc[i & 15]); }
            else acc[i & 15] = fmaf(q[i], y[i], acc[i & 15]);
        }
    }
    float r = reduce16(acc);
    return metric == GO_L2 ? (double)r : (double)(-r);
}

/* ------------------------------------------------------------------------------------------ */
/* graph file (glass/graph.hpp:106-153, HNSWInitializer.hpp:64-86)                             */

int go_graph_load(const char *path, go_graph *g) {
    memset(g, 0, sizeof(*g));
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    int ok = 1;
    ok &= fread(&g->nep, 4, 1, f) == 1;
    if (!ok || g->nep < 0) { fclose(f); return -2; }
    g->eps = (int32_t *)malloc(sizeof(int32_t) * (size_t)(g->nep > 0 ? g->nep : 1));
    ok &= fread(g->eps, 4, (size_t)g->nep, f) == (size_t)g->nep;
    ok &= fread(&g->N, 4, 1, f) == 1;
    ok &= fread(&g->K, 4, 1, f) == 1;
    if (!ok || g->N <= 0 || g->K <= 0) { fclose(f); return -2; }
    size_t nk = (size_t)g->N * (size_t)g->K;
    g->adj = (int32_t *)malloc(sizeof(int32_t) * nk);
    ok &= fread(g->adj, 4, nk, f) == nk;
    if (!ok) { fclose(f); return -2; }
    int32_t hN;
    if (fread(&hN, 4, 1, f) == 1) {
        g->has_hnsw = 1;
        ok &= fread(&g->hK, 4, 1, f) == 1;
        ok &= fread(&g->hep, 4, 1, f) == 1;
        g->levels = (int32_t *)calloc((size_t)g->N, sizeof(int32_t));
        g->loff = (int64_t *)calloc((size_t)g->N + 1, sizeof(int64_t));
        size_t cap = 1 << 20, used = 0;
        g->lists = (int32_t *)malloc(sizeof(int32_t) * cap);
        for (int32_t i = 0; i < g->N && ok; ++i) {
            int32_t cur;
            ok &= fread(&cur, 4, 1, f) == 1;
            g->levels[i] = cur / g->hK;
            g->loff[i] = (int64_t)used;
            if (used + (size_t)cur > cap) {
                while (used + (size_t)cur > cap) cap *= 2;
                g->lists = (int32_t *)realloc(g->lists, sizeof(int32_t) * cap);
            }
            ok &= fread(g->lists + used, 4, (size_t)cur, f) == (size_t)cur;
            used += (size_t)cur;
        }
        g->loff[g->N] = (int64_t)used;
    }
    fclose(f);
    return ok ? 0 : -2;
}

/* NSG-format graph (glass/graph.hpp:224-246, Graph::load_nsg): K, the entry point, then per node
 * its neighbour count and ids; N is the number of node records the file holds and rows are padded
 * with -1 to K.  A count outside [0, K] or a truncated record is an error here, where the
 * reference would read past its row. */
int go_graph_load_nsg(const char *path, go_graph *g) {
    memset(g, 0, sizeof(*g));
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    int32_t hdr[2];
    if (fread(hdr, 4, 2, f) != 2 || hdr[0] <= 0) { fclose(f); return -2; }
    g->K = hdr[0];
    g->nep = 1;
    g->eps = (int32_t *)malloc(sizeof(int32_t));
    g->eps[0] = hdr[1];
    size_t cap = 1 << 16, n = 0;
    g->adj = (int32_t *)malloc(sizeof(int32_t) * cap * (size_t)g->K);
    int32_t c;
    while (fread(&c, 4, 1, f) == 1) {
        if (c < 0 || c > g->K) { fclose(f); return -2; }
        if (n == cap) {
            cap *= 2;
            g->adj = (int32_t *)realloc(g->adj, sizeof(int32_t) * cap * (size_t)g->K);
        }
        int32_t *row = g->adj + n * (size_t)g->K;
        if (fread(row, 4, (size_t)c, f) != (size_t)c) { fclose(f); return -2; }
        for (int32_t j = c; j < g->K; ++j) row[j] = -1;
        ++n;
    }
    fclose(f);
    if (n == 0 || n > 0x7fffffff) return -2;
    g->N = (int32_t)n;
    return 0;
}

void go_graph_free(go_graph *g) {
    free(g->adj); free(g->eps); free(g->levels); free(g->loff); free(g->lists);
    memset(g, 0, sizeof(*g));
}

/* ------------------------------------------------------------------------------------------ */
/* candidate pool (neighbor.hpp:320-433) and visited bitset (neighbor.hpp:31-79)               */

typedef struct {
    int32_t size, cur, ef, cap;
    int32_t *id;       /* bit 31 = expanded ("checked"), neighbor.hpp:416-419 */
    double *dist;      /* int32 and float distances both convert exactly */
    uint64_t *vis;
    int64_t nwords;
} pool_t;

static void pool_reset(pool_t *p, int ef, int cap) {   /* neighbor.hpp:350-359 */
    p->size = p->cur = 0;
    p->ef = ef;
    p->cap = cap;
    memset(p->vis, 0, sizeof(uint64_t) * (size_t)p->nwords);
}

static inline int vis_get(const pool_t *p, int32_t u) { return (int)((p->vis[u >> 6] >> (u & 63)) & 1u); }
static inline void vis_set(pool_t *p, int32_t u) { p->vis[u >> 6] |= (uint64_t)1 << (u & 63); }

/* insert (neighbor.hpp:382-396): upper-bound position, reject when full and dist >= last. */
static int pool_insert(pool_t *p, int32_t u, double d) {
    if (p->size == p->cap && d >= p->dist[p->size - 1]) return 0;
    int lo = 0, hi = p->size;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (p->dist[mid] > d) hi = mid; else lo = mid + 1;
    }
    int n = p->size - lo;                   /* moves into slot cap when full (array has cap+1) */
    memmove(p->id + lo + 1, p->id + lo, sizeof(int32_t) * (size_t)n);
    memmove(p->dist + lo + 1, p->dist + lo, sizeof(double) * (size_t)n);
    p->id[lo] = u;
    p->dist[lo] = d;
    if (p->size < p->cap) p->size++;
    if (lo < p->cur) p->cur = lo;
    return 1;
}

static int32_t pool_pop(pool_t *p) {        /* neighbor.hpp:398-405 */
    p->id[p->cur] |= (int32_t)0x80000000u;
    int pre = p->cur;
    while (p->cur < p->size && (p->id[p->cur] & (int32_t)0x80000000u)) p->cur++;
    return p->id[pre] & 0x7fffffff;
}

static inline int pool_has_next(const pool_t *p) { return p->cur < p->size && p->cur < p->ef; }  /* :407 */

/* ------------------------------------------------------------------------------------------ */
/* search                                                                                      */

typedef struct {
    const go_index *ix;
    uint8_t qenc[1 << 16];
    int64_t cmps;
} computer_t;

static inline double comp_dist(computer_t *c, int32_t u) {  /* computer.hpp:67-72 */
    c->cmps++;
    return go_distance(c->ix->kind, c->ix->metric, c->qenc, c->ix->codes + (int64_t)u * c->ix->csize,
                       c->ix->dalign);
}

/* Graph::initialize_search (graph.hpp:229-238) with HNSWInitializer::initialize
 * (HNSWInitializer.hpp:41-62): greedy descent; the list scanned is the one of the node held at
 * the start of each pass. */
static void initialize_search(const go_graph *g, pool_t *p, computer_t *c) {
    if (g->has_hnsw) {
        int32_t u = g->hep;
        double cur = comp_dist(c, u);
        for (int32_t level = g->levels[u]; level > 0; --level) {
            int changed = 1;
            while (changed) {
                changed = 0;
                const int32_t *list = g->lists + g->loff[u] + (int64_t)(level - 1) * g->hK;
                for (int32_t i = 0; i < g->hK && list[i] != -1; ++i) {
                    int32_t v = list[i];
                    double d = comp_dist(c, v);
                    if (d < cur) { cur = d; u = v; changed = 1; }
                }
            }
        }
        pool_insert(p, u, cur);
        vis_set(p, u);
    } else {
        for (int32_t i = 0; i < g->nep; ++i) {
            int32_t ep = g->eps[i];
            pool_insert(p, ep, comp_dist(c, ep));
            vis_set(p, ep);
        }
    }
}

/* SearchImpl2 (graph_searcher.hpp:196-224); SearchImpl1 (:161-194) visits the same nodes in the
 * same order and inserts the same distances, so one loop serves both. */
/* Prefetch distance for code rows: the reference's default `po` of 1 (graph_searcher.hpp:29), each
 * row's cache lines in full.  Only timing depends on it. */
#ifndef GO_PREFETCH_AHEAD
#define GO_PREFETCH_AHEAD 1
#endif
static void search_impl(const go_graph *g, pool_t *p, computer_t *c, int32_t *edge) {
    while (pool_has_next(p)) {
        int32_t u = pool_pop(p);
        int n = 0;
        const int32_t *row = g->adj + (int64_t)u * g->K;
        for (int32_t i = 0; i < g->K; ++i) {
            int32_t v = row[i];
            if (v == -1) break;
            if (vis_get(p, v)) continue;
            vis_set(p, v);
            edge[n++] = v;
        }
        /* prefetch the code rows of the next neighbours, as the reference does (:211-218) */
        const int64_t cs = c->ix->csize;
        const uint8_t *codes = c->ix->codes;
        for (int i = 0; i < n && i < GO_PREFETCH_AHEAD; ++i)
            for (int64_t b = 0; b < cs; b += 64) __builtin_prefetch(codes + (int64_t)edge[i] * cs + b, 0, 3);
        for (int i = 0; i < n; ++i) {
            if (i + GO_PREFETCH_AHEAD < n)
                for (int64_t b = 0; b < cs; b += 64)
                    __builtin_prefetch(codes + (int64_t)edge[i + GO_PREFETCH_AHEAD] * cs + b, 0, 3);
            pool_insert(p, edge[i], comp_dist(c, edge[i]));
        }
    }
}

typedef struct { int32_t id; float d; } nb_t;

static int nb_less(nb_t a, nb_t b) { return a.d < b.d || (a.d == b.d && a.id < b.id); }  /* neighbor.hpp:205-207 */

static float refine_dist(const go_index *ix, const float *qpad, int32_t id) {
    const int esize = ix->r_kind == GO_FP16 ? 2 : 4;
    const uint8_t *row = (const uint8_t *)ix->r_codes + (int64_t)id * ix->r_dalign * esize;
    return (float)go_distance(ix->r_kind == GO_FP16 ? GO_FP16 : GO_FP32, ix->metric, qpad, row, ix->r_dalign);
}

void go_search(const go_index *ix, const float *queries, int64_t nq, int k, int ef, const int32_t *ef_per_query,
               const int32_t *k_per_query, int single, int32_t *ids, float *dis, int64_t *cmps, int nthreads) {
    const go_graph *g = ix->g;
    int kmax = k;
    if (k_per_query)
        for (int64_t i = 0; i < nq; ++i) if (k_per_query[i] > kmax) kmax = k_per_query[i];
    int efmax = ef;
    if (ef_per_query)
        for (int64_t i = 0; i < nq; ++i) if (ef_per_query[i] > efmax) efmax = ef_per_query[i];
    int rk_max = ix->has_refine ? (int)((float)kmax * ix->refine_factor) : kmax;
    int capmax = (rk_max > efmax ? rk_max : efmax) + 1;
    if (nthreads <= 0) nthreads = omp_get_max_threads();

#pragma omp parallel num_threads(nthreads)
    {
        pool_t p;
        p.nwords = ((int64_t)g->N + 63) / 64;
        p.vis = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)p.nwords);
        p.id = (int32_t *)malloc(sizeof(int32_t) * (size_t)(capmax + 1));
        p.dist = (double *)malloc(sizeof(double) * (size_t)(capmax + 1));
        computer_t *c = (computer_t *)malloc(sizeof(computer_t));
        c->ix = ix;
        nb_t *cand = (nb_t *)malloc(sizeof(nb_t) * (size_t)(capmax + 1));
        float *qpad = (float *)malloc(sizeof(float) * (size_t)(ix->has_refine ? ix->r_dalign : 1));
        int32_t *edge = (int32_t *)malloc(sizeof(int32_t) * (size_t)g->K);

#pragma omp for schedule(dynamic)
        for (int64_t qi = 0; qi < nq; ++qi) {
            const float *q = queries + qi * ix->d;
            int kq = k_per_query ? k_per_query[qi] : k;
            int efq = ef_per_query ? ef_per_query[qi] : ef;
            /* Refiner::SearchBatch / Search: reorder_k = (int)(k * factor) (refiner.hpp:46,73) */
            int rk = ix->has_refine ? (int)((float)kq * ix->refine_factor) : kq;
            int refine = ix->has_refine && rk != kq;
            int kin = refine ? rk : kq;
            int cap = kin > efq ? kin : efq;
            /* SearchBatch resets the pool with (ef, max(k,ef)); Search with (max(k,ef), max(k,ef)) */
            int ef_expand = single ? cap : efq;
            go_encode_query(ix->kind, ix->metric, ix->kind == GO_SQ8 ? ix->pp : ix->p, q, ix->d, c->qenc);
            c->cmps = 0;
            pool_reset(&p, ef_expand, cap);
            initialize_search(g, &p, c);
            search_impl(g, &p, c, edge);
            int32_t *out_i = ids + qi * kmax;
            float *out_d = dis + qi * kmax;
            for (int j = 0; j < kmax; ++j) { out_i[j] = -1; out_d[j] = INFINITY; }
            int avail = p.size < kin ? p.size : kin;
            if (!refine) {
                for (int j = 0; j < avail; ++j) {         /* to_sorted (neighbor.hpp:421-428) */
                    out_i[j] = p.id[j] & 0x7fffffff;
                    out_d[j] = (float)p.dist[j];
                }
            } else {
                /* Refiner::RefineImpl (refiner.hpp:92-110): FP32 rescoring of the reorder_k ids,
                 * keep the k smallest by (dist, id), ascending. */
                memset(qpad, 0, sizeof(float) * (size_t)ix->r_dalign);
                memcpy(qpad, q, sizeof(float) * (size_t)ix->d);
                for (int j = 0; j < avail; ++j) {
                    int32_t id = p.id[j] & 0x7fffffff;
                    cand[j].id = id;
                    cand[j].d = refine_dist(ix, qpad, id);
                }
                /* selection of the kq smallest (insertion sort - avail <= a few hundred) */
                for (int a = 1; a < avail; ++a) {
                    nb_t x = cand[a];
                    int b = a - 1;
                    while (b >= 0 && nb_less(x, cand[b])) { cand[b + 1] = cand[b]; b--; }
                    cand[b + 1] = x;
                }
                int nout = avail < kq ? avail : kq;
                for (int j = 0; j < nout; ++j) { out_i[j] = cand[j].id; out_d[j] = cand[j].d; }
            }
            if (cmps) cmps[qi] = c->cmps;
        }
        free(p.vis); free(p.id); free(p.dist); free(c); free(cand); free(qpad); free(edge);
    }
}

/* Distances of every query to a list of rows: out[qi*m+j] = dist(query qi, row ids[qi*m+j]),
 * each query encoded as get_computer does (computer.hpp:54-63). */
void go_query_distances(int kind, int metric, const float *p, int d, const float *queries, int64_t nq,
                        const uint8_t *codes, const int32_t *ids, int m, double *out) {
    int dalign, csize;
    go_layout(kind, d, &dalign, &csize);
#pragma omp parallel
    {
        uint8_t *qenc = (uint8_t *)malloc((size_t)dalign * 12 + 64);
#pragma omp for schedule(static)
        for (int64_t qi = 0; qi < nq; ++qi) {
            go_encode_query(kind, metric, p, queries + qi * d, d, qenc);
            for (int j = 0; j < m; ++j) {
                int64_t id = ids[qi * m + j];
                out[qi * m + j] = go_distance(kind, metric, qenc, codes + id * csize, dalign);
            }
        }
        free(qenc);
    }
}
