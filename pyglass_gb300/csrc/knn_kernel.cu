// Exact k-nearest-neighbour ground truth by brute force on the 5th-generation tensor cores.
//
// The recall checks of the search need the exact top-k of every query over the whole base set.
// Scores s = q.x come from bf16 tensor-core products with fp32 accumulation: each value is split
// into hi = bf16(v) and lo = bf16(v - hi), and s = qh.xh + qh.xl + ql.xh (three MMAs into one
// accumulator; one MMA when every input is exactly representable in bf16, e.g. integer data in
// 0..255, which makes the scores exact).  The approximate distances (L2: |x|^2 - 2s, IP: -s) select
// 16 candidates per query per half of every 128-column tile stream; the candidates are then
// rescored exactly in fp64 on the CUDA cores and the top k (k <= 16) kept by (distance, id).
//
// Kernel layout (one CTA per SM, persistent over (query tile, base chunk) units):
//   warp 0      TMA producer: query tile (128 x 128 bf16) and base tiles (128 x 128 bf16), 128-byte
//               swizzled, two stages
//   warp 1      TMEM allocation (all 512 columns = four 128x128 fp32 accumulators, so that the
//               tensor cores run up to four tiles ahead of the slowest epilogue warp) and the MMA issuer
//               (one elected thread, tcgen05.mma kind::f16, M=128 N=128 K=16)
//   warps 4-11  epilogue: tcgen05.ld of the accumulator (warp w reads TMEM lanes 32*(w%4).., half
//               (w-4)/4 of the columns), distance = fma(neg_scale, score, bias) for 32 columns at a
//               time, and only when their minimum beats the list's threshold the per-query candidate
//               list in shared memory
// Every mbarrier wait is bounded; on timeout the CTA records an error and leaves after its copies
// have drained, freeing its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "gsx_host.h"

namespace gsx {

namespace {

constexpr int kTM = 128;          // queries per tile (MMA M)
constexpr int kTN = 128;          // base rows per tile (MMA N)
constexpr int kKB = 64;           // bf16 elements per 128-byte swizzled K block
constexpr int kCand = 16;         // candidates kept per query per epilogue half per unit
constexpr int kBuf = 32;          // candidates a thread may hold unmerged (exact inputs)
constexpr int kEpiWarps = 8;
constexpr int kThreads = 32 * (4 + kEpiWarps);
constexpr int kAcc = 4;           // accumulators in TMEM (one CTA per SM holds all 512 columns)
constexpr uint32_t kTmemCols = kAcc * kTN;

struct KnnParams {
    int nq, N, dp;                // dp = padded dimension (multiple of 64)
    int n_mt, n_chunks, tiles_per_chunk, n_tiles;
    int passes;                   // 1 (exact bf16 inputs) or 3 (hi/lo split)
    int ip;                       // 1 = inner product
    float neg_scale;              // -2 (L2) or -1 (IP): approximate distance = bias + neg_scale * score
    const float *bias;            // n_tiles*kTN: |x|^2 (L2) or 0 (IP) per base row, +inf past N
    int *bound;                   // nq or null: order-preserving key of the smallest kCand-th approximate
                                  // distance any finished unit found for the query (exact inputs, k <= kCand)
    int32_t *cand;                // nq x n_chunks x 2 x kCand ids (-1 = none)
    float *cand_d;                // matching approximate distances
    unsigned *error;              // set on a timed-out wait
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// Waits for the phase of parity `par` to complete; false after ~2 s.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t par) {
    const uint32_t a = smem_u32(b);
    const long long t0 = clock64();
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(a), "r"(par)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > 4000000000ll) return false;
        __nanosleep(32);
    }
}

__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor of a K-major operand in the 128-byte swizzled layout: rows of
// 128 bytes, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;             // descriptor version
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}

// Instruction descriptor: kind::f16, bf16 x bf16 -> fp32, both K-major, M x N.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTN >> 3) << 17) | ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(kIdesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct __align__(1024) KnnSmem {
    // per pass p: query block [p][kb] and base block [stage][p][kb]; 1024-byte aligned blocks
    __nv_bfloat16 q[2][2][kTM * kKB];          // [hi, lo][K block]          (2 x 2 x 16 KB)
    __nv_bfloat16 x[2][2][2][kTN * kKB];       // [stage][hi, lo][K block]   (2 x 2 x 2 x 16 KB)
};

// the candidate buffers fit the low-half operand blocks of one stage each (values, then ids)
static_assert(sizeof(float) * kBuf * kEpiWarps * 32 <= sizeof(__nv_bfloat16) * 2 * kTN * kKB,
              "candidate buffer larger than a stage's low-half operand blocks");
// dynamic shared memory carve-up (bytes): operands, then candidate lists, then barriers
constexpr size_t kOpBytes = sizeof(KnnSmem);
constexpr size_t kCandBytes = (size_t)kCand * kEpiWarps * 32 * 8;
constexpr size_t kSmemBytes = kOpBytes + kCandBytes + 256 + 1024;
// the barrier area holds 4 + 2 * kAcc + 2 mbarriers and the TMEM address word
static_assert((7 + 2 * kAcc) * 8 <= 256, "barrier area too small");
// a second CTA on an SM would find no TMEM columns left: the shared memory admits one
static_assert(kSmemBytes > 228 * 1024 / 2, "two CTAs per SM would contend for TMEM");

// Inserts (dist, n) into this thread's ascending candidate list (stride kEpiWarps*32 in shared
// memory), dropping the last entry; returns the new threshold (the last entry).  Kept out of line:
// its 32 call sites in the unrolled epilogue would otherwise swamp the instruction cache.
// Order-preserving int key of a float (no NaN): keys compare as the floats do.
__device__ __forceinline__ int fkey(float f) {
    const int b = __float_as_int(f);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float fkey_inv(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

__device__ __noinline__ float cand_insert(float *cd, int32_t *ci, int slot, float dist, int n) {
    int pos = kCand - 1;
    while (pos > 0 && cd[(pos - 1) * kEpiWarps * 32 + slot] > dist) {
        cd[pos * kEpiWarps * 32 + slot] = cd[(pos - 1) * kEpiWarps * 32 + slot];
        ci[pos * kEpiWarps * 32 + slot] = ci[(pos - 1) * kEpiWarps * 32 + slot];
        --pos;
    }
    cd[pos * kEpiWarps * 32 + slot] = dist;
    ci[pos * kEpiWarps * 32 + slot] = n;
    return cd[(kCand - 1) * kEpiWarps * 32 + slot];
}

__global__ void __launch_bounds__(kThreads, 1)
knn_tc_kernel(const __grid_constant__ CUtensorMap tq_hi, const __grid_constant__ CUtensorMap tq_lo,
              const __grid_constant__ CUtensorMap tx_hi, const __grid_constant__ CUtensorMap tx_lo, KnnParams P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    KnnSmem &S = *reinterpret_cast<KnnSmem *>(base);
    float *cd = reinterpret_cast<float *>(base + kOpBytes);
    int32_t *ci = reinterpret_cast<int32_t *>(base + kOpBytes + kCandBytes / 2);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + kOpBytes + kCandBytes);
    uint64_t *full = bars, *empty = bars + 2, *tfull = bars + 4, *tempty = bars + 4 + kAcc,
             *qfull = bars + 4 + 2 * kAcc, *qempty = bars + 5 + 2 * kAcc;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 6 + 2 * kAcc);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kblocks = P.dp / kKB;  // 2 for d <= 128
    const uint32_t qbytes = (uint32_t)(P.passes == 1 ? 1 : 2) * kblocks * kTM * kKB * 2;
    const uint32_t xbytes = (uint32_t)(P.passes == 1 ? 1 : 2) * kblocks * kTN * kKB * 2;

    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < kAcc; ++i) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], kEpiWarps);
        }
        mbar_init(qfull, 1);
        mbar_init(qempty, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const int units = P.n_mt * P.n_chunks;
    bool ok = true;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0, ut = 0;
            for (int u = blockIdx.x; u < units && ok; u += gridDim.x, ++ut) {
                const int mt = u % P.n_mt, nc = u / P.n_mt;
                if (!mbar_wait(qempty, (ut & 1) ^ 1)) { ok = false; break; }
                mbar_expect_tx(qfull, qbytes);
                for (int kb = 0; kb < kblocks; ++kb) {
                    tma_2d(S.q[0][kb], &tq_hi, qfull, kb * kKB, mt * kTM);
                    if (P.passes == 3) tma_2d(S.q[1][kb], &tq_lo, qfull, kb * kKB, mt * kTM);
                }
                const int t0 = nc * P.tiles_per_chunk, t1 = min(P.n_tiles, t0 + P.tiles_per_chunk);
                for (int t = t0; t < t1; ++t, ++it) {
                    const int st = it & 1;
                    if (!mbar_wait(&empty[st], ((it >> 1) & 1) ^ 1)) { ok = false; break; }
                    mbar_expect_tx(&full[st], xbytes);
                    for (int kb = 0; kb < kblocks; ++kb) {
                        tma_2d(S.x[st][0][kb], &tx_hi, &full[st], kb * kKB, t * kTN);
                        if (P.passes == 3) tma_2d(S.x[st][1][kb], &tx_lo, &full[st], kb * kKB, t * kTN);
                    }
                }
            }
            if (!ok) atomicExch(P.error, 1u);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            uint32_t it = 0, ut = 0;
            for (int u = blockIdx.x; u < units && ok; u += gridDim.x, ++ut) {
                const int nc = u / P.n_mt;
                if (!mbar_wait(qfull, ut & 1)) { ok = false; break; }
                const int t0 = nc * P.tiles_per_chunk, t1 = min(P.n_tiles, t0 + P.tiles_per_chunk);
                for (int t = t0; t < t1; ++t, ++it) {
                    const int st = it & 1, ab = it % kAcc;
                    if (!mbar_wait(&full[st], (it >> 1) & 1)) { ok = false; break; }
                    if (!mbar_wait(&tempty[ab], ((it / kAcc) & 1) ^ 1)) { ok = false; break; }
                    fence_after();
                    const uint32_t d = tmem + (uint32_t)(ab * kTN);
                    uint32_t acc = 0;
                    // (hi, hi), then (hi, lo) and (lo, hi) for the split
                    for (int pass = 0; pass < P.passes; ++pass) {
                        const int qa = pass == 2 ? 1 : 0, xb = pass == 1 ? 1 : 0;
                        for (int kb = 0; kb < kblocks; ++kb) {
                            const uint32_t qa_addr = smem_u32(S.q[qa][kb]);
                            const uint32_t xb_addr = smem_u32(S.x[st][xb][kb]);
#pragma unroll
                            for (int ks = 0; ks < kKB / 16; ++ks) {
                                mma_bf16(d, sw128_desc(qa_addr + 32 * ks), sw128_desc(xb_addr + 32 * ks), acc);
                                acc = 1;
                            }
                        }
                    }
                    mma_commit(&empty[st]);
                    mma_commit(&tfull[ab]);
                }
                mma_commit(qempty);
            }
            if (!ok) atomicExch(P.error, 1u);
        }
    } else if (warp >= 4) {
        const int ew = warp - 4;             // 0..7
        const int quarter = warp & 3;        // TMEM lanes 32*quarter .. +31
        const int half = ew >> 2;            // columns half*kTN/2 .. +kTN/2-1
        const int slot = ew * 32 + lane;     // this thread's candidate list
        const int row = quarter * 32 + lane; // query row within the tile
        // with exact inputs (one pass) the low halves of the operand buffers are unused: they hold the
        // per-thread candidate buffers (kBuf values and ids a thread, same stride as the lists)
        const bool buffered = P.passes == 1;
        float *bd = reinterpret_cast<float *>(S.x[0][1][0]);
        int32_t *bi = reinterpret_cast<int32_t *>(S.x[1][1][0]);
        int nb = 0;
        uint32_t it = 0;
        for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
            const int mt = u % P.n_mt, nc = u / P.n_mt;
            for (int c = 0; c < kCand; ++c) {
                cd[c * kEpiWarps * 32 + slot] = __int_as_float(0x7f800000);
                ci[c * kEpiWarps * 32 + slot] = -1;
            }
            // the threshold starts at the best bound other units have published for the query, raised
            // by one ulp so that rows equal to it still enter (ties are ranked by id later), and never
            // rises above it: a full list of kCand rows at or below a value bounds the query's kCand-th
            // nearest, so no row above it can be among the top k <= kCand
            const int qs = mt * kTM + row;
            float cap = __int_as_float(0x7f800000);
            if (P.bound && qs < P.nq) {
                const int bk = *reinterpret_cast<volatile const int *>(P.bound + qs);
                const float bf = fkey_inv(bk);
                if (bf < __int_as_float(0x7f800000)) cap = nextafterf(bf, __int_as_float(0x7f800000));
            }
            float thr = cap;
            const int t0 = nc * P.tiles_per_chunk, t1 = min(P.n_tiles, t0 + P.tiles_per_chunk);
            for (int t = t0; t < t1; ++t, ++it) {
                const int ab = it % kAcc;
                if (!mbar_wait(&tfull[ab], (it / kAcc) & 1)) { ok = false; break; }
                fence_after();
                for (int c = 0; c < kTN / 64; ++c) {
                    const int n0 = t * kTN + half * (kTN / 2) + c * 32;
                    // the 32 columns' bias: the same addresses in every lane (broadcast loads), issued
                    // before the accumulator read
                    float b[32];
                    const float4 *b4 = reinterpret_cast<const float4 *>(P.bias + n0);
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const float4 x = __ldg(b4 + i);
                        b[4 * i] = x.x;
                        b[4 * i + 1] = x.y;
                        b[4 * i + 2] = x.z;
                        b[4 * i + 3] = x.w;
                    }
                    float v[32];
                    const uint32_t col0 = (uint32_t)(ab * kTN + half * (kTN / 2) + c * 32);
                    tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + col0, v);
                    // four independent partial minima keep the dependency chain short
                    float m4[4] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000),
                                   __int_as_float(0x7f800000)};
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        v[j] = fmaf(P.neg_scale, v[j], b[j]);
                        m4[j & 3] = fminf(m4[j & 3], v[j]);
                    }
                    const float dmin = fminf(fminf(m4[0], m4[1]), fminf(m4[2], m4[3]));
                    if (buffered) {
                        // exact inputs: the values that beat this thread's threshold are appended to its
                        // buffer (the threshold is only refreshed when the buffers merge), and the warp
                        // merges every lane's buffer into its list at once when one could overflow, so
                        // that no lane inserts alone while the other 31 wait
                        if (!__any_sync(0xffffffffu, dmin < thr)) continue;
                        int cnt = 0;
#pragma unroll
                        for (int j = 0; j < 32; ++j) cnt += v[j] < thr;
                        if (__any_sync(0xffffffffu, nb + cnt > kBuf)) {
                            for (int i = 0; i < nb; ++i) {
                                const float dist = bd[i * kEpiWarps * 32 + slot];
                                if (dist < thr)
                                    thr = fminf(cap, cand_insert(cd, ci, slot, dist, bi[i * kEpiWarps * 32 + slot]));
                            }
                            nb = 0;
                            __syncwarp();
                        }
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            if (v[j] < thr) {
                                bd[nb * kEpiWarps * 32 + slot] = v[j];
                                bi[nb * kEpiWarps * 32 + slot] = n0 + j;
                                ++nb;
                            }
                        }
                        continue;
                    }
                    if (!(dmin < thr)) continue;
#pragma unroll
                    for (int j = 0; j < 32; ++j) {
                        const int n = n0 + j;
                        const float dist = v[j];
                        if (dist < thr) thr = fminf(cap, cand_insert(cd, ci, slot, dist, n));
                    }
                }
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&tempty[ab]);
            }
            if (buffered) {  // the unit's last buffered values
                for (int i = 0; i < nb; ++i) {
                    const float dist = bd[i * kEpiWarps * 32 + slot];
                    if (dist < thr) thr = fminf(cap, cand_insert(cd, ci, slot, dist, bi[i * kEpiWarps * 32 + slot]));
                }
                nb = 0;
            }
            const int qi = mt * kTM + row;
            if (P.bound && qi < P.nq && ok) {
                // a full list publishes its last entry as a bound for the query's later units
                const float last = cd[(kCand - 1) * kEpiWarps * 32 + slot];
                if (last < __int_as_float(0x7f800000)) atomicMin(P.bound + qi, fkey(last));
            }
            if (qi < P.nq) {
                const size_t o = (((size_t)qi * P.n_chunks + nc) * 2 + half) * kCand;
                for (int c = 0; c < kCand; ++c) {
                    P.cand[o + c] = ci[c * kEpiWarps * 32 + slot];
                    P.cand_d[o + c] = cd[c * kEpiWarps * 32 + slot];
                }
            }
        }
        if (!ok && lane == 0) atomicExch(P.error, 1u);
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
    }
}

// hi/lo bf16 split of fp32 rows, padded to dp columns; counts values whose lo part is nonzero.
__global__ void split_bf16(const float *__restrict__ x, int64_t n, int d, int dp, __nv_bfloat16 *__restrict__ hi,
                           __nv_bfloat16 *__restrict__ lo, unsigned *inexact) {
    unsigned cnt = 0;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n * dp; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / dp;
        const int j = (int)(t - r * dp);
        const float v = j < d ? x[r * d + j] : 0.0f;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const float rest = v - __bfloat162float(h);
        hi[t] = h;
        lo[t] = __float2bfloat16_rn(rest);
        cnt += rest != 0.0f;
    }
    if (cnt) atomicAdd(inexact, cnt);
}

// bias[n] = |x_n|^2 (L2) or 0 (IP) for n < N, +inf for the padding up to total
__global__ void make_bias(const float *__restrict__ xn, int64_t N, int ip, int64_t total, float *__restrict__ bias) {
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < total; n += (int64_t)gridDim.x * blockDim.x)
        bias[n] = n < N ? (ip ? 0.0f : xn[n]) : __int_as_float(0x7f800000);
}

__global__ void row_norms(const float *__restrict__ x, int64_t n, int d, float *__restrict__ out) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double s = 0;
        for (int j = 0; j < d; ++j) s += (double)x[r * d + j] * x[r * d + j];
        out[r] = (float)s;
    }
}

// One warp per query: exact fp64 distances of the candidates, top k by (distance, id).
// Order-preserving 64-bit key of a distance (-0 taken as +0), so that the ranking below compares
// integers: GB300's fp64 pipe is a small fraction of its integer and fp32 rate.
__device__ __forceinline__ unsigned long long dist_key(double s) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(s + 0.0);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// squared L2 in fp32: four fmaf chains over dimensions j = 4i + t, summed (c0 + c1) + (c2 + c3)
__device__ __forceinline__ float l2_chain(const float *a, const float *b, int d, bool vec4) {
    float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
    int j = 0;
    if (vec4) {
        for (; j < d; j += 4) {
            const float4 x = __ldg(reinterpret_cast<const float4 *>(a + j));
            const float4 y = *reinterpret_cast<const float4 *>(b + j);
            const float t0 = x.x - y.x, t1 = x.y - y.y, t2 = x.z - y.z, t3 = x.w - y.w;
            c0 = fmaf(t0, t0, c0);
            c1 = fmaf(t1, t1, c1);
            c2 = fmaf(t2, t2, c2);
            c3 = fmaf(t3, t3, c3);
        }
    }
    for (; j < d; ++j) {
        const float t = a[j] - b[j];
        const int c = j & 3;
        if (c == 0) c0 = fmaf(t, t, c0);
        else if (c == 1) c1 = fmaf(t, t, c1);
        else if (c == 2) c2 = fmaf(t, t, c2);
        else c3 = fmaf(t, t, c3);
    }
    return (c0 + c1) + (c2 + c3);
}

// self_base >= 0: query qi is base row self_base + qi and is left out of its own list.
// fp32_l2: the distances are squared L2 in the fp32 order of l2_chain (the graph build's own
// distance), else exact-ish fp64 (the recall ground truth).
// recheck (may be null): queries whose top k may miss a row that a full candidate list dropped
// (its last kept approximate distance not clearly above the k-th distance, approximate distances
// being the L2 distance minus |q|^2), or that have fewer than k candidates, are appended to
// recheck[1..] (count in recheck[0]) for the brute-force pass.
__global__ void rescore(const float *__restrict__ base, const float *__restrict__ queries, int nq, int d, int ncand,
                        const int32_t *__restrict__ cand, const float *__restrict__ cand_d, int ip, int k,
                        int32_t *__restrict__ out_ids, float *__restrict__ out_dis, int64_t self_base, int fp32_l2,
                        int32_t *__restrict__ recheck) {
    extern __shared__ unsigned char sm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int qi = blockIdx.x * (blockDim.x >> 5) + wib;
    if (qi >= nq) return;
    const int wpb = blockDim.x >> 5;
    const size_t cs = (size_t)ncand + 1;  // per-warp stride: the candidates and one spare slot
    double *dd = reinterpret_cast<double *>(sm) + (size_t)wib * cs;
    unsigned long long *kk =
        reinterpret_cast<unsigned long long *>(reinterpret_cast<double *>(sm) + (size_t)wpb * cs) + (size_t)wib * cs;
    int32_t *id = reinterpret_cast<int32_t *>(reinterpret_cast<unsigned long long *>(sm) + (size_t)2 * wpb * cs) +
                  (size_t)wib * cs;
    const float *q = queries + (size_t)qi * d;
    const bool vec4 =
        (d & 3) == 0 && ((reinterpret_cast<uintptr_t>(base) | reinterpret_cast<uintptr_t>(queries)) & 15) == 0;
    for (int c = lane; c < ncand; c += 32) {
        int32_t n = cand[(size_t)qi * ncand + c];
        if (self_base >= 0 && n == self_base + qi) n = -1;
        double s = 0;
        if (n >= 0 && fp32_l2) {
            s = (double)l2_chain(base + (size_t)n * d, q, d, vec4);
        } else if (n >= 0) {
            // four independent fp64 chains over dimensions j = 4i + t (exact for integer-valued data;
            // otherwise within a few fp64 ulps of any other order), 16-byte loads when rows allow
            const float *x = base + (size_t)n * d;
            double a4[4] = {0.0, 0.0, 0.0, 0.0};
            int j = 0;
            if ((d & 3) == 0 && ((reinterpret_cast<uintptr_t>(base) | reinterpret_cast<uintptr_t>(queries)) & 15) == 0) {
                for (; j < d; j += 4) {
                    const float4 xv = __ldg(reinterpret_cast<const float4 *>(x + j));
                    const float4 qv = *reinterpret_cast<const float4 *>(q + j);
                    const double xs[4] = {xv.x, xv.y, xv.z, xv.w}, qs[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
                    for (int t = 0; t < 4; ++t) a4[t] += ip ? qs[t] * xs[t] : (qs[t] - xs[t]) * (qs[t] - xs[t]);
                }
            }
            for (; j < d; ++j) {
                const double a = q[j], b = x[j];
                a4[j & 3] += ip ? a * b : (a - b) * (a - b);
            }
            s = (a4[0] + a4[1]) + (a4[2] + a4[3]);
            s = ip ? -s : s;
        }
        dd[c] = n >= 0 ? s : 1e300;
        kk[c] = n >= 0 ? dist_key(s) : ~0ull;
        id[c] = n;
    }
    __syncwarp();
    for (int c = lane; c < ncand; c += 32) {
        const unsigned long long kc = kk[c];
        const double dc = dd[c];
        const int32_t ic = id[c];
        if (ic < 0) continue;
        int rank = 0;
        for (int o = 0; o < ncand; ++o) {
            const unsigned long long x = kk[o];
            const int32_t io = id[o];
            rank += io >= 0 && (x < kc || (x == kc && io < ic));
        }
        if (rank < k) {
            out_ids[(size_t)qi * k + rank] = ic;
            if (out_dis) out_dis[(size_t)qi * k + rank] = (float)dc;
        }
        if (rank == k - 1) dd[ncand] = dc;  // spare slot past this warp's candidates: the k-th distance
    }
    // fewer than k candidates: the rest of the row is empty
    int nvalid = 0;
    for (int c = lane; c < ncand; c += 32) nvalid += id[c] >= 0;
    for (int o = 16; o; o >>= 1) nvalid += __shfl_xor_sync(0xffffffffu, nvalid, o);
    for (int r = nvalid + lane; r < k; r += 32) {
        out_ids[(size_t)qi * k + r] = -1;
        if (out_dis) out_dis[(size_t)qi * k + r] = __int_as_float(0x7f800000);
    }
    if (recheck) {
        __syncwarp();
        bool flag = nvalid < k;
        if (!flag) {
            const double kth = dd[ncand];
            double qn = 0.0;
            for (int j = 0; j < d; ++j) qn += (double)q[j] * q[j];
            const double lim = kth - qn + 1e-4 * (qn + fabs(kth)) + 1e-30;
            for (int l = lane; l < ncand / kCand; l += 32) {
                const size_t last = (size_t)qi * ncand + (size_t)l * kCand + kCand - 1;
                flag |= cand[last] >= 0 && (double)cand_d[last] <= lim;
            }
        }
        if (__any_sync(0xffffffffu, flag) && lane == 0) {
            const int at = atomicAdd(recheck, 1);
            recheck[1 + at] = qi;
        }
    }
}

// keeps the k smallest (distance, id) pairs of one warp, sorted (k + 1 slots)
__device__ __forceinline__ void top_insert(float *td, int32_t *ti, int &n, int k, float dist, int32_t id, int lane) {
    if (n == k && !(dist < td[k - 1] || (dist == td[k - 1] && id < ti[k - 1]))) return;
    int pos = 0;
    for (int b = 0; b < n; b += 32) {
        const int i = b + lane;
        pos += __popc(__ballot_sync(0xffffffffu, i < n && (td[i] < dist || (td[i] == dist && ti[i] < id))));
    }
    for (int top = n; top > pos; top -= 32) {
        const int i = top - 1 - lane;
        float a = 0.0f;
        int32_t b = 0;
        if (i >= pos) {
            a = td[i];
            b = ti[i];
        }
        __syncwarp();
        if (i >= pos) {
            td[i + 1] = a;
            ti[i + 1] = b;
        }
        __syncwarp();
    }
    if (lane == 0) {
        td[pos] = dist;
        ti[pos] = id;
    }
    __syncwarp();
    if (n < k) ++n;
}

// Exact top k of listed queries by brute force over all N rows (one warp per query), in the same
// fp32 order as the rescoring; for the queries the candidate lists may have cut short, and for
// small sets.  qlist == nullptr: queries 0..nq-1.
__global__ void knn_brute(const float *__restrict__ base, int64_t N, int d, const float *__restrict__ queries,
                          const int32_t *__restrict__ qlist, int nq, int k, int64_t self_base,
                          int32_t *__restrict__ out_ids) {
    extern __shared__ unsigned char sm[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    float *td = reinterpret_cast<float *>(sm) + (size_t)wib * (k + 1);
    int32_t *ti = reinterpret_cast<int32_t *>(reinterpret_cast<float *>(sm) + (size_t)wpb * (k + 1)) +
                  (size_t)wib * (k + 1);
    const bool vec4 =
        (d & 3) == 0 && ((reinterpret_cast<uintptr_t>(base) | reinterpret_cast<uintptr_t>(queries)) & 15) == 0;
    for (int w = blockIdx.x * wpb + wib; w < nq; w += gridDim.x * wpb) {
        const int qi = qlist ? qlist[w] : w;
        const float *q = queries + (size_t)qi * d;
        int n = 0;
        for (int64_t r0 = 0; r0 < N; r0 += 32) {
            const int64_t r = r0 + lane;
            const bool ok = r < N && !(self_base >= 0 && r == self_base + qi);
            const float dist = ok ? l2_chain(base + (size_t)r * d, q, d, vec4) : 0.0f;
            const bool lt_last = n < k || dist < td[k - 1] || (dist == td[k - 1] && (int32_t)r < ti[k - 1]);
            unsigned m = __ballot_sync(0xffffffffu, ok && lt_last);
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                const float dv = __shfl_sync(0xffffffffu, dist, src);
                top_insert(td, ti, n, k, dv, (int32_t)(r0 + src), lane);
            }
        }
        for (int j = lane; j < k; j += 32) out_ids[(size_t)qi * k + j] = j < n ? ti[j] : -1;
        __syncwarp();
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_map(CUtensorMap *m, void *ptr, int64_t rows, int dp, int box_rows) {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
            return fail(GSX_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
        fn = (EncodeTiledFn)p;
    }
    cuuint64_t dims[2] = {(cuuint64_t)dp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)dp * 2};
    cuuint32_t box[2] = {(cuuint32_t)kKB, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(GSX_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return GSX_OK;
}

}  // namespace

}  // namespace gsx

using namespace gsx;

namespace gsx {

// Top k of every query over the base set by (distance, id) from the tensor-core candidate lists.
// The base is split into at least min_chunks chunks, and each 64-column half of a chunk keeps its
// kCand best candidates: exact when k <= kCand.  With fp32_l2 (the graph build's distance) larger
// k are exact too: queries for which a full list may have dropped a row of the top k are redone by
// brute force (*rechecked, may be null, counts them).  self_base >= 0 leaves base row
// self_base + qi out of query qi's list (kNN graph of the base set).
int knn_select(const float *d_base, int64_t N, int32_t d, const float *d_queries, int32_t nq, int32_t k, int32_t ip,
               int min_chunks, int64_t self_base, int fp32_l2, int32_t *d_ids, float *d_dis, int32_t *exact_inputs,
               int32_t *rechecked, cudaStream_t st) {
    if (!d_base || !d_queries || !d_ids || N <= 0 || nq <= 0 || d <= 0) return fail(GSX_ERR_INVALID, "bad arguments");
    if (k <= 0 || k > 4 * kCand) return fail(GSX_ERR_INVALID, "k must be in [1, %d]", 4 * kCand);
    if (d > 128) return fail(GSX_ERR_UNSUPPORTED, "exact kNN supports d <= 128");
    if (N > (int64_t)INT32_MAX) return fail(GSX_ERR_INVALID, "N too large");
    const int dp = 128;  // two 64-element K blocks
    DevBuf xh, xl, qh, ql, xn, bias, cand, cand_d, cnt, bnd;
    int rc;
    if ((rc = xh.ensure((size_t)N * dp * 2)) || (rc = xl.ensure((size_t)N * dp * 2)) ||
        (rc = qh.ensure((size_t)nq * dp * 2)) || (rc = ql.ensure((size_t)nq * dp * 2)) || (rc = xn.ensure((size_t)N * 4)) ||
        (rc = cnt.ensure(16)))
        return rc;
    GSX_CUDA(cudaMemsetAsync(cnt.p, 0, 16, st));
    split_bf16<<<4096, 256, 0, st>>>(d_base, N, d, dp, xh.as<__nv_bfloat16>(), xl.as<__nv_bfloat16>(), cnt.as<unsigned>());
    split_bf16<<<1024, 256, 0, st>>>(d_queries, nq, d, dp, qh.as<__nv_bfloat16>(), ql.as<__nv_bfloat16>(),
                                     cnt.as<unsigned>());
    row_norms<<<1024, 256, 0, st>>>(d_base, N, d, xn.as<float>());
    GSX_CUDA(cudaGetLastError());
    unsigned inexact = 0;
    GSX_CUDA(cudaMemcpyAsync(&inexact, cnt.p, 4, cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaStreamSynchronize(st));
    if (exact_inputs) *exact_inputs = inexact == 0;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    KnnParams P{};
    P.nq = nq;
    P.N = (int)N;
    P.dp = dp;
    P.n_mt = (nq + kTM - 1) / kTM;
    P.n_tiles = (int)((N + kTN - 1) / kTN);
    // chunks so that units cover about four waves of the SMs
    int chunks = std::max(min_chunks, (4 * nsm + P.n_mt - 1) / P.n_mt);
    chunks = std::min(std::min(chunks, P.n_tiles), 16);  // at most 512 candidates per query
    P.tiles_per_chunk = (P.n_tiles + chunks - 1) / chunks;
    P.n_chunks = (P.n_tiles + P.tiles_per_chunk - 1) / P.tiles_per_chunk;
    P.passes = inexact ? 3 : 1;
    P.ip = ip ? 1 : 0;
    P.neg_scale = ip ? -1.0f : -2.0f;
    const int64_t nbias = (int64_t)P.n_tiles * kTN;
    if ((rc = bias.ensure((size_t)nbias * 4))) return rc;
    make_bias<<<1024, 256, 0, st>>>(xn.as<float>(), N, P.ip, nbias, bias.as<float>());
    GSX_CUDA(cudaGetLastError());
    P.bias = bias.as<float>();
    const size_t ncand = (size_t)P.n_chunks * 2 * kCand;
    if ((rc = cand.ensure((size_t)nq * ncand * 4)) || (rc = cand_d.ensure((size_t)nq * ncand * 4))) return rc;
    P.cand = cand.as<int32_t>();
    P.cand_d = cand_d.as<float>();
    P.error = cnt.as<unsigned>() + 1;
    // exact inputs and k <= kCand without rechecks (the ground truth): units share per-query bounds
    P.bound = nullptr;
    if (P.passes == 1 && !fp32_l2 && self_base < 0 && k <= kCand) {
        if ((rc = bnd.ensure((size_t)nq * 4))) return rc;
        GSX_CUDA(cudaMemsetAsync(bnd.p, 0x7f, (size_t)nq * 4, st));  // key 0x7f7f7f7f: 3.4e38, above every distance
        P.bound = bnd.as<int>();
    }
    CUtensorMap mqh, mql, mxh, mxl;
    if ((rc = encode_map(&mqh, qh.p, nq, dp, kTM)) || (rc = encode_map(&mql, ql.p, nq, dp, kTM)) ||
        (rc = encode_map(&mxh, xh.p, N, dp, kTN)) || (rc = encode_map(&mxl, xl.p, N, dp, kTN)))
        return rc;
    GSX_CUDA(cudaFuncSetAttribute(knn_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes));
    const int units = P.n_mt * P.n_chunks;
    knn_tc_kernel<<<std::min(units, nsm), kThreads, kSmemBytes, st>>>(mqh, mql, mxh, mxl, P);
    GSX_CUDA(cudaGetLastError());
    const int wpb = 4;
    // one spare double per warp past the candidates (the k-th distance for the recheck)
    const size_t rs_smem = (size_t)wpb * (ncand + 1) * 20;
    if (rs_smem > 227 * 1024) return fail(GSX_ERR_UNSUPPORTED, "too many candidate lists");
    DevBuf rlist;
    int32_t *recheck = nullptr;
    if (fp32_l2) {
        if ((rc = rlist.ensure((size_t)(nq + 1) * 4))) return rc;
        GSX_CUDA(cudaMemsetAsync(rlist.p, 0, 4, st));
        recheck = rlist.as<int32_t>();
    }
    GSX_CUDA(cudaFuncSetAttribute(rescore, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rs_smem));
    rescore<<<(nq + wpb - 1) / wpb, wpb * 32, rs_smem, st>>>(d_base, d_queries, nq, d, (int)ncand, P.cand,
                                                             P.cand_d, P.ip, k, d_ids, d_dis, self_base, fp32_l2,
                                                             recheck);
    GSX_CUDA(cudaGetLastError());
    unsigned err = 0;
    GSX_CUDA(cudaMemcpyAsync(&err, cnt.as<unsigned>() + 1, 4, cudaMemcpyDeviceToHost, st));
    int32_t n_re = 0;
    if (recheck) GSX_CUDA(cudaMemcpyAsync(&n_re, recheck, 4, cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaStreamSynchronize(st));
    if (err) return fail(GSX_ERR_TIMEOUT, "tensor-core kNN kernel gave up waiting on a pipeline barrier");
    if (n_re > 0) {
        const int bw = 4;
        const size_t bs = (size_t)bw * (k + 1) * 8;
        knn_brute<<<std::min((n_re + bw - 1) / bw, 16 * nsm), bw * 32, bs, st>>>(d_base, N, d, d_queries, recheck + 1,
                                                                                n_re, k, self_base, d_ids);
        GSX_CUDA(cudaGetLastError());
        GSX_CUDA(cudaStreamSynchronize(st));
    }
    if (rechecked) *rechecked = n_re;
    return GSX_OK;
}

}  // namespace gsx

extern "C" int gsx_knn_exact(const float *d_base, int64_t N, int32_t d, const float *d_queries, int32_t nq, int32_t k,
                             int32_t ip, int32_t *d_ids, float *d_dis, int32_t *exact_inputs, void *stream) {
    try {
        if (!d_dis) return fail(GSX_ERR_INVALID, "bad arguments");
        if (k > kCand) return fail(GSX_ERR_INVALID, "k must be in [1, %d]", kCand);
        return knn_select(d_base, N, d, d_queries, nq, k, ip, 1, -1, 0, d_ids, d_dis, exact_inputs, nullptr,
                          (cudaStream_t)stream);
    } GSX_ABI_GUARD("gsx_knn_exact")
}
