// Internal types shared by the host runtime (gsx_api.cu) and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gsx {

// Quantizer kinds and metrics (values follow glass/quant/quant.hpp:25-43 and glass/common.hpp).
enum Kind : int {
    K_FP32 = 0, K_FP16 = 1, K_BF16 = 2, K_E5M2 = 3, K_SQ8U = 4, K_SQ8 = 5, K_SQ4U = 7, K_SQ4UA = 8, K_SQ2U = 11, K_SQ1 = 12
};

// Kinds whose codes decode to floats compared against the fp32 query (the float engines).
// Bytes of shared memory the encoded query of an integer kind takes (prepare_query's layout): two
// planes for the 4-bit kinds, four for SQ2U, the code itself for SQ8U and SQ1; 0 for float kinds.
inline int query_code_bytes(int kind, int csize) {
    switch (kind) {
        case K_SQ4U:
        case K_SQ4UA: return 2 * csize;
        case K_SQ2U: return 4 * csize;
        case K_SQ8U:
        case K_SQ1: return csize;
        default: return 0;
    }
}

// SQ8 (per-dimension affine codes) decodes each code to a float with its dimension's min and dif.
inline bool is_float_kind(int k) { return k == K_FP32 || k == K_FP16 || k == K_BF16 || k == K_E5M2 || k == K_SQ8; }
enum MetricId : int { M_L2 = 0, M_IP = 1 };

constexpr int kMaxDegree = 64;       // graph degree handled per row (two 32-wide chunks)
constexpr int kMaxCap = 1024;        // largest pool capacity max(k*factor, ef)
constexpr int kMinTableBits = 7;     // smallest visited table: 128 slots
constexpr int kGlobalOnly = 1;       // table_bits value: no shared table, visited set in global memory
constexpr int kPrefetchCodes = 1;    // tuning.prefetch bit: L1 prefetch of the predicted row's codes
constexpr int kSpeculateRow = 2;     // tuning.prefetch bit: load the predicted next row during the merge
constexpr int kPrefetchNeighbours = 4;  // tuning.prefetch bit: L1 prefetch of each neighbour's codes
                                        // before its visited check
constexpr int kNoStageCodes = 8;     // tuning.prefetch bit: do not stage neighbour code rows in shared
                                     // memory during the visited check (integer kinds with rows of at
                                     // most 128 bytes; E5M2 rows of at most 256)
constexpr int kNoBatchOrder = 16;    // tuning.prefetch bit: run large batches in index order instead of
                                     // sorted by their principal-direction projection
constexpr int kPrefetchBuckets = 32; // tuning.prefetch bit: once the next row has arrived, prefetch the
                                     // visited-table buckets of its neighbours (global tables)
constexpr int kOrderBins = 2048;     // bins of that sort

// Device-resident index, as the kernels see it.
struct IndexView {
    int32_t N, K;
    const int32_t *adj;       // N*K, -1 padded (glass/graph.hpp:26-104)
    int32_t nep;
    const int32_t *eps;
    int32_t has_hnsw, hK, hep;
    const int32_t *levels;    // N
    const int64_t *loff;      // N+1 offsets into lists
    const int32_t *lists;     // upper-level lists, levels[u]*hK per node (HNSWInitializer.hpp:64-75)
    int32_t kind, metric, d, dalign, csize;
    float p0, p1;             // calibrator (min, dif) or (max, 0)
    const uint8_t *codes;     // N*csize
    const float *sq8p;        // SQ8: mins[dalign] then difs[dalign] of its calibrator, else null
    int32_t has_refine;
    float refine_factor;
    int32_t r_dalign;
    const uint8_t *r_codes;   // N*r_dalign rows of the refine quantizer (fp32, or fp16 when r_kind = K_FP16)
    int32_t r_kind;           // K_FP32 or K_FP16
};

// One batched launch.
struct BatchView {
    const float *queries;     // nq*d fp32
    int32_t nq;
    int32_t k, ef;            // uniform values
    const int32_t *k_per;     // optional per-query k
    const int32_t *ef_per;    // optional per-query ef
    const int32_t *order;     // optional work order (a permutation of 0..nq-1)
    int32_t single;           // Searcher.search semantics: expansion limit max(k, ef)
    int32_t out_stride;
    int32_t *out_ids;
    float *out_dis;
    int32_t *cmps;            // optional per-query distance counts
    int32_t *expansions;      // optional per-query expansion counts (adjacency rows read)
    int32_t *status;          // per-query: 0 ok, 1 visited table full (query left unanswered)
    unsigned int *counter;    // work-queue head, zeroed before the launch
    unsigned int *overflow;   // number of overflowed queries
    uint32_t *gtab;           // optional global visited tables, one per warp slot: 2^gtab_bits
                              // slots of (tag << gtab_shift | id), tag 1..2^(32-gtab_shift)-1
    uint32_t *gtab_epoch;     // their query counters (zero-initialised)
    int32_t gtab_bits;
    int32_t gtab_shift;       // id bits of the graph (visited_id_bits(N))
};

// Bits that hold every node id of an n-node graph in a global visited-table slot; the remaining
// high bits tag the query that wrote the slot.
inline int visited_id_bits(int64_t n) {
    int b = 1;
    while (b < 31 && (1ll << b) < n) ++b;
    return b;
}

// Byte offsets of one warp's slice of dynamic shared memory.
struct WarpLayout {
    int pool_key, pool_id, cand_id, cand_key, acc_ub, acc_key, acc_id, fq, qc, table;
    int stage;                // 32 code rows staged by cp.async (byte offset), when stage_row > 0
    int stage_row;            // bytes per staged row (the code size), 0 = no staging
    int stage_stride;         // bytes between staged rows
    int total;                // bytes per warp (multiple of 16)
    int cap;                  // pool capacity available
    int pool_cap;             // largest pool capacity max(k * factor, ef) the launch's queries use
    int fq_len;               // floats in the fp32 query buffer
    int table_bits;           // 0 => visited table in global memory (BatchView::gtab)
    int prefetch;
};

struct LaunchCfg {
    int warps_per_block;
    int lanes_per_row;
    int blocks;
    int max_blocks;           // resident blocks of this shape on the whole GPU (spill slots / warps)
    WarpLayout L;
};

// Computes the per-warp layout; returns false if it cannot fit in shared memory.
bool make_layout(const IndexView &ix, int cap, int table_bits, int prefetch, WarpLayout *L);

// Kernel launchers (search_kernel.cu).  Return cudaGetLastError() of the launch.
cudaError_t launch_search(const IndexView &ix, const BatchView &bv, const LaunchCfg &cfg, cudaStream_t st);
int search_max_blocks_per_sm(const IndexView &ix, const LaunchCfg &cfg);
// The fast form (search_fast.cu) for integer codes staged as 64- or 128-byte rows, degree <= 32,
// visited sets in global tables only and pools of at most 256 entries; same results.
bool search_fast_fits(const IndexView &ix, const LaunchCfg &cfg);
cudaError_t launch_search_fast(const IndexView &ix, const BatchView &bv, const LaunchCfg &cfg, cudaStream_t st);
int search_fast_max_blocks_per_sm(const IndexView &ix, const LaunchCfg &cfg);

// Encoding and distance kernels (encode_kernel.cu).
cudaError_t launch_encode(int kind, int metric, const float *data, int64_t n, int d, int dalign, int csize, float p0,
                          float p1, uint8_t *out, cudaStream_t st);
cudaError_t launch_pad_rows(const float *data, int64_t n, int d, int dalign, float *out, cudaStream_t st);

// Calibration on the device (calib_kernel.cu).  Keys are order-preserving images of floats.
// launch_minmax_keys: out[0..1] = min and max key of x[0..n) (of |x| when absval); launch_radix_hist2:
// hist[0..511] = for s = 0, 1 the counts by 8-bit digit at `shift` of the keys matching prefix_s on
// mask (out and hist are device words).  float_of_key inverts a key.
cudaError_t launch_minmax_keys(const float *x, int64_t n, int absval, unsigned *out, cudaStream_t st);
cudaError_t launch_radix_hist2(const float *x, int64_t n, uint32_t prefix0, uint32_t prefix1, uint32_t mask, int shift,
                               unsigned *hist, cudaStream_t st);
float float_of_key(uint32_t k);
// SQ8's calibrator: mins[j], difs[j] = min and max-min of the j-th block of n consecutive floats of x
// (j < d; see calib_kernel.cu); entries d..dalign-1 zero.  out = mins[dalign] then difs[dalign].
cudaError_t launch_block_minmax(const float *x, int64_t n, int d, int dalign, float *out, cudaStream_t st);
cudaError_t launch_encode_sq8(const float *data, int64_t n, int d, int dalign, const float *p, uint8_t *out,
                              cudaStream_t st);

// Work order of a batch (order_kernel.cu): order[0..nq) = the queries sorted by the bin of their
// projection (q - mean) . dir; dirmean = dir[d] then mean[d]; keys = nq words of scratch.
cudaError_t launch_batch_order(const float *q, int nq, int d, const float *dirmean, float lo, float scale,
                               uint32_t *keys, int32_t *order, cudaStream_t st);
cudaError_t launch_distances(const IndexView &ix, int refine, const float *queries, int nq, const int32_t *ids,
                             int m, double *out, cudaStream_t st);

}  // namespace gsx
