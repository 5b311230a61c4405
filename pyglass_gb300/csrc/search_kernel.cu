// Launches of the batched search (search_core.cuh), the distance kernel behind ComputerImpl, and the
// per-warp shared-memory layout.  The common shapes go to the fast form in search_fast.cu.
#include "search_core.cuh"

namespace gsx {

namespace {

template <int KIND, int METRIC, int LPR>
struct DistF {
    static cudaError_t run(const IndexView &ix, int refine, const float *queries, int nq, const int32_t *ids, int m,
                           double *out, cudaStream_t st) {
        WarpLayout L;
        make_layout(ix, 2 * kMaxDegree, 0, 0, &L);
        const int wpb = 4;
        const size_t smem = (size_t)wpb * L.total;
        auto k = distance_kernel<KIND, METRIC, LPR>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<(nq + wpb - 1) / wpb, wpb * 32, smem, st>>>(ix, refine, queries, nq, ids, m, out, L);
        return cudaGetLastError();
    }
};

template <int KIND, int METRIC, int LPR>
cudaError_t launch_t(const IndexView &ix, const BatchView &bv, const LaunchCfg &cfg, cudaStream_t st) {
    const size_t smem = (size_t)cfg.warps_per_block * (size_t)cfg.L.total;
    auto k = search_kernel<KIND, METRIC, LPR>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<cfg.blocks, cfg.warps_per_block * 32, smem, st>>>(ix, bv, cfg.L);
    return cudaGetLastError();
}

template <int KIND, int METRIC, int LPR>
int occ_t(const LaunchCfg &cfg) {
    const size_t smem = (size_t)cfg.warps_per_block * (size_t)cfg.L.total;
    auto k = search_kernel<KIND, METRIC, LPR>;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, cfg.warps_per_block * 32, smem) != cudaSuccess) return 0;
    return nb;
}

template <template <int, int, int> class F, typename... A>
auto dispatch(int kind, int metric, int lpr, A &&...a) {
    const bool ip = metric == M_IP;
    switch (kind) {
        case K_SQ4UA:  // L2SqrSQ8SQ4 for both metrics (sq4ua_quant.hpp:48)
            if (lpr >= 4) return F<K_SQ4UA, M_L2, 4>::run(a...);
            if (lpr == 2) return F<K_SQ4UA, M_L2, 2>::run(a...);
            return F<K_SQ4UA, M_L2, 1>::run(a...);
        case K_SQ1:  // Hamming for both metrics (sq1_quant.hpp:64)
            if (lpr >= 4) return F<K_SQ1, M_L2, 4>::run(a...);
            if (lpr == 2) return F<K_SQ1, M_L2, 2>::run(a...);
            return F<K_SQ1, M_L2, 1>::run(a...);
        case K_SQ2U:  // L2 on codes for both metrics (sq2u_quant.hpp:55)
            if (lpr >= 4) return F<K_SQ2U, M_L2, 4>::run(a...);
            if (lpr == 2) return F<K_SQ2U, M_L2, 2>::run(a...);
            return F<K_SQ2U, M_L2, 1>::run(a...);
        case K_SQ4U:  // L2 on codes for both metrics (sq4u_quant.hpp:343)
            if (lpr >= 4) return F<K_SQ4U, M_L2, 4>::run(a...);
            if (lpr == 2) return F<K_SQ4U, M_L2, 2>::run(a...);
            return F<K_SQ4U, M_L2, 1>::run(a...);
        case K_SQ8U:
            if (ip) {
                if (lpr >= 4) return F<K_SQ8U, M_IP, 4>::run(a...);
                if (lpr == 2) return F<K_SQ8U, M_IP, 2>::run(a...);
                return F<K_SQ8U, M_IP, 1>::run(a...);
            }
            if (lpr >= 4) return F<K_SQ8U, M_L2, 4>::run(a...);
            if (lpr == 2) return F<K_SQ8U, M_L2, 2>::run(a...);
            return F<K_SQ8U, M_L2, 1>::run(a...);
        case K_E5M2:
            if (ip) return lpr == 1 ? F<K_E5M2, M_IP, 1>::run(a...) : F<K_E5M2, M_IP, 4>::run(a...);
            return lpr == 1 ? F<K_E5M2, M_L2, 1>::run(a...) : F<K_E5M2, M_L2, 4>::run(a...);
        case K_SQ8:
            if (ip) return lpr == 1 ? F<K_SQ8, M_IP, 1>::run(a...) : F<K_SQ8, M_IP, 4>::run(a...);
            return lpr == 1 ? F<K_SQ8, M_L2, 1>::run(a...) : F<K_SQ8, M_L2, 4>::run(a...);
        case K_FP16:
            if (ip) return lpr == 1 ? F<K_FP16, M_IP, 1>::run(a...) : F<K_FP16, M_IP, 4>::run(a...);
            return lpr == 1 ? F<K_FP16, M_L2, 1>::run(a...) : F<K_FP16, M_L2, 4>::run(a...);
        case K_BF16:
            if (ip) return lpr == 1 ? F<K_BF16, M_IP, 1>::run(a...) : F<K_BF16, M_IP, 4>::run(a...);
            return lpr == 1 ? F<K_BF16, M_L2, 1>::run(a...) : F<K_BF16, M_L2, 4>::run(a...);
        default:
            if (ip) return lpr == 1 ? F<K_FP32, M_IP, 1>::run(a...) : F<K_FP32, M_IP, 4>::run(a...);
            return lpr == 1 ? F<K_FP32, M_L2, 1>::run(a...) : F<K_FP32, M_L2, 4>::run(a...);
    }
}

template <int KIND, int METRIC, int LPR>
struct LaunchF {
    static cudaError_t run(const IndexView &ix, const BatchView &bv, const LaunchCfg &cfg, cudaStream_t st) {
        return launch_t<KIND, METRIC, LPR>(ix, bv, cfg, st);
    }
};
template <int KIND, int METRIC, int LPR>
struct OccF {
    static int run(const LaunchCfg &cfg) { return occ_t<KIND, METRIC, LPR>(cfg); }
};

}  // namespace

cudaError_t launch_search(const IndexView &ix, const BatchView &bv, const LaunchCfg &cfg, cudaStream_t st) {
    if (bv.gtab && search_fast_fits(ix, cfg)) return launch_search_fast(ix, bv, cfg, st);
    return dispatch<LaunchF>(ix.kind, ix.metric, cfg.lanes_per_row, ix, bv, cfg, st);
}

int search_max_blocks_per_sm(const IndexView &ix, const LaunchCfg &cfg) {
    if (search_fast_fits(ix, cfg)) return search_fast_max_blocks_per_sm(ix, cfg);
    return dispatch<OccF>(ix.kind, ix.metric, cfg.lanes_per_row, cfg);
}

cudaError_t launch_distances(const IndexView &ix, int refine, const float *queries, int nq, const int32_t *ids,
                             int m, double *out, cudaStream_t st) {
    if (nq <= 0 || m <= 0) return cudaSuccess;
    return dispatch<DistF>(ix.kind, ix.metric, 1, ix, refine, queries, nq, ids, m, out, st);
}

bool make_layout(const IndexView &ix, int cap, int table_bits, int prefetch, WarpLayout *L) {
    auto up = [](int x, int a) { return (x + a - 1) / a * a; };
    const int capa = up(cap + 1, 32);
    int off = 0;
    L->pool_key = off; off += capa * 4;
    L->pool_id = off; off += capa * 4;
    L->cand_id = off; off += kMaxDegree * 4;
    L->cand_key = off; off += kMaxDegree * 4;
    L->acc_ub = off; off += kMaxDegree * 4;
    L->acc_key = off; off += kMaxDegree * 4;
    L->acc_id = off; off += kMaxDegree * 4;
    int fq = ix.d;
    if (is_float_kind(ix.kind)) fq = fq > ix.dalign ? fq : ix.dalign;
    if (ix.has_refine) fq = fq > ix.r_dalign ? fq : ix.r_dalign;
    fq = up(fq, 16);
    L->fq = off; off += fq * 4;
    L->fq_len = fq;
    L->qc = off;
    off += up(query_code_bytes(ix.kind, ix.csize), 16);
    L->table = off;
    if (table_bits > 0) off += (1 << table_bits) * 4;
    off = up(off, 16);
    L->stage = off;
    L->stage_row = 0;
    // integer rows up to 128 bytes; E5M2 rows up to 256 bytes.  Staged rows are scored one lane per
    // row; for FP16, BF16 and SQ8 that is slower than teams of lanes reading global memory (measured on
    // 1M x 128: FP16 3.40 vs 2.84 ms at ef 128), for E5M2 it is faster (0.93 vs 1.04 ms at ef 32)
    const bool int_kind = ix.kind == K_SQ4U || ix.kind == K_SQ8U || ix.kind == K_SQ2U || ix.kind == K_SQ4UA ||
                          ix.kind == K_SQ1;
    const bool small_float = ix.kind == K_E5M2;
    L->stage_stride = 0;
    if ((int_kind || small_float) && !(prefetch & kNoStageCodes) && ix.csize <= (int_kind ? 128 : 256) &&
        ix.csize % 16 == 0) {
        // rows 16 bytes apart beyond their size: a lane's 16-byte reads of its own row then fall on
        // other banks than its neighbours' (a stride that is a multiple of 64 bytes puts four lanes of
        // every quarter warp on the same banks)
        L->stage_row = ix.csize;
        L->stage_stride = ix.csize + 16;
        off += 32 * L->stage_stride;
    }
    L->total = up(off, 16);
    L->cap = capa - 1;
    L->pool_cap = cap;
    L->table_bits = table_bits;
    L->prefetch = prefetch;
    return L->total <= 227 * 1024;
}

}  // namespace gsx
