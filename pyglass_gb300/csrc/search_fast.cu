// The fast form of the batched search (search_core.cuh with NCH > 0) for the shapes the benchmark
// workloads take: integer codes staged in shared memory as 64- or 128-byte rows, degree <= 32, visited
// sets in the warps' global tables only and pools of at most 256 entries.  The search and its results
// are those of the general form; the runtime tests it drops become compile-time facts, and the fresh
// staged rows are scored by teams of four lanes, which cuts the warp-instructions per launch (on
// 1M x 128 SQ4U at ef 128, 10,000 queries: 1089 M in the general form, 849 M here).
// Compiled in its own translation unit so that it builds in parallel with the general launches.
#include "search_core.cuh"

namespace gsx {

namespace {

template <int KIND, int METRIC, int NCH>
struct FastLaunch {
    static cudaError_t run(const IndexView &ix, const BatchView &bv, const LaunchCfg &cfg, cudaStream_t st) {
        const size_t smem = (size_t)cfg.warps_per_block * (size_t)cfg.L.total;
        auto k = search_kernel<KIND, METRIC, 4, NCH>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<cfg.blocks, cfg.warps_per_block * 32, smem, st>>>(ix, bv, cfg.L);
        return cudaGetLastError();
    }
};

template <int KIND, int METRIC, int NCH>
struct FastOcc {
    static int run(const LaunchCfg &cfg) {
        const size_t smem = (size_t)cfg.warps_per_block * (size_t)cfg.L.total;
        auto k = search_kernel<KIND, METRIC, 4, NCH>;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, cfg.warps_per_block * 32, smem) != cudaSuccess) return 0;
        return nb;
    }
};

// Kind and metric as the general dispatch maps them: the 4-bit, 2-bit and 1-bit kinds compare codes
// the same way under both metrics; SQ8U has an inner-product form.
template <template <int, int, int> class F, int NCH, typename... A>
auto fast_dispatch(int kind, int metric, A &&...a) {
    switch (kind) {
        case K_SQ4UA: return F<K_SQ4UA, M_L2, NCH>::run(a...);
        case K_SQ1: return F<K_SQ1, M_L2, NCH>::run(a...);
        case K_SQ2U: return F<K_SQ2U, M_L2, NCH>::run(a...);
        case K_SQ4U: return F<K_SQ4U, M_L2, NCH>::run(a...);
        default: return metric == M_IP ? F<K_SQ8U, M_IP, NCH>::run(a...) : F<K_SQ8U, M_L2, NCH>::run(a...);
    }
}

}  // namespace

bool search_fast_fits(const IndexView &ix, const LaunchCfg &cfg) {
    const bool int_kind = ix.kind == K_SQ4U || ix.kind == K_SQ8U || ix.kind == K_SQ2U || ix.kind == K_SQ4UA ||
                          ix.kind == K_SQ1;
    return int_kind && (cfg.L.stage_row == 64 || cfg.L.stage_row == 128) && ix.K <= 32 && cfg.L.table_bits == 0 &&
           cfg.L.pool_cap <= 256;
}

cudaError_t launch_search_fast(const IndexView &ix, const BatchView &bv, const LaunchCfg &cfg, cudaStream_t st) {
    if (cfg.L.stage_row == 128) return fast_dispatch<FastLaunch, 8>(ix.kind, ix.metric, ix, bv, cfg, st);
    return fast_dispatch<FastLaunch, 4>(ix.kind, ix.metric, ix, bv, cfg, st);
}

int search_fast_max_blocks_per_sm(const IndexView &ix, const LaunchCfg &cfg) {
    if (cfg.L.stage_row == 128) return fast_dispatch<FastOcc, 8>(ix.kind, ix.metric, cfg);
    return fast_dispatch<FastOcc, 4>(ix.kind, ix.metric, cfg);
}

}  // namespace gsx
