// The C ABI of libglass_gb300 (include/glass_gb300.h): GraphSearcherBase
// (glass/searcher/searcher_base.hpp:7-19) and create_searcher (graph_searcher.hpp:256-391) over
// the device kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "gsx_host.h"

namespace gsx {

namespace {
thread_local std::string g_err;
}

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    cudaGetLastError();  // clear a sticky launch error of this thread
    return fail(e == cudaErrorMemoryAllocation ? GSX_ERR_NOMEM : GSX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int DevBuf::ensure(size_t n) {
    if (n <= bytes && p) return GSX_OK;
    release();
    size_t want = n < 256 ? 256 : n;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    bytes = want;
    return GSX_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

int SpillTables::ensure(size_t n, int b, int sh, cudaStream_t st, uint32_t **tab, uint32_t **epoch) {
    const size_t tbytes = n * ((size_t)1 << b) * 4;
    if (!buf.p || n != slots || b != bits || sh != shift) {
        int rc = buf.ensure(tbytes + n * 4);
        if (rc) return rc;
        GSX_CUDA(cudaMemsetAsync(buf.p, 0, tbytes + n * 4, st));
        slots = n;
        bits = b;
        shift = sh;
    }
    *tab = buf.as<uint32_t>();
    *epoch = reinterpret_cast<uint32_t *>(reinterpret_cast<char *>(buf.p) + tbytes);
    return GSX_OK;
}

namespace {

// quantizer_map (glass/quant/quant.hpp:25-43); operator[] on an unknown key yields FP32.
int parse_quant(const std::string &q, int *kind) {
    static const char *unsupported[] = {"SQ6", "SQ4", "SQ8P", "PQ8"};
    if (q == "SQ8U") *kind = K_SQ8U;
    else if (q == "SQ4U") *kind = K_SQ4U;
    else if (q == "SQ2U") *kind = K_SQ2U;
    else if (q == "SQ8") *kind = K_SQ8;
    else if (q == "SQ4UA") *kind = K_SQ4UA;
    else if (q == "SQ1") *kind = K_SQ1;
    else if (q == "E5M2") *kind = K_E5M2;
    else if (q == "FP16") *kind = K_FP16;
    else if (q == "BF16") *kind = K_BF16;
    else {
        for (const char *u : unsupported)
            if (q == u) return fail(GSX_ERR_UNSUPPORTED, "quantizer %s is outside the GPU search path", u);
        *kind = K_FP32;
    }
    return GSX_OK;
}

int layout(int kind, int d, int *dalign, int *csize) {
    int align = 16, nbits = 32;
    if (kind == K_SQ8U) { align = 64; nbits = 8; }
    else if (kind == K_SQ4U) { align = 128; nbits = 4; }
    else if (kind == K_SQ2U) { align = 256; nbits = 2; }  // sq2u_quant.hpp:11
    else if (kind == K_SQ8) { align = 16; nbits = 8; }    // sq8_quant.hpp:15-16
    else if (kind == K_SQ4UA) { align = 128; nbits = 4; } // sq4ua_quant.hpp:13
    else if (kind == K_SQ1) { align = 512; nbits = 1; }   // sq1_quant.hpp:16
    else if (kind == K_E5M2) { align = 16; nbits = 8; }
    // fp16_quant.hpp:10-16, bf16_quant.hpp:9-15: align 16 unless built with AVX512-FP16/BF16 macros that
    // the reference's build never defines
    else if (kind == K_FP16 || kind == K_BF16) { align = 16; nbits = 16; }
    *dalign = (d + align - 1) / align * align;  // tensor.hpp:122-123
    *csize = *dalign * nbits / 8;
    return GSX_OK;
}

// r-th smallest (0-based) of two ranks among x[0..n) on the device: radix select over the
// order-preserving float keys, 8 bits a pass, both ranks in the same sweeps.
int device_kth2(const float *x, int64_t n, int64_t r0, int64_t r1, unsigned *scratch, cudaStream_t st, float *v0,
                float *v1) {
    uint32_t prefix[2] = {0u, 0u}, mask = 0u;
    int64_t rank[2] = {r0, r1};
    std::vector<unsigned> h(512);
    for (int shift = 24; shift >= 0; shift -= 8) {
        GSX_CUDA(launch_radix_hist2(x, n, prefix[0], prefix[1], mask, shift, scratch, st));
        GSX_CUDA(cudaMemcpyAsync(h.data(), scratch, 512 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        GSX_CUDA(cudaStreamSynchronize(st));
        for (int sel = 0; sel < 2; ++sel) {
            int b = 0;
            while (b < 255 && rank[sel] >= (int64_t)h[sel * 256 + b]) rank[sel] -= h[sel * 256 + b++];
            prefix[sel] |= (uint32_t)b << shift;
        }
        mask |= 255u << shift;
    }
    *v0 = float_of_key(prefix[0]);
    *v1 = float_of_key(prefix[1]);
    return GSX_OK;
}

// Calibrator training (calibrator.hpp:481-514, quant/utils.hpp:584-603, sq8u_quant.hpp:240,
// sq4u_quant.hpp:307-309) on the base data already on the device (`x`, n*d floats).  find_minmax
// keeps the top = int64(nitems*ratio)+1 smallest / largest values; the result is the top-th
// smallest and top-th largest.
int calibrate(int kind, int metric, const float *x, int64_t n, int d, float *p, DevBuf &scratch, cudaStream_t st) {
    p[0] = p[1] = 0.0f;
    if (kind != K_SQ8U && kind != K_SQ4U && kind != K_SQ2U && kind != K_SQ4UA) return GSX_OK;
    int rc = scratch.ensure(512 * sizeof(unsigned));
    if (rc) return rc;
    unsigned *w = scratch.as<unsigned>();
    if (kind == K_SQ8U) {
        const int64_t nitems = n * d;
        unsigned mm[2];
        GSX_CUDA(launch_minmax_keys(x, nitems, metric == M_L2 ? 0 : 1, w, st));
        GSX_CUDA(cudaMemcpyAsync(mm, w, sizeof(mm), cudaMemcpyDeviceToHost, st));
        GSX_CUDA(cudaStreamSynchronize(st));
        if (metric == M_L2) {
            p[0] = float_of_key(mm[0]);
            p[1] = float_of_key(mm[1]) - p[0];
        } else {
            // the symmetric calibrator starts from 0: |x| >= 0, so the largest |x| (or 0 for all-zero data)
            p[0] = float_of_key(mm[1]);
        }
        return GSX_OK;
    }
    // SQ4U / SQ2U train on the first 10%, SQ4UA on all n*d floats (sq4ua_quant.hpp:26)
    int64_t nitems = kind == K_SQ4UA ? n * (int64_t)d : (int64_t)((float)(n * (int64_t)d) * 0.1f);
    if (nitems < 1) nitems = 1;
    // find_minmax's drop ratio: 1% for SQ4U, 5% for SQ2U (sq2u_quant.hpp:16-29)
    int64_t top = (int64_t)((float)nitems * (kind == K_SQ2U ? 0.05f : 0.01f)) + 1;  // SQ4UA: 1% as well
    if (top > nitems) top = nitems;
    float mn = 0.0f, mx = 0.0f;
    if ((rc = device_kth2(x, nitems, top - 1, nitems - top, w, st, &mn, &mx))) return rc;
    p[0] = mn;
    p[1] = mx - mn;
    return GSX_OK;
}

int set_device(const gsx_searcher *s) {
    GSX_CUDA(cudaSetDevice(s->device));
    return GSX_OK;
}

template <typename T>
int upload(DevBuf &b, const T *src, size_t n, cudaStream_t st) {
    int rc = b.ensure(n * sizeof(T));
    if (rc) return rc;
    if (n) GSX_CUDA(cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, st));
    return GSX_OK;
}

// Shared-memory visited-table size.  A query whose visited set outgrows it moves the set into its
// warp's global spill table and continues (exact), so the size trades occupancy against the
// share of queries that spill: it is sized for about twice the typical visit count (the mean
// seen on this searcher, else ef*K/2), between 2^9 and 2^13 slots.
int default_table_bits(const gsx_searcher *s, int efmax) {
    int64_t want = s->visit_avg > 0 ? (int64_t)(1.5 * s->visit_avg) : (int64_t)efmax * s->ix.K / 2;
    int bits = 9;
    while ((1ll << bits) < want && bits < 13) ++bits;
    return bits;
}

int kin_of(const gsx_searcher *s, int k) {
    const int rk = s->has_refine ? (int)((float)k * s->refine_factor) : k;
    return rk;
}

// Prepares a launch configuration for a batch whose largest k/ef are kmax/efmax.
int make_cfg(gsx_searcher *s, int kmax, int efmax, int nq, bool single, int table_bits_override, LaunchCfg *cfg) {
    const int cap = std::max(kin_of(s, kmax), efmax);
    if (cap > kMaxCap) return fail(GSX_ERR_UNSUPPORTED, "pool capacity %d (k, ef) exceeds %d", cap, kMaxCap);
    // default: the visited set lives in the warp's global table (the shared memory it would take
    // buys more resident warps instead)
    int bits = table_bits_override > 0 ? table_bits_override : (s->tuning.table_bits > 0 ? s->tuning.table_bits : kGlobalOnly);
    int wpb = single ? 1 : (s->tuning.warps_per_block > 0 ? s->tuning.warps_per_block : 4);
    int lpr = s->tuning.lanes_per_row > 0 ? s->tuning.lanes_per_row
              : (is_float_kind(s->kind) ? 4 : (s->ix.csize > 256 ? 4 : 1));
    WarpLayout L;
    if (bits == kGlobalOnly) {
        // no shared-memory table: every query keeps its visited set in its warp's global table
        if (!make_layout(s->ix, cap, 0, s->tuning.prefetch, &L))
            return fail(GSX_ERR_UNSUPPORTED, "per-query state does not fit in shared memory");
    } else {
        // shrink the table (down to the minimum) until one warp's slice fits
        while (!make_layout(s->ix, cap, bits, s->tuning.prefetch, &L) && bits > kMinTableBits) --bits;
        if (!make_layout(s->ix, cap, bits, s->tuning.prefetch, &L))
            return fail(GSX_ERR_UNSUPPORTED, "per-query state does not fit in shared memory");
    }
    while (wpb > 1 && (size_t)wpb * L.total > 227 * 1024) wpb >>= 1;
    cfg->warps_per_block = wpb;
    cfg->lanes_per_row = lpr;
    cfg->L = L;
    int per_sm = search_max_blocks_per_sm(s->ix, *cfg);
    if (per_sm < 1) per_sm = 1;
    const int want = (nq + wpb - 1) / wpb;
    cfg->max_blocks = per_sm * s->num_sms;
    cfg->blocks = std::max(1, std::min(want, cfg->max_blocks));
    return GSX_OK;
}

// Global visited-table size (4 bytes a slot, read in 32-byte buckets): the largest visit count
// seen on this searcher with 25% headroom (before any batch: half of ef*K), at the kernel's 7/8
// load limit, then one size up so that buckets rarely fill, 2^11..2^20 slots.  A query that still
// outgrows it is re-run by resolve_overflow.
// The automatic size also covers three quarters of (pool capacity x degree) visits, so that a launch
// with a larger ef than any batch seen so far (a serving mix up to ef 256 after an ef-128 batch) does
// not start on tables sized for the smaller pools.
int auto_spill_bits(const gsx_searcher *s, const LaunchCfg &cfg) {
    int64_t want = s->visit_hint > 0 ? (int64_t)s->visit_hint * 5 / 4 + s->ix.K : (int64_t)cfg.L.cap * s->ix.K / 2;
    want = std::max<int64_t>(want, (int64_t)cfg.L.pool_cap * s->ix.K * 3 / 4);
    int bits = 10;
    while ((1ll << bits) - ((1ll << bits) >> 3) < want && bits < 19) ++bits;
    return bits + 1;
}

// A size set through set_tuning is used as given (a caller may want small tables).  One picked by
// optimize (from one size below the automatic size to one above) holds for launches whose automatic
// size is at most the one it was tuned against; a launch with larger pools, or after larger visit
// counts than optimize saw, gets at least the automatic size.
int spill_bits_for(const gsx_searcher *s, const LaunchCfg &cfg) {
    if (s->tuning.spill_bits > 0 && !s->spill_from_optimize) return s->tuning.spill_bits;
    const int a = auto_spill_bits(s, cfg);
    if (s->tuning.spill_bits > 0 && a <= s->spill_auto_at_opt) return s->tuning.spill_bits;
    return s->tuning.spill_bits > a ? s->tuning.spill_bits : a;
}

// Direction of the batch order: the principal direction of the sampled base rows (power iteration
// from the all-ones vector, 30 steps, in double), their mean, and the bin scale that spreads the
// sample's projections over the order's bins with 10% margin on each side.
int batch_order_setup(gsx_searcher *s) {
    const int n = s->sample_n, d = s->ix.d;
    std::vector<double> mean(d, 0.0), v(d, 1.0 / std::sqrt((double)d)), w(d);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < d; ++j) mean[j] += s->sample[(size_t)i * d + j];
    for (int j = 0; j < d; ++j) mean[j] /= n > 0 ? n : 1;
    std::vector<double> proj(n);
    for (int it = 0; it < 30; ++it) {
        std::fill(w.begin(), w.end(), 0.0);
        for (int i = 0; i < n; ++i) {
            const float *x = &s->sample[(size_t)i * d];
            double p = 0.0;
            for (int j = 0; j < d; ++j) p += (x[j] - mean[j]) * v[j];
            for (int j = 0; j < d; ++j) w[j] += p * (x[j] - mean[j]);
        }
        double nrm = 0.0;
        for (double x : w) nrm += x * x;
        nrm = std::sqrt(nrm);
        if (!(nrm > 0.0)) break;  // no spread: keep the current direction
        for (int j = 0; j < d; ++j) v[j] = w[j] / nrm;
    }
    double lo = 0.0, hi = 0.0;
    for (int i = 0; i < n; ++i) {
        double p = 0.0;
        for (int j = 0; j < d; ++j) p += (s->sample[(size_t)i * d + j] - mean[j]) * v[j];
        lo = i == 0 || p < lo ? p : lo;
        hi = i == 0 || p > hi ? p : hi;
    }
    const double margin = 0.1 * (hi - lo);
    s->order_lo = (float)(lo - margin);
    s->order_scale = hi > lo ? (float)(kOrderBins / (hi - lo + 2 * margin)) : 0.0f;
    std::vector<float> dm(2 * (size_t)d);
    for (int j = 0; j < d; ++j) {
        dm[j] = (float)v[j];
        dm[d + j] = (float)mean[j];
    }
    int rc = upload(s->pdir, dm.data(), dm.size(), s->stream);
    if (rc) return rc;
    GSX_CUDA(cudaStreamSynchronize(s->stream));
    return GSX_OK;
}

// Enqueues one batch on `st`; nothing is synchronised.
int enqueue(gsx_searcher *s, const float *d_q, int nq, int k, int ef, const int32_t *d_ef, const int32_t *d_k,
            int kmax, int efmax, int32_t *d_ids, float *d_dis, int32_t *d_cmps, bool single, cudaStream_t st,
            const LaunchCfg *cfg_in = nullptr, int32_t *d_exp = nullptr) {
    if (nq <= 0) return GSX_OK;
    LaunchCfg cfg;
    if (cfg_in) cfg = *cfg_in;
    else {
        int rc = make_cfg(s, kmax, efmax, nq, single, 0, &cfg);
        if (rc) return rc;
    }
    int rc = s->status.ensure((size_t)nq * 4);
    if (rc) return rc;
    if ((rc = s->counters.ensure(256))) return rc;
    GSX_CUDA(cudaMemsetAsync(s->counters.p, 0, 8, st));
    BatchView bv{};
    bv.queries = d_q;
    bv.nq = nq;
    bv.k = k;
    bv.ef = ef;
    bv.k_per = d_k;
    bv.ef_per = d_ef;
    bv.order = nullptr;
    bv.single = single ? 1 : 0;
    bv.out_stride = kmax;
    bv.out_ids = d_ids;
    bv.out_dis = d_dis;
    bv.cmps = d_cmps;
    bv.expansions = d_exp;
    bv.status = s->status.as<int32_t>();
    bv.counter = s->counters.as<unsigned>();
    bv.overflow = s->counters.as<unsigned>() + 1;
    // more queries than resident warps: run them sorted along the base data's principal direction,
    // so that the queries in flight together touch nearby parts of the index
    if (!single && s->pdir.p && !(s->tuning.prefetch & kNoBatchOrder) &&
        nq > cfg.max_blocks * cfg.warps_per_block) {
        if ((rc = s->qkeys.ensure((size_t)nq * 4))) return rc;
        if ((rc = s->qorder.ensure((size_t)nq * 4))) return rc;
        GSX_CUDA(launch_batch_order(d_q, nq, s->ix.d, s->pdir.as<float>(), s->order_lo, s->order_scale,
                                    s->qkeys.as<uint32_t>(), s->qorder.as<int32_t>(), st));
        bv.order = s->qorder.as<int32_t>();
    }
    // one global visited table per resident warp of this launch shape
    const int sbits = spill_bits_for(s, cfg);
    const size_t slots = (size_t)cfg.max_blocks * cfg.warps_per_block;
    bv.gtab_shift = visited_id_bits(s->ix.N);
    if ((rc = s->spill.ensure(slots, sbits, bv.gtab_shift, st, &bv.gtab, &bv.gtab_epoch))) return rc;
    bv.gtab_bits = sbits;
    GSX_CUDA(launch_search(s->ix, bv, cfg, st));
    return GSX_OK;
}

// Re-runs the queries whose visited table overflowed with a global-memory table large enough
// for every node of the graph (exact for any ef), then patches their results in place.
int resolve_overflow(gsx_searcher *s, const float *d_q, int nq, int k, int ef, const int32_t *d_ef,
                     const int32_t *d_k, int kmax, int efmax, int32_t *d_ids, float *d_dis, int32_t *d_cmps,
                     bool single, cudaStream_t st) {
    unsigned nover = 0;
    GSX_CUDA(cudaMemcpyAsync(&nover, s->counters.as<unsigned>() + 1, 4, cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaStreamSynchronize(st));
    if (nover == 0) return GSX_OK;
    s->h_status.resize((size_t)nq);
    GSX_CUDA(cudaMemcpyAsync(s->h_status.data(), s->status.p, (size_t)nq * 4, cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaStreamSynchronize(st));
    std::vector<int32_t> redo;
    for (int i = 0; i < nq; ++i)
        if (s->h_status[i]) redo.push_back(i);
    int gbits = 12;
    while ((1ll << gbits) < 2ll * s->ix.N + 2 * kMaxDegree && gbits < 28) ++gbits;
    LaunchCfg cfg;
    int rc = make_cfg(s, kmax, efmax, (int)redo.size(), single, kMinTableBits, &cfg);
    if (rc) return rc;
    cfg.L.table_bits = 0;
    cfg.warps_per_block = 4;
    const int slots_max = 16;
    cfg.blocks = std::max(1, std::min(((int)redo.size() + 3) / 4, slots_max / 4));
    const size_t slots = (size_t)cfg.blocks * cfg.warps_per_block;
    uint32_t *gt = nullptr, *ge = nullptr;
    const int shift = visited_id_bits(s->ix.N);
    if ((rc = s->gtab.ensure(slots, gbits, shift, st, &gt, &ge))) return rc;
    if ((rc = upload(s->order, redo.data(), redo.size(), st))) return rc;
    if ((rc = s->status.ensure((size_t)nq * 4))) return rc;
    GSX_CUDA(cudaMemsetAsync(s->counters.p, 0, 8, st));
    BatchView bv{};
    bv.queries = d_q;
    bv.nq = (int)redo.size();
    bv.k = k;
    bv.ef = ef;
    bv.k_per = d_k;
    bv.ef_per = d_ef;
    bv.order = s->order.as<int32_t>();
    bv.single = single ? 1 : 0;
    bv.out_stride = kmax;
    bv.out_ids = d_ids;
    bv.out_dis = d_dis;
    bv.cmps = d_cmps;
    bv.status = s->status.as<int32_t>();
    bv.counter = s->counters.as<unsigned>();
    bv.overflow = s->counters.as<unsigned>() + 1;
    bv.gtab = gt;
    bv.gtab_epoch = ge;
    bv.gtab_bits = gbits;
    bv.gtab_shift = shift;
    GSX_CUDA(launch_search(s->ix, bv, cfg, st));
    GSX_CUDA(cudaMemcpyAsync(&nover, s->counters.as<unsigned>() + 1, 4, cudaMemcpyDeviceToHost, st));
    GSX_CUDA(cudaStreamSynchronize(st));
    if (nover) return fail(GSX_ERR_STATE, "visited table overflow persisted for %u queries", nover);
    return GSX_OK;
}

// Host-buffer batch: copies in, searches, resolves overflows, copies out, synchronises.
int host_batch(gsx_searcher *s, const float *queries, int nq, int k, const int32_t *ef_per, const int32_t *k_per,
               int kmax, int32_t *ids, float *dis, bool single) {
    if (!s->has_data) return fail(GSX_ERR_STATE, "search before set_data");
    if (nq < 0 || k <= 0 || kmax < k) return fail(GSX_ERR_INVALID, "bad nq/k (nq=%d k=%d kmax=%d)", nq, k, kmax);
    if (nq == 0) return GSX_OK;
    int rc = set_device(s);
    if (rc) return rc;
    cudaStream_t st = s->stream;
    const int d = s->ix.d;
    int efmax = s->ef;
    if (ef_per) {
        efmax = 1;
        for (int i = 0; i < nq; ++i) {
            if (ef_per[i] <= 0) return fail(GSX_ERR_INVALID, "ef must be positive");
            efmax = std::max(efmax, ef_per[i]);
        }
    }
    if (k_per)
        for (int i = 0; i < nq; ++i)
            if (k_per[i] <= 0 || k_per[i] > kmax) return fail(GSX_ERR_INVALID, "per-query k out of range");
    if ((rc = upload(s->q, queries, (size_t)nq * d, st))) return rc;
    if ((rc = s->ids.ensure((size_t)nq * kmax * 4))) return rc;
    if ((rc = s->dis.ensure((size_t)nq * kmax * 4))) return rc;
    if ((rc = s->cmps.ensure((size_t)nq * 4))) return rc;
    const int32_t *d_ef = nullptr, *d_k = nullptr;
    if (ef_per) {
        if ((rc = upload(s->efp, ef_per, (size_t)nq, st))) return rc;
        d_ef = s->efp.as<int32_t>();
    }
    if (k_per) {
        if ((rc = upload(s->kp, k_per, (size_t)nq, st))) return rc;
        d_k = s->kp.as<int32_t>();
    }
    rc = enqueue(s, s->q.as<float>(), nq, k, s->ef, d_ef, d_k, kmax, efmax, s->ids.as<int32_t>(), s->dis.as<float>(),
                 s->cmps.as<int32_t>(), single, st);
    if (rc) return rc;
    // the results and the overflow count come back together, with one wait; a batch in which a query
    // overflowed its visited table (rare) re-runs those queries and copies the results again
    s->h_cmps.resize((size_t)nq);
    unsigned nover = 0;
    for (int pass = 0; pass < 2; ++pass) {
        GSX_CUDA(cudaMemcpyAsync(ids, s->ids.p, (size_t)nq * kmax * 4, cudaMemcpyDeviceToHost, st));
        if (dis) GSX_CUDA(cudaMemcpyAsync(dis, s->dis.p, (size_t)nq * kmax * 4, cudaMemcpyDeviceToHost, st));
        GSX_CUDA(cudaMemcpyAsync(s->h_cmps.data(), s->cmps.p, (size_t)nq * 4, cudaMemcpyDeviceToHost, st));
        if (pass == 0) GSX_CUDA(cudaMemcpyAsync(&nover, s->counters.as<unsigned>() + 1, 4, cudaMemcpyDeviceToHost, st));
        GSX_CUDA(cudaStreamSynchronize(st));
        if (pass == 1 || nover == 0) break;
        rc = resolve_overflow(s, s->q.as<float>(), nq, k, s->ef, d_ef, d_k, kmax, efmax, s->ids.as<int32_t>(),
                              s->dis.as<float>(), s->cmps.as<int32_t>(), single, st);
        if (rc) return rc;
    }
    int32_t mx = 0;
    int64_t sum = 0;
    for (int i = 0; i < nq; ++i) {
        mx = std::max(mx, s->h_cmps[i]);
        sum += s->h_cmps[i];
    }
    s->visit_hint = std::max(s->visit_hint, mx);
    if (nq >= 32) s->visit_avg = (double)sum / nq;
    if (!single) s->last_batch_nq = nq;
    if (!single) {
        // SearchBatch: average distance computations (graph_searcher.hpp:156-158)
        int64_t tot = 0;
        for (int i = 0; i < nq; ++i) tot += s->h_cmps[i];
        s->last_avg_cmps = (double)tot / nq;
    }
    return GSX_OK;
}

}  // namespace

// Launch configuration of the allocation-free search (noalloc.cu): no spill tables exist there, so
// the shared-memory visited table is the largest default (2^13 slots) unless tuned.
int noalloc_make_cfg(gsx_searcher *s, int kmax, int efmax, int nq, LaunchCfg *cfg) {
    const int tb = s->tuning.table_bits >= kMinTableBits ? s->tuning.table_bits : 13;
    return make_cfg(s, kmax, efmax, nq, false, tb, cfg);
}

// Hooks of the serving loop (gsx_server.cpp).
int server_make_cfg(gsx_searcher *s, int kmax, int efmax, int nq, LaunchCfg *cfg, int *spill_bits) {
    const int rc = make_cfg(s, kmax, efmax, nq, false, 0, cfg);
    *spill_bits = spill_bits_for(s, *cfg);
    return rc;
}

int server_resolve_one(gsx_searcher *s, const float *q, int k, int ef, int32_t *ids, float *dis) {
    const int32_t efp = ef;
    const double keep = s->last_avg_cmps;
    const int rc = host_batch(s, q, 1, k, &efp, nullptr, k, ids, dis, false);
    s->last_avg_cmps = keep;
    return rc;
}

// Attaches HNSW upper levels to a host graph (HNSWInitializer layout, glass/hnsw/HNSWInitializer.hpp:22-86).
// Built on a copy and swapped in only when valid, so the graph is unchanged on any error.
int set_levels(HostGraph &h, int32_t hK, int32_t ep, const int32_t *levels, const int32_t *lists) {
    if (h.N == 0) return fail(GSX_ERR_STATE, "graph is empty");
    HostGraph t = h;
    t.has_hnsw = 1;
    t.hK = hK;
    t.hep = ep;
    t.levels.assign(levels, levels + t.N);
    t.loff.assign((size_t)t.N + 1, 0);
    for (int32_t u = 0; u < t.N; ++u) {
        if (t.levels[u] < 0) return fail(GSX_ERR_INVALID, "negative level for node %d", u);
        t.loff[u + 1] = t.loff[u] + (int64_t)t.levels[u] * hK;
    }
    if (t.loff[t.N] > 0 && !lists) return fail(GSX_ERR_INVALID, "null level lists");
    t.lists.assign(lists, lists + t.loff[t.N]);
    const int rc = validate_graph(t);
    if (rc) return rc;
    h = std::move(t);
    return GSX_OK;
}

}  // namespace gsx

using namespace gsx;

extern "C" {

const char *gsx_last_error(void) { return g_err.c_str(); }

const char *gsx_version(void) { return "glass-gb300 0.1.0 (sm_103a)"; }

int gsx_device_count(void) {
    try {
        int n = 0;
        if (cudaGetDeviceCount(&n) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
        return n;
    } GSX_ABI_GUARD("gsx_device_count")
}

int gsx_graph_load(const char *filename, const char *format, gsx_graph **out) {
    try {
        if (!filename || !out) return fail(GSX_ERR_INVALID, "null argument");
        std::unique_ptr<gsx_graph> g(new gsx_graph);
        int rc = graph_load(filename, format, g->g);
        if (rc) return rc;
        *out = g.release();
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_graph_load")
}

int gsx_graph_create(const int32_t *adj, int32_t N, int32_t K, const int32_t *eps, int32_t nep, gsx_graph **out) {
    try {
        if (!adj || !out || N <= 0 || K <= 0 || nep < 0 || (nep && !eps)) return fail(GSX_ERR_INVALID, "bad graph arguments");
        if (K > kMaxDegree) return fail(GSX_ERR_UNSUPPORTED, "graph degree %d exceeds %d", K, kMaxDegree);
        std::unique_ptr<gsx_graph> g(new gsx_graph);
        g->g.N = N;
        g->g.K = K;
        g->g.adj.assign(adj, adj + (size_t)N * K);
        g->g.eps.assign(eps, eps + nep);
        int rc = validate_graph(g->g);
        if (rc) return rc;
        *out = g.release();
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_graph_create")
}

int gsx_graph_set_levels(gsx_graph *g, int32_t hK, int32_t ep, const int32_t *levels, const int32_t *lists) {
    try {
        if (!g || !levels || (hK <= 0)) return fail(GSX_ERR_INVALID, "bad level arguments");
        if (hK > kMaxDegree) return fail(GSX_ERR_UNSUPPORTED, "HNSW level degree %d unsupported", hK);
        return set_levels(g->g, hK, ep, levels, lists);
    } GSX_ABI_GUARD("gsx_graph_set_levels")
}

int gsx_graph_save(const gsx_graph *g, const char *filename) {
    try {
        if (!g || !filename) return fail(GSX_ERR_INVALID, "null argument");
        if (g->g.N == 0) return fail(GSX_ERR_STATE, "graph is empty (moved into a searcher?)");
        return graph_save(g->g, filename);
    } GSX_ABI_GUARD("gsx_graph_save")
}

int gsx_graph_info(const gsx_graph *g, int32_t *N, int32_t *K, int32_t *nep, int32_t *has_hnsw) {
    try {
        if (!g) return fail(GSX_ERR_INVALID, "null graph");
        if (N) *N = g->g.N;
        if (K) *K = g->g.K;
        if (nep) *nep = (int32_t)g->g.eps.size();
        if (has_hnsw) *has_hnsw = g->g.has_hnsw;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_graph_info")
}

int gsx_graph_adjacency(const gsx_graph *g, int32_t *adj_out) {
    try {
        if (!g || !adj_out) return fail(GSX_ERR_INVALID, "null argument");
        std::memcpy(adj_out, g->g.adj.data(), g->g.adj.size() * 4);
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_graph_adjacency")
}

int gsx_graph_eps(const gsx_graph *g, int32_t *eps_out) {
    try {
        if (!g || !eps_out) return fail(GSX_ERR_INVALID, "null argument");
        std::memcpy(eps_out, g->g.eps.data(), g->g.eps.size() * 4);
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_graph_eps")
}

void gsx_graph_destroy(gsx_graph *g) { delete g; }

int gsx_searcher_create(gsx_graph *graph, const char *metric, const char *quantizer, const char *refine_quant,
                        int device, gsx_searcher **out) {
    try {
        if (!graph || !out) return fail(GSX_ERR_INVALID, "null argument");
        if (graph->g.N == 0) return fail(GSX_ERR_STATE, "graph is empty (already moved into a searcher?)");
        int ndev = gsx_device_count();
        if (ndev == 0) return fail(GSX_ERR_CUDA, "no CUDA device is visible");
        if (device < 0 || device >= ndev) return fail(GSX_ERR_INVALID, "device %d out of range", device);
        int kind;
        int rc = parse_quant(quantizer ? quantizer : "", &kind);
        if (rc) return rc;
        const std::string rq = refine_quant ? refine_quant : "";
        // get_refine_factor (graph_searcher.hpp:227-238): 1.5 for SQ8U/SQ8/SQ4U, 3 for SQ2U, 1.0 otherwise (in which
        // case the Refiner forwards to the inner searcher unchanged, refiner.hpp:47-50)
        const float factor = (kind == K_SQ2U || kind == K_SQ1)                                           ? 3.0f
                             : (kind == K_SQ8U || kind == K_SQ4U || kind == K_SQ8 || kind == K_SQ4UA) ? 1.5f
                                                                                                      : 1.0f;
        // make_refiner (graph_searcher.hpp:240-254): FP16 -> FP16 store; FP32 or a name the quantizer map
        // does not know -> FP32 store; SQ8U / SQ8 -> their own refiners; any other known name -> none
        int rkind = K_FP32;
        bool refiner = false;
        if (!rq.empty()) {
            static const char *no_refiner[] = {"BF16", "E5M2", "SQ6", "SQ4U", "SQ4UA", "SQ4", "SQ8P", "SQ1", "SQ2U", "PQ8"};
            refiner = true;
            if (rq == "FP16") rkind = K_FP16;
            for (const char *u : no_refiner)
                if (rq == u) refiner = false;
            if ((rq == "SQ8U" || rq == "SQ8") && factor != 1.0f)
                return fail(GSX_ERR_UNSUPPORTED, "refine quantizer %s is outside the GPU search path", rq.c_str());
            if (rq == "SQ8U" || rq == "SQ8") refiner = false;  // factor 1: the refiner only forwards
        }
        if (kind == K_SQ1 && !(metric && std::string(metric) == "IP"))  // graph_searcher.hpp:362-369
            return fail(GSX_ERR_UNSUPPORTED, "SQ1 searchers exist for the IP metric only");
        auto *s = new gsx_searcher;
        s->kind = kind;
        // metric_map (common.hpp:13-19): unknown names fall on the default-constructed L2
        s->metric = (metric && std::string(metric) == "IP") ? M_IP : M_L2;
        s->has_refine = (refiner && factor != 1.0f) ? 1 : 0;
        s->r_kind = rkind;
        s->refine_factor = factor;
        s->device = device;
        s->graph = std::move(graph->g);  // the Python Graph is moved from (python/bindings.cc:98)
        graph->g = HostGraph();
        auto bad = [&](int code) {
            gsx_searcher_destroy(s);
            return code;
        };
        if ((rc = set_device(s))) return bad(rc);
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return bad(cuda_fail(e, "cudaStreamCreate"));
        cudaEventCreate(&s->ev0);
        cudaEventCreate(&s->ev1);
        cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, device);
        const HostGraph &g = s->graph;
        if ((rc = upload(s->adj, g.adj.data(), g.adj.size(), s->stream))) return bad(rc);
        if ((rc = upload(s->eps, g.eps.data(), g.eps.size(), s->stream))) return bad(rc);
        if (g.has_hnsw) {
            if ((rc = upload(s->levels, g.levels.data(), g.levels.size(), s->stream))) return bad(rc);
            if ((rc = upload(s->loff, g.loff.data(), g.loff.size(), s->stream))) return bad(rc);
            if ((rc = upload(s->lists, g.lists.data(), std::max<size_t>(g.lists.size(), 1), s->stream))) return bad(rc);
        }
        e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) return bad(cuda_fail(e, "graph upload"));
        IndexView &ix = s->ix;
        ix.N = g.N;
        ix.K = g.K;
        ix.adj = s->adj.as<int32_t>();
        ix.nep = (int32_t)g.eps.size();
        ix.eps = s->eps.as<int32_t>();
        ix.has_hnsw = g.has_hnsw;
        ix.hK = g.hK;
        ix.hep = g.hep;
        ix.levels = s->levels.as<int32_t>();
        ix.loff = s->loff.as<int64_t>();
        ix.lists = s->lists.as<int32_t>();
        ix.kind = kind;
        ix.metric = s->metric;
        ix.has_refine = s->has_refine;
        ix.refine_factor = factor;
        *out = s;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_create")
}

void gsx_searcher_destroy(gsx_searcher *s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (DevBuf *b : {&s->adj, &s->eps, &s->levels, &s->loff, &s->lists, &s->codes, &s->r_codes, &s->sq8p, &s->q, &s->ids,
                      &s->dis, &s->status, &s->cmps, &s->efp, &s->kp, &s->order, &s->counters, &s->gtab.buf,
                      &s->spill.buf, &s->dist_out, &s->dist_ids, &s->pdir, &s->qkeys, &s->qorder})
        b->release();
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int gsx_searcher_set_data(gsx_searcher *s, const float *data, int32_t n, int32_t dim) {
    try {
        if (!s || !data) return fail(GSX_ERR_INVALID, "null argument");
        if (dim <= 0 || n <= 0) return fail(GSX_ERR_INVALID, "bad data shape %d x %d", n, dim);
        if (n < s->ix.N) return fail(GSX_ERR_INVALID, "data has %d rows but the graph has %d nodes", n, s->ix.N);
        int rc = set_device(s);
        if (rc) return rc;
        IndexView &ix = s->ix;
        ix.d = dim;
        layout(s->kind, dim, &ix.dalign, &ix.csize);
        cudaStream_t st = s->stream;
        DevBuf raw, scratch;
        if ((rc = upload(raw, data, (size_t)n * dim, st))) return rc;
        float p[2];
        if ((rc = calibrate(s->kind, s->metric, raw.as<float>(), n, dim, p, scratch, st))) return rc;
        ix.p0 = p[0];
        ix.p1 = p[1];
        if ((rc = s->codes.ensure((size_t)n * ix.csize))) return rc;
        ix.sq8p = nullptr;
        if (s->kind == K_FP32) {
            GSX_CUDA(launch_pad_rows(raw.as<float>(), n, dim, ix.dalign, s->codes.as<float>(), st));
        } else if (s->kind == K_SQ8) {
            // the per-dimension calibrator trained and applied on the device (calib_kernel.cu)
            if ((rc = s->sq8p.ensure((size_t)2 * ix.dalign * 4))) return rc;
            GSX_CUDA(launch_block_minmax(raw.as<float>(), n, dim, ix.dalign, s->sq8p.as<float>(), st));
            GSX_CUDA(launch_encode_sq8(raw.as<float>(), n, dim, ix.dalign, s->sq8p.as<float>(), s->codes.as<uint8_t>(), st));
            s->h_sq8p.resize((size_t)2 * ix.dalign);
            GSX_CUDA(cudaMemcpyAsync(s->h_sq8p.data(), s->sq8p.p, s->h_sq8p.size() * 4, cudaMemcpyDeviceToHost, st));
            ix.sq8p = s->sq8p.as<float>();
        } else {
            GSX_CUDA(launch_encode(s->kind, s->metric, raw.as<float>(), n, dim, ix.dalign, ix.csize, ix.p0, ix.p1,
                                   s->codes.as<uint8_t>(), st));
        }
        if (s->has_refine) {
            ix.r_dalign = (dim + 15) / 16 * 16;
            if (s->r_kind == K_FP16) {
                if ((rc = s->r_codes.ensure((size_t)n * ix.r_dalign * 2))) return rc;
                GSX_CUDA(launch_encode(K_FP16, s->metric, raw.as<float>(), n, dim, ix.r_dalign, ix.r_dalign * 2, 0.0f, 0.0f,
                                       s->r_codes.as<uint8_t>(), st));
            } else {
                if ((rc = s->r_codes.ensure((size_t)n * ix.r_dalign * 4))) return rc;
                GSX_CUDA(launch_pad_rows(raw.as<float>(), n, dim, ix.r_dalign, s->r_codes.as<float>(), st));
            }
        }
        GSX_CUDA(cudaStreamSynchronize(st));
        ix.codes = s->codes.as<uint8_t>();
        ix.r_codes = s->r_codes.as<uint8_t>();
        ix.r_kind = s->r_kind;
        // keep 1,000 sampled rows for optimize (graph_searcher.hpp:62-69)
        s->sample_n = std::min(1000, n);
        std::mt19937 rng(12345);
        s->sample.resize((size_t)s->sample_n * dim);
        for (int i = 0; i < s->sample_n; ++i) {
            const int r = (int)(rng() % (uint32_t)n);
            std::memcpy(&s->sample[(size_t)i * dim], data + (size_t)r * dim, (size_t)dim * 4);
        }
        if ((rc = batch_order_setup(s))) return rc;
        s->has_data = true;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_set_data")
}

int gsx_searcher_set_ef(gsx_searcher *s, int32_t ef) {
    try {
        if (!s) return fail(GSX_ERR_INVALID, "null searcher");
        if (ef <= 0) return fail(GSX_ERR_INVALID, "ef must be positive");
        s->ef = ef;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_set_ef")
}

int gsx_searcher_get_ef(const gsx_searcher *s, int32_t *ef) {
    try {
        if (!s || !ef) return fail(GSX_ERR_INVALID, "null argument");
        *ef = s->ef;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_get_ef")
}

int gsx_searcher_search(gsx_searcher *s, const float *query, int32_t k, int32_t *ids, float *dis) {
    try {
        if (!s || !query || !ids) return fail(GSX_ERR_INVALID, "null argument");
        return host_batch(s, query, 1, k, nullptr, nullptr, k, ids, dis, true);
    } GSX_ABI_GUARD("gsx_searcher_search")
}

int gsx_searcher_search_batch(gsx_searcher *s, const float *queries, int32_t nq, int32_t k, int32_t *ids, float *dis) {
    try {
        if (!s || (nq > 0 && (!queries || !ids))) return fail(GSX_ERR_INVALID, "null argument");
        return host_batch(s, queries, nq, k, nullptr, nullptr, k, ids, dis, false);
    } GSX_ABI_GUARD("gsx_searcher_search_batch")
}

int gsx_searcher_search_batch_mixed(gsx_searcher *s, const float *queries, int32_t nq, int32_t k, const int32_t *ef,
                                    const int32_t *kq, int32_t kmax, int32_t *ids, float *dis) {
    try {
        if (!s || (nq > 0 && (!queries || !ids))) return fail(GSX_ERR_INVALID, "null argument");
        if (kq && kmax <= 0) return fail(GSX_ERR_INVALID, "kmax required with per-query k");
        if (!kq) kmax = k;
        return host_batch(s, queries, nq, k, ef, kq, kmax, ids, dis, false);
    } GSX_ABI_GUARD("gsx_searcher_search_batch_mixed")
}

int gsx_searcher_search_batch_device(gsx_searcher *s, const float *d_queries, int32_t nq, int32_t k,
                                     const int32_t *d_ef, const int32_t *d_k, int32_t kmax, int32_t *d_ids,
                                     float *d_dis, int32_t *d_cmps, int32_t *d_expansions, void *stream) {
    try {
        if (!s || (nq > 0 && (!d_queries || !d_ids))) return fail(GSX_ERR_INVALID, "null argument");
        if (!s->has_data) return fail(GSX_ERR_STATE, "search before set_data");
        if (k <= 0) return fail(GSX_ERR_INVALID, "k must be positive");
        if (kmax < k) kmax = k;
        int rc = set_device(s);
        if (rc) return rc;
        cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
        // with per-query ef on the device the caller's searcher ef is the upper bound
        return enqueue(s, d_queries, nq, k, s->ef, d_ef, d_k, kmax, s->ef, d_ids, d_dis, d_cmps, false, st, nullptr,
                       d_expansions);
    } GSX_ABI_GUARD("gsx_searcher_search_batch_device")
}

int gsx_searcher_get_last_search_avg_dist_cmps(const gsx_searcher *s, double *out) {
    try {
        if (!s || !out) return fail(GSX_ERR_INVALID, "null argument");
        *out = s->last_avg_cmps;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_get_last_search_avg_dist_cmps")
}

int gsx_searcher_get_tuning(const gsx_searcher *s, gsx_tuning *t) {
    try {
        if (!s || !t) return fail(GSX_ERR_INVALID, "null argument");
        *t = s->tuning;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_get_tuning")
}

int gsx_searcher_set_tuning(gsx_searcher *s, const gsx_tuning *t) {
    try {
        if (!s || !t) return fail(GSX_ERR_INVALID, "null argument");
        if (t->warps_per_block < 0 || t->warps_per_block > 8 || (t->warps_per_block & (t->warps_per_block - 1)))
            return fail(GSX_ERR_INVALID, "warps_per_block must be 0 or a power of two <= 8");
        if (t->lanes_per_row != 0 && t->lanes_per_row != 1 && t->lanes_per_row != 2 && t->lanes_per_row != 4)
            return fail(GSX_ERR_INVALID, "lanes_per_row must be 0, 1, 2 or 4");
        if (t->table_bits != 0 && t->table_bits != kGlobalOnly && (t->table_bits < kMinTableBits || t->table_bits > 16))
            return fail(GSX_ERR_INVALID, "table_bits must be 0 (automatic), 1 (global table only) or in [%d, 16]",
                        kMinTableBits);
        if (t->prefetch < 0 || t->prefetch > 63) return fail(GSX_ERR_INVALID, "prefetch must be in [0, 63]");
        if (t->spill_bits != 0 && (t->spill_bits < kMinTableBits || t->spill_bits > 20))
            return fail(GSX_ERR_INVALID, "spill_bits must be 0 or in [%d, 20]", kMinTableBits);
        s->tuning = *t;
        s->spill_from_optimize = false;
        if (is_float_kind(s->kind) && s->tuning.lanes_per_row == 2) s->tuning.lanes_per_row = 4;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_set_tuning")
}

int gsx_searcher_optimize(gsx_searcher *s, int32_t num_threads) {
    try {
        (void)num_threads;
        if (!s) return fail(GSX_ERR_INVALID, "null searcher");
        if (!s->has_data) return fail(GSX_ERR_STATE, "optimize before set_data");
        int rc = set_device(s);
        if (rc) return rc;
        // the sample is tiled to the size of the last host batch (a batch smaller than one wave of
        // resident warps is bound by its queries' latency, a larger one by throughput, and the best
        // settings differ), or, before any batch, to enough queries to fill the GPU several times over
        const int want = s->last_batch_nq > 0 ? std::min(std::max(s->last_batch_nq, 256), 65536) : 16384;
        const int reps = std::max(1, (want + s->sample_n - 1) / s->sample_n);
        const int nq = std::min(s->sample_n * reps, want), k = 10, d = s->ix.d;
        cudaStream_t st = s->stream;
        std::vector<float> tiled((size_t)nq * d);
        for (int r = 0; r < reps; ++r) {
            const int rows = std::min(s->sample_n, nq - r * s->sample_n);
            if (rows > 0)
                std::memcpy(tiled.data() + (size_t)r * s->sample_n * d, s->sample.data(), (size_t)rows * d * 4);
        }
        if ((rc = upload(s->q, tiled.data(), (size_t)nq * d, st))) return rc;
        if ((rc = s->ids.ensure((size_t)nq * k * 4))) return rc;
        if ((rc = s->dis.ensure((size_t)nq * k * 4))) return rc;
        const gsx_tuning saved = s->tuning;
        const int base_bits = default_table_bits(s, std::max(s->ef, kin_of(s, k)));
        std::vector<int> lprs = is_float_kind(s->kind) ? std::vector<int>{1, 4} : std::vector<int>{1, 2, 4};
        gsx_tuning best = saved;
        float best_ms = 1e30f;
        // visited sets in global tables only, or a small shared table in front; sparse global tables
        std::vector<int> bit_choices{kGlobalOnly, 9};
        (void)base_bits;
        const int sb0 = s->tuning.spill_bits;
        const bool sfo0 = s->spill_from_optimize;
        const int sao0 = s->spill_auto_at_opt;
        s->spill_from_optimize = false;  // the sweep's sizes are used as given
        s->tuning.spill_bits = 0;
        LaunchCfg probe;
        int auto_sb = 14;
        if (make_cfg(s, k, s->ef, nq, false, 0, &probe) == GSX_OK) auto_sb = spill_bits_for(s, probe);
        s->tuning.spill_bits = sb0;
        // integer kinds whose code rows are staged in shared memory score them one lane per row
        // whatever lanes_per_row says, so only one value is tried for them
        LaunchCfg staged_probe;
        if (make_cfg(s, k, s->ef, nq, false, 0, &staged_probe) == GSX_OK && staged_probe.L.stage_row > 0 &&
            !is_float_kind(s->kind))
            lprs = {1};
        // row speculation (the merge settles the next pop and loads its row), with and without
        // prefetching that row's code rows and visited-table buckets, against none
        const int spec = kSpeculateRow;
        const std::vector<int> pfs{0, kPrefetchNeighbours, spec, spec | kPrefetchCodes, spec | kPrefetchBuckets,
                                   spec | kPrefetchCodes | kPrefetchBuckets};
        for (int wpb : {2, 4})
            for (int lpr : lprs)
                for (int bits : bit_choices)
                for (int pf : pfs)
                for (int sb : {auto_sb - 1, auto_sb, auto_sb + 1}) {
                    gsx_tuning t{wpb, bits, lpr, pf, sb};
                    s->tuning = t;
                    float ms_min = 1e30f;
                    bool ok = true;
                    for (int rep = 0; rep < 3 && ok; ++rep) {
                        cudaEventRecord(s->ev0, st);
                        rc = enqueue(s, s->q.as<float>(), nq, k, s->ef, nullptr, nullptr, k, s->ef, s->ids.as<int32_t>(),
                                     s->dis.as<float>(), nullptr, false, st);
                        if (rc) { ok = false; break; }
                        cudaEventRecord(s->ev1, st);
                        unsigned nover = 0;
                        cudaMemcpyAsync(&nover, s->counters.as<unsigned>() + 1, 4, cudaMemcpyDeviceToHost, st);
                        if (cudaStreamSynchronize(st) != cudaSuccess) {
                            s->tuning = saved;
                            s->spill_from_optimize = sfo0;
                            s->spill_auto_at_opt = sao0;
                            return cuda_fail(cudaGetLastError(), "optimize");
                        }
                        if (nover) { ok = false; break; }  // a table that overflows is not a candidate
                        float ms = 0;
                        cudaEventElapsedTime(&ms, s->ev0, s->ev1);
                        ms_min = std::min(ms_min, ms);
                    }
                    if (ok && ms_min < best_ms) {
                        best_ms = ms_min;
                        best = t;
                    }
                }
        s->tuning = best;
        if (best_ms < 1e30f) {
            s->spill_from_optimize = best.spill_bits > 0;
            s->spill_auto_at_opt = auto_sb;
        } else {  // nothing ran: the saved tuning stands, with its own origin
            s->spill_from_optimize = sfo0;
            s->spill_auto_at_opt = sao0;
        }
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_optimize")
}

int gsx_searcher_memory(const gsx_searcher *s, size_t *index_bytes, size_t *per_query_bytes) {
    try {
        if (!s) return fail(GSX_ERR_INVALID, "null searcher");
        if (index_bytes)
            *index_bytes = s->adj.bytes + s->eps.bytes + s->levels.bytes + s->loff.bytes + s->lists.bytes + s->codes.bytes +
                           s->r_codes.bytes + s->sq8p.bytes;
        if (per_query_bytes) {
            // device bytes one in-flight query holds outside the resident index: its fp32 row,
            // outputs (k up to 256), status and counter
            *per_query_bytes = (size_t)s->ix.d * 4 + 256 * 8 + 16;
        }
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_memory")
}

int gsx_searcher_distances(gsx_searcher *s, const float *queries, int32_t nq, const int32_t *ids, int32_t m,
                           int32_t refine, double *out) {
    try {
        if (!s || !queries || !ids || !out) return fail(GSX_ERR_INVALID, "null argument");
        if (!s->has_data) return fail(GSX_ERR_STATE, "distances before set_data");
        if (refine && !s->has_refine) return fail(GSX_ERR_STATE, "searcher has no refine store");
        for (int64_t i = 0; i < (int64_t)nq * m; ++i)
            if (ids[i] < 0 || ids[i] >= s->ix.N) return fail(GSX_ERR_INVALID, "id %d out of range", ids[i]);
        int rc = set_device(s);
        if (rc) return rc;
        cudaStream_t st = s->stream;
        if ((rc = upload(s->q, queries, (size_t)nq * s->ix.d, st))) return rc;
        if ((rc = upload(s->dist_ids, ids, (size_t)nq * m, st))) return rc;
        if ((rc = s->dist_out.ensure((size_t)nq * m * 8))) return rc;
        GSX_CUDA(launch_distances(s->ix, refine, s->q.as<float>(), nq, s->dist_ids.as<int32_t>(), m,
                                  s->dist_out.as<double>(), st));
        GSX_CUDA(cudaMemcpyAsync(out, s->dist_out.p, (size_t)nq * m * 8, cudaMemcpyDeviceToHost, st));
        GSX_CUDA(cudaStreamSynchronize(st));
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_distances")
}

int gsx_searcher_codes(const gsx_searcher *s, uint8_t *codes, float *params, int32_t *code_size) {
    try {
        if (!s) return fail(GSX_ERR_INVALID, "null searcher");
        if (!s->has_data) return fail(GSX_ERR_STATE, "codes before set_data");
        if (code_size) *code_size = s->ix.csize;
        if (params) {
            const bool sq8 = s->kind == K_SQ8 && !s->h_sq8p.empty();
            params[0] = sq8 ? s->h_sq8p[0] : s->ix.p0;
            params[1] = sq8 ? s->h_sq8p[s->h_sq8p.size() / 2] : s->ix.p1;
        }
        if (codes) {
            int rc = set_device(s);
            if (rc) return rc;
            GSX_CUDA(cudaMemcpy(codes, s->codes.p, (size_t)s->ix.N * s->ix.csize, cudaMemcpyDeviceToHost));
        }
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_codes")
}

int gsx_searcher_params(const gsx_searcher *s, float *params, int32_t *count) {
    try {
        if (!s || !count) return fail(GSX_ERR_INVALID, "null argument");
        if (!s->has_data) return fail(GSX_ERR_STATE, "params before set_data");
        if (s->kind == K_SQ8) {
            *count = (int32_t)s->h_sq8p.size();
            if (params) std::memcpy(params, s->h_sq8p.data(), s->h_sq8p.size() * 4);
        } else {
            *count = 2;
            if (params) {
                params[0] = s->ix.p0;
                params[1] = s->ix.p1;
            }
        }
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_params")
}

int gsx_searcher_overflow_count(gsx_searcher *s, uint32_t *count) {
    try {
        if (!s || !count) return fail(GSX_ERR_INVALID, "null argument");
        *count = 0;
        if (!s->counters.p) return GSX_OK;
        int rc = set_device(s);
        if (rc) return rc;
        GSX_CUDA(cudaMemcpyAsync(count, s->counters.as<unsigned>() + 1, 4, cudaMemcpyDeviceToHost, s->stream));
        GSX_CUDA(cudaStreamSynchronize(s->stream));
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_searcher_overflow_count")
}

}  // extern "C"
