// Device code of the batched search, shared by search_kernel.cu (the general launches, distance
// kernel, layout) and search_fast.cu (the fast form for the common shapes).
#pragma once

// Warp-per-query beam search over a fixed-degree graph: the GPU form of GraphSearcher
// (glass/searcher/graph_searcher.hpp:131-224) with LinearPool/Bitset (glass/neighbor.hpp:31-79,
// 320-433), the HNSW upper-level descent (glass/hnsw/HNSWInitializer.hpp:41-62) and the FP32
// Refiner tail (glass/searcher/refiner.hpp:45-110) fused after the traversal.
//
// One warp owns one query at a time and takes the next query from a device work queue
// (persistent kernel).  Per expansion the warp
//   1. finds the first unexpanded pool entry (ballot over the pool),
//   2. reads the adjacency row with one coalesced load (lane i <- neighbour i),
//   3. drops repeats inside the row (match.any) and visited ids (shared-memory hash table,
//      atomicCAS), keeping row order,
//   4. computes the distances of the new neighbours, a team of LPR lanes per row,
//   5. merges them into the sorted pool.
// The merge places every candidate exactly where the reference's sequential insert would
// (upper-bound position, earlier inserts first among equal distances, truncation at capacity),
// so on equal distances the pool, the expansion order, the distance count and the result are
// those of the CPU searcher.
#include <cuda_runtime.h>

#include <cstdint>

#include "gsx_device.cuh"
#include "gsx_internal.h"

namespace gsx {

namespace {

constexpr int32_t kChecked = (int32_t)0x80000000;
constexpr int32_t kIdMask = 0x7fffffff;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Visited set, open addressing.  Two storages:
//  * the shared-memory table: 2^bits int32 slots, -1 = empty, linear probing, cleared for every
//    query;
//  * the warp's global table: 2^bits uint32 slots in buckets of eight (one 32-byte load reads a
//    bucket), probed bucket after bucket.  A slot holds (tag << shift | id), shift = the graph's id
//    bits; it is empty unless its tag is the current query's.  Tags run 1..2^(32-shift)-1 over
//    the warp's successive queries and the table is cleared only when they wrap, so a query
//    starts on a clean table without writing it.
// Probing is bounded by the table size; the caller keeps the load under 3/4 (shared) or 7/8
// (global) so a free slot always exists.
__device__ __forceinline__ uint32_t slot_of(int32_t v, int bits) { return ((uint32_t)v * 0x9E3779B1u) >> (32 - bits); }

// Returns true if v was absent (and is now present).
__device__ __forceinline__ bool visit_shared(int32_t *tab, int bits, int32_t v) {
    const uint32_t mask = (1u << bits) - 1u;
    uint32_t h = slot_of(v, bits);
    for (uint32_t p = 0; p <= mask; ++p) {
        int32_t old = atomicCAS(tab + h, -1, v);
        if (old == -1) return true;
        if (old == v) return false;
        h = (h + 1u) & mask;
    }
    return false;
}

struct Bucket {
    uint32_t e[8];
};

// One 32-byte bucket (an L2 sector) in one load.  Plain (weak, L1-cached) loads and stores are
// enough: a table is used by one warp only, and within a launch a warp stays on one SM, so its
// lanes' accesses are ordered by __syncwarp.  No atomics touch the global tables.
__device__ __forceinline__ Bucket load_bucket(const uint32_t *p) {
    Bucket b;
    asm volatile("ld.global.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(b.e[0]), "=r"(b.e[1]), "=r"(b.e[2]), "=r"(b.e[3]), "=r"(b.e[4]), "=r"(b.e[5]), "=r"(b.e[6]),
                   "=r"(b.e[7])
                 : "l"(p)
                 : "memory");
    return b;
}

__device__ __forceinline__ void store_slot(uint32_t *p, uint32_t v) {
    asm volatile("st.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr int kBucketFull = 16;

// What one bucket says about `mine` (= tag << shift | id): 0..7 = not there, and its first free slot;
// 8 = already there; kBucketFull = the bucket holds eight other ids.  Tags only grow between two
// clears of the table, so a slot is the current query's exactly when it is >= tag << shift; and
// inserts take the first free slot along the probe sequence and never free one under a tag, so the
// current query's slots are a prefix of the bucket and their count is the first free slot.
__device__ __forceinline__ int scan_bucket(const Bucket &b, uint32_t mine, int shift, uint32_t tag) {
    const uint32_t base = tag << shift;
    bool found = false;
    int n = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        found |= b.e[j] == mine;
        n += b.e[j] >= base;
    }
    return found ? 8 : (n < 8 ? n : kBucketFull);
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// First index in [lo, hi) whose entry is not yet expanded, or hi; `node` = its id (-1 when none).
__device__ __forceinline__ int first_unchecked(const int32_t *pid, int lo, int hi, int lane, int32_t &node) {
    for (int base = lo; base < hi; base += 32) {
        const int i = base + lane;
        const int32_t v = i < hi ? pid[i] : -1;  // bit 31 set: expanded (or past the range)
        const unsigned b = __ballot_sync(kFull, v >= 0);
        if (b) {
            const int src = __ffs(b) - 1;
            node = __shfl_sync(kFull, v, src);
            return base + src;
        }
    }
    node = -1;
    return hi;
}

__device__ __forceinline__ int upper_bound_u32(const uint32_t *a, int n, uint32_t x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] > x) hi = mid; else lo = mid + 1;
    }
    return lo;
}

struct WarpState {
    uint32_t *pkey;
    int32_t *pid;
    int32_t *cand_id;
    uint32_t *cand_key;
    int32_t *acc_ub;
    uint32_t *acc_key;
    int32_t *acc_id;
    float *fq;
    uint32_t *qc;
    unsigned char *stage;        // staged code rows (one per lane)
    int32_t *src;                // fast form: lane that staged fresh neighbour j of the row (acc_ub's
                                 // words, free until the merge)
    int32_t *tab;                // shared-memory table (null when the query runs on the spill table)
    int tbits;
    uint32_t *spill;             // this warp's global table (tagged slots), or null
    uint32_t *spill_epoch;       // its query counter
    int sbits;
    int shift;                   // id bits of a global-table slot
    uint32_t epoch;              // tag of the current query in the global table (0 = not used)
    bool shared_first;           // queries start in the shared-memory table
};

// Warp-wide visited check in the global table, one candidate per lane (`want`): one bucket load
// per lane, then plain stores, since the table belongs to this warp alone.  Lanes that pick the
// same free slot are ordered by lane: the lowest one stores, the others read the bucket again after
// the store.  Returns true where v was absent (and is now present).  `bad` is set if a lane's probe
// went round the whole table (cannot happen under the load limit).
__device__ __forceinline__ bool visit_global_warp(WarpState &w, bool want, int32_t v, bool &bad) {
    const uint32_t mine = (w.epoch << w.shift) | (uint32_t)v;
    const uint32_t bmask = (1u << (w.sbits - 3)) - 1u;
    uint32_t h = want ? slot_of(v, w.sbits - 3) : 0u;
    uint32_t probes = 0;
    bool pending = want, fresh = false;
    while (__any_sync(kFull, pending)) {
        int r = kBucketFull;
        if (pending) r = scan_bucket(load_bucket(w.spill + 8 * h), mine, w.shift, w.epoch);
        const bool ins = pending && r < 8;
        const unsigned grp = __match_any_sync(kFull, ins ? 8u * h + (uint32_t)r : 0xffffffffu);
        if (ins) {
            if ((grp & lanemask_lt()) == 0) {
                store_slot(w.spill + 8 * h + r, mine);
                fresh = true;
                pending = false;
            }
        } else if (pending) {
            if (r < kBucketFull) {
                pending = false;  // already visited
            } else {
                h = (h + 1u) & bmask;
                if (++probes > bmask) {
                    pending = false;
                    bad = true;
                }
            }
        }
        __syncwarp();
    }
    return fresh;
}

// Warp-collective visited check of one candidate per lane (`want`) in the query's current table.
__device__ __forceinline__ bool visit_all(WarpState &w, bool want, int32_t v, bool &bad) {
    if (w.epoch) return visit_global_warp(w, want, v, bad);
    return want && visit_shared(w.tab, w.tbits, v);
}

// Gives the current query the next tag of the warp's global table; when the tags wrap, the
// table is cleared first so that no slot carries a reused tag.
__device__ __forceinline__ void spill_begin(WarpState &w, int lane) {
    uint32_t c = 0;
    if (lane == 0) c = atomicAdd(w.spill_epoch, 1u);
    c = __shfl_sync(kFull, c, 0);
    const uint32_t ntags = (1u << (32 - w.shift)) - 1u;
    const uint32_t t = c % ntags;
    if (t == 0) {
        const int n = 1 << w.sbits;
        for (int j = lane * 4; j < n; j += 128) *reinterpret_cast<uint4 *>(w.spill + j) = make_uint4(0, 0, 0, 0);
        __syncwarp();
    }
    w.epoch = t + 1u;
}

// Moves the visited set from the shared-memory table into the warp's global table under a fresh
// tag and continues there: the set is unchanged, only its storage grows.
__device__ __forceinline__ void migrate_visited(WarpState &w, int lane, bool &bad) {
    spill_begin(w, lane);
    const int tsize = 1 << w.tbits;
    for (int j0 = 0; j0 < tsize; j0 += 32) {
        const int32_t v = w.tab[j0 + lane];
        visit_global_warp(w, v != -1, v, bad);
    }
    __syncwarp();
}

// The pop of the next expansion, settled by the merge before it moves any pool entry: its pool index
// (exact: the first unexpanded entry of the merged pool) and its node, whose adjacency row is
// loaded right away when speculation is on, so that it arrives while the merge runs.
struct NextPop {
    int f = -1;                // pool index of the next pop; -1 = not known (the loop top looks it up)
    int32_t node = -1;         // its node (valid when f is below the expansion limit)
    int u = -1;                // its node when its row was loaded (-1: nothing loaded)
    int32_t r0 = -1, r1 = -1;  // that row: entries lane and 32 + lane
};

// f0 = first unexpanded index of the pool before the merge (lim if none below min(S, lim)) and node0
// its node, lo = the slot of the best candidate that enters (INT_MAX when none does).  The merged
// pool's first unexpanded entry is the candidate when lo <= f0 (it lands at or before f0's entry),
// else f0's entry, which no candidate passes.  `cand` is the candidate's node (used when lo <= f0).
__device__ __forceinline__ void settle_next(const IndexView &ix, NextPop &np, bool speculate, int f0, int32_t node0,
                                            int lo, int lim, int32_t cand, int lane) {
    const int f = lo <= f0 ? lo : f0;
    const int32_t u = lo <= f0 ? cand : node0;
    np.f = f;
    np.node = u;
    np.u = -1;
    if (!speculate || f >= lim || u < 0) return;
    const int32_t *row = ix.adj + (size_t)u * (size_t)ix.K;
    np.u = u;
    np.r0 = lane < ix.K ? __ldg(row + lane) : -1;
    np.r1 = lane + 32 < ix.K ? __ldg(row + 32 + lane) : -1;
}

// merge() for at most 32 surviving candidates (cand_{key,id}[0..ns), arrival order) and a pool of at
// most 32*GS entries (GS = 4 or 8).  Candidate j (lane j): rank_j among the candidates by (key,
// arrival), and ub_j = pool entries with key <= key_j, found from the last keys of the pool's
// GS-entry groups (one ballot per candidate) and one read of its group; its slot is ub_j + rank_j,
// taken when below cap (slots rise with rank, so the taken candidates are ranks 0..n-1).  The pool
// from the first slot up is then rebuilt in one parallel pass: the taken slots are gathered into
// 32-position bit words (redux.or), so for every position q the number c of taken slots below q is
// a prefix popcount; q holds the candidate of rank c when it is a taken slot, else the old entry
// q - c.  Every position reads before any writes, and whatever lands at cap or beyond is dropped.
template <int GS>
__device__ __forceinline__ void merge_small(WarpState &w, int &S, int cap, int &lb, int m, int ns, int lane,
                                            const IndexView &ix, NextPop *np, bool speculate, int f0, int32_t node0,
                                            int lim) {
    const bool has = lane < ns;
    const uint32_t kj = has ? w.cand_key[lane] : 0xffffffffu;
    const int32_t ij = has ? w.cand_id[lane] : 0;
    const bool full = GS * lane + GS - 1 < S;
    const uint32_t piv = full ? w.pkey[GS * lane + GS - 1] : 0u;
    int rank = 0, grp = 0;
#pragma unroll 4
    for (int i = 0; i < ns; ++i) {
        const uint32_t ki = __shfl_sync(kFull, kj, i);
        const unsigned b = __ballot_sync(kFull, full && piv <= ki);
        if (lane == i) grp = __popc(b);
        rank += (ki < kj) || (ki == kj && i < lane);
    }
    int ub = 0x7fffffff;  // lanes without a candidate
    if (has) {
        // the group's keys: GS*grp + GS-1 < capacity rounded up to 32, so the reads stay in the pool
        const int g0 = GS * grp;
        int c = 0;
#pragma unroll
        for (int h = 0; h < GS / 4; ++h) {
            const uint4 gk = *reinterpret_cast<const uint4 *>(w.pkey + g0 + 4 * h);
            const int b0 = g0 + 4 * h;
            c += (int)(b0 < S && gk.x <= kj) + (int)(b0 + 1 < S && gk.y <= kj) + (int)(b0 + 2 < S && gk.z <= kj) +
                 (int)(b0 + 3 < S && gk.w <= kj);
        }
        ub = g0 + c;
    }
    const int slot = has ? ub + rank : 0x7fffffff;
    const bool acc = has && slot < cap;
    // the rank-0 candidate always fits (its key is below the last entry of a full pool)
    const int lo = (int)__reduce_min_sync(kFull, acc ? (unsigned)slot : 0x7fffffffu);
    const int sl = __popc(__ballot_sync(kFull, has && ub <= lb));
    if (np) {
        // the rank-0 candidate holds slot lo; its node is the next pop when lo <= f0
        const unsigned r0 = __ballot_sync(kFull, acc && slot == lo);
        const int32_t cand = __shfl_sync(kFull, ij, r0 ? __ffs(r0) - 1 : 0);
        settle_next(ix, *np, speculate, f0, node0, lo, lim, cand, lane);
    }
    if (acc) {
        w.acc_key[rank] = kj;
        w.acc_id[rank] = ij;
    }
    const int newS = (S + m) < cap ? (S + m) : cap;
    // positions below 32 * (GS + 1) hold every slot: S <= 32 * GS and at most 32 candidates
    constexpr int NW = GS + 1;
    uint32_t word[NW];
#pragma unroll
    for (int t = 0; t < NW; ++t)
        word[t] = __reduce_or_sync(kFull, (acc && (slot >> 5) == t) ? 1u << (slot & 31) : 0u);
    __syncwarp();
    const unsigned ltm = lanemask_lt();
    uint32_t nk[NW];
    int32_t ni[NW];
    int before = 0;
#pragma unroll
    for (int t = 0; t < NW; ++t) {
        const int q = 32 * t + lane;
        nk[t] = 0u;
        ni[t] = 0;
        if (32 * t + 31 >= lo && 32 * t < newS) {
            const int c = before + __popc(word[t] & ltm);
            if (q >= lo && q < newS) {
                if ((word[t] >> lane) & 1u) {
                    nk[t] = w.acc_key[c];
                    ni[t] = w.acc_id[c];
                } else {
                    nk[t] = w.pkey[q - c];
                    ni[t] = w.pid[q - c];
                }
            }
        }
        before += __popc(word[t]);
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < NW; ++t) {
        const int q = 32 * t + lane;
        if (32 * t + 31 >= lo && 32 * t < newS && q >= lo && q < newS) {
            w.pkey[q] = nk[t];
            w.pid[q] = ni[t];
        }
    }
    // new lower bound of the first unexpanded entry: the first candidate, or where the old bound
    // moved to
    const int nl = lb + sl;
    lb = lo < nl ? lo : nl;
    S = newS;
    __syncwarp();
}

// Merges candidates cand_{id,key}[0..m) (in insertion order, m <= 64) into the pool
// pkey/pid[0..S) of capacity cap.  Exactly the state LinearPool::insert (neighbor.hpp:382-396)
// reaches by inserting them one after the other: a candidate lands after every pool entry with
// an equal or smaller key and after the earlier candidates with equal keys; entries pushed past
// cap are dropped.  `lb` is a lower bound of the first unexpanded index and is updated.
//
// Candidate j's final slot is ub_j + rank_j (ub = upper bound in the pool, rank = position among
// the candidates ordered by (key, arrival)); the accepted candidates are those whose slot is below
// cap, i.e. the lowest ranks.  The pool is then rebuilt from the top in 32-slot chunks: a
// redux.or of the candidates' slot bits in the chunk says which slots take a candidate, and every
// other slot p takes the pool entry p - (candidates placed below p).  A chunk only reads entries
// at or below its own slots, so no entry is overwritten before it is read.
//
// With np given, f0 is the first unexpanded index before the merge (lim if none below min(S, lim)),
// node0 its node, and the next expansion's pop is settled (settle_next) before any entry moves.
template <bool SMALL = false>  // SMALL: at most 32 candidates and a pool of at most 256 entries
__device__ __forceinline__ void merge(WarpState &w, int &S, int cap, int &lb, int m, int lane,
                                      const IndexView &ix, NextPop *np = nullptr, bool speculate = false, int f0 = 0,
                                      int32_t node0 = -1, int lim = 0) {
    // survivors: with a full pool a candidate whose key is not below the last entry can never
    // enter, and its larger key does not change the rank of one that does
    const unsigned ltm = (1u << lane) - 1u;
    const uint32_t last = S == cap ? w.pkey[S - 1] : 0xffffffffu;
    const bool v0 = lane < m, v1 = !SMALL && lane + 32 < m;
    const uint32_t k0 = v0 ? w.cand_key[lane] : 0u, k1 = v1 ? w.cand_key[lane + 32] : 0u;
    const int32_t i0 = v0 ? w.cand_id[lane] : 0, i1 = v1 ? w.cand_id[lane + 32] : 0;
    const bool s0 = v0 && (S < cap || k0 < last), s1 = v1 && (S < cap || k1 < last);
    const unsigned b0 = __ballot_sync(kFull, s0), b1 = SMALL ? 0u : __ballot_sync(kFull, s1);
    const int ns = __popc(b0) + __popc(b1);
    if (ns == 0) {
        S = (S + m) < cap ? (S + m) : cap;
        if (np) settle_next(ix, *np, speculate, f0, node0, 0x7fffffff, lim, -1, lane);
        return;
    }
    // compact the survivors in arrival order
    __syncwarp();
    if (s0) {
        const int t = __popc(b0 & ltm);
        w.cand_key[t] = k0;
        w.cand_id[t] = i0;
    }
    if (s1) {
        const int t = __popc(b0) + __popc(b1 & ltm);
        w.cand_key[t] = k1;
        w.cand_id[t] = i1;
    }
    __syncwarp();
    if (ns <= 32 && S <= 128) {
        merge_small<4>(w, S, cap, lb, m, ns, lane, ix, np, speculate, f0, node0, lim);
        return;
    }
    if (SMALL || (ns <= 32 && S <= 256)) {
        merge_small<8>(w, S, cap, lb, m, ns, lane, ix, np, speculate, f0, node0, lim);
        return;
    }
    if constexpr (SMALL) return;
    int nacc = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int j = lane + 32 * h;
        const bool valid = j < ns;
        const uint32_t kj = valid ? w.cand_key[j] : 0u;
        int acc = 0, ub = 0, rank = 0;
        if (valid) {
            for (int i = 0; i < ns; ++i) {
                const uint32_t ki = w.cand_key[i];
                rank += (ki < kj) || (ki == kj && i < j);
            }
            ub = upper_bound_u32(w.pkey, S, kj);
            acc = (ub + rank) < cap;
        }
        if (acc) {
            w.acc_ub[rank] = ub;
            w.acc_key[rank] = kj;
            w.acc_id[rank] = w.cand_id[j];
        }
        nacc += __popc(__ballot_sync(kFull, acc));
        if (ns <= 32) break;
    }
    __syncwarp();
    if (nacc == 0) {  // cannot happen: the rank-0 survivor always fits
        if (np) settle_next(ix, *np, speculate, f0, node0, 0x7fffffff, lim, -1, lane);
        return;
    }
    // slots of the accepted candidates, rank r held by lane r (and r+32)
    constexpr int kNone = 0x7fffffff;
    const int ub0 = lane < nacc ? w.acc_ub[lane] : kNone;
    const int ub1 = lane + 32 < nacc ? w.acc_ub[lane + 32] : kNone;
    const int p0 = ub0 == kNone ? kNone : ub0 + lane;
    const int p1 = ub1 == kNone ? kNone : ub1 + lane + 32;
    const int lo = __shfl_sync(kFull, p0, 0);  // slot of the rank-0 candidate = acc_ub[0]
    if (np) settle_next(ix, *np, speculate, f0, node0, lo, lim, w.acc_id[0], lane);
    const int newS = (S + m) < cap ? (S + m) : cap;
    const int nchunks = (newS - lo + 31) >> 5;
    for (int c = nchunks - 1; c >= 0; --c) {
        const int base = lo + 32 * c;
        const int below = __popc(__ballot_sync(kFull, p0 < base)) + __popc(__ballot_sync(kFull, p1 < base));
        unsigned bits = 0;
        if (p0 >= base && p0 < base + 32) bits |= 1u << (p0 - base);
        if (p1 >= base && p1 < base + 32) bits |= 1u << (p1 - base);
        const unsigned cm = __reduce_or_sync(kFull, bits);
        const int p = base + lane;
        const int r = below + __popc(cm & ltm);
        uint32_t k = 0;
        int32_t id = 0;
        if (p < newS) {
            if ((cm >> lane) & 1u) {
                k = w.acc_key[r];
                id = w.acc_id[r];
            } else {
                k = w.pkey[p - r];
                id = w.pid[p - r];
            }
        }
        __syncwarp();
        if (p < newS) {
            w.pkey[p] = k;
            w.pid[p] = id;
        }
        __syncwarp();
    }
    // new lower bound of the first unexpanded entry: the first candidate, or where the old bound
    // moved to
    const int sl = __popc(__ballot_sync(kFull, ub0 <= lb)) + __popc(__ballot_sync(kFull, ub1 <= lb));
    const int nl = lb + sl;
    lb = lo < nl ? lo : nl;
    S = newS;
    __syncwarp();
}

// Distances of cand_id[0..m) -> cand_key[0..m).
template <int KIND, int METRIC, int LPR>
__device__ __forceinline__ void compute_dists(const IndexView &ix, WarpState &w, int m, int32_t qsq, int lane) {
    constexpr int TEAMS = 32 / LPR;
    const int team = lane / LPR, sub = lane % LPR;
    for (int b = 0; b < m; b += TEAMS) {
        const int j = b + team;
        const bool act = j < m;
        const int id = act ? w.cand_id[j] : 0;
        uint32_t key;
        if (IsIntKind<KIND>::value) {
            int32_t part = act ? sq_partial<KIND, METRIC, LPR>(ix.codes, ix.csize, id, sub, w.qc) : 0;
            key = key_of(sq_finish<KIND, METRIC, LPR>(part, qsq));
        } else {
            const uint8_t *row = ix.codes + (size_t)id * (size_t)ix.csize;
            float dv = float_dist<KIND, METRIC, LPR>(row, ix.dalign >> 4, sub, w.fq, act, ix.sq8p);
            key = key_of(dv);
        }
        if (act && sub == 0) w.cand_key[j] = key;
    }
    __syncwarp();
}

// Refine distance (FP32 or FP16 store) of ids[0..m) into out, 4 lanes per row.
template <int METRIC>
__device__ __forceinline__ void refine_dists(const IndexView &ix, const int32_t *ids, float *out, int m,
                                             const float *fq, int lane) {
    const int team = lane >> 2, sub = lane & 3;
    for (int b = 0; b < m; b += 8) {
        const int j = b + team;
        const bool act = j < m;
        const int id = act ? ids[j] : 0;
        const size_t esize = ix.r_kind == K_FP16 ? 2 : 4;
        const uint8_t *row = ix.r_codes + (size_t)id * (size_t)ix.r_dalign * esize;
        float dv = ix.r_kind == K_FP16 ? float_dist<K_FP16, METRIC, 4>(row, ix.r_dalign >> 4, sub, fq, act)
                                       : float_dist<K_FP32, METRIC, 4>(row, ix.r_dalign >> 4, sub, fq, act);
        if (act && sub == 0) out[j] = dv;
    }
    __syncwarp();
}

// Encodes the query held in w.fq into w.qc (SQ kinds); returns the sum of squared codes.
template <int KIND, int METRIC>
__device__ __forceinline__ int32_t prepare_query(const IndexView &ix, WarpState &w, int lane) {
    if (!IsIntKind<KIND>::value) return 0;
    const int nw = ix.csize >> 2;
    int32_t sq = 0;
    for (int wi = lane; wi < nw; wi += 32) {
        if (KIND == K_SQ4UA) {
            // sq4ua_quant.hpp:52-58 (encode8): each dimension on 0..127; base word wi holds dimensions
            // 8wi..8wi+7, the even ones in its low nibbles and the odd ones in its high nibbles
            uint32_t qe = 0, qo = 0;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int j0 = 8 * wi + 2 * t, j1 = j0 + 1;
                const uint32_t c0 = j0 < ix.d ? (uint32_t)affine_code(w.fq[j0], ix.p0, ix.p1, 127.0f) : 0u;
                const uint32_t c1 = j1 < ix.d ? (uint32_t)affine_code(w.fq[j1], ix.p0, ix.p1, 127.0f) : 0u;
                qe |= c0 << (8 * t);
                qo |= c1 << (8 * t);
            }
            w.qc[wi] = qe;
            w.qc[nw + wi] = qo;
            sq = __dp4a(qe, qe, (uint32_t)sq);
            sq = __dp4a(qo, qo, (uint32_t)sq);
            continue;
        }
        uint32_t word = 0;
#pragma unroll
        for (int t = 0; t < 4; ++t)
            word |= sq_code_byte<KIND, METRIC>(w.fq, ix.d, 4 * wi + t, ix.p0, ix.p1) << (8 * t);
        if (KIND == K_SQ2U) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t x = (word >> (2 * k)) & 0x03030303u;
                w.qc[k * nw + wi] = x;
                sq = __dp4a(x, x, (uint32_t)sq);
            }
        } else if (KIND == K_SQ4U) {
            uint32_t lo = word & 0x0F0F0F0Fu, hi = (word >> 4) & 0x0F0F0F0Fu;
            w.qc[wi] = lo;
            w.qc[nw + wi] = hi;
            sq = __dp4a(lo, lo, (uint32_t)sq);
            sq = __dp4a(hi, hi, (uint32_t)sq);
        } else {
            w.qc[wi] = word;
            sq = __dp4a(word, word, (uint32_t)sq);
        }
    }
    sq = team_sum<32>(sq);
    __syncwarp();
    return sq;
}

// NCH > 0 compiles the fast form of the expansion loop for the common shapes: integer codes staged in
// shared memory as NCH 16-byte chunks, degree <= 32, visited sets in the warps' global tables and pools
// of at most 256 entries (the host launches it only then).  The search is the same; only the runtime
// tests of the general form become compile-time facts.
template <int KIND, int METRIC, int LPR, int NCH>
__device__ void search_one(const IndexView &ix, const BatchView &bv, const WarpLayout &L, WarpState &w, int qi,
                           int lane) {
    // a per-query k outside [0, out_stride] (a caller error on the device entry points) is clamped,
    // so that no write leaves the query's output row
    int kq = bv.k_per ? bv.k_per[qi] : bv.k;
    kq = kq < 0 ? 0 : (kq > bv.out_stride ? bv.out_stride : kq);
    const int efq = bv.ef_per ? bv.ef_per[qi] : bv.ef;
    // Refiner: reorder_k = (int)(k * factor) (refiner.hpp:46, 73)
    const int rk = ix.has_refine ? (int)((float)kq * ix.refine_factor) : kq;
    const bool refine = ix.has_refine && rk != kq;
    const int kin = refine ? rk : kq;
    int cap = kin > efq ? kin : efq;
    if (cap > L.cap) cap = L.cap;  // host sizes L.cap >= every query's capacity
    // SearchBatch: pool.reset(nb, ef, max(k, ef)); Search: pool.reset(nb, max(k,ef), max(k,ef))
    const int ef_expand = bv.single ? cap : efq;

    // query -> shared memory (fp32, zero padded), then the quantizer's encoding
    const float *q = bv.queries + (size_t)qi * (size_t)ix.d;
    for (int j = lane; j < L.fq_len; j += 32) w.fq[j] = j < ix.d ? __ldg(q + j) : 0.0f;
    __syncwarp();
    const int32_t qsq = prepare_query<KIND, METRIC>(ix, w, lane);

    // visited set: a cleared shared-memory table, or (when the launch has none) a fresh epoch of the
    // warp's global table
    int tlimit;
    if (w.shared_first) {
        w.epoch = 0;
        const int tsize = 1 << w.tbits;
        for (int j = lane * 4; j < tsize; j += 128) *reinterpret_cast<int4 *>(w.tab + j) = make_int4(-1, -1, -1, -1);
        __syncwarp();
        tlimit = (tsize >> 2) * 3;
    } else {
        spill_begin(w, lane);
        tlimit = (1 << w.sbits) - ((1 << w.sbits) >> 3);
    }

    int S = 0, lb = 0, nvis = 0, cmps = 0, nexp = 0;
    bool overflow = false;

    // ---- initialize_search (graph.hpp:229-238) ----
    if (ix.has_hnsw) {
        // HNSWInitializer::initialize (HNSWInitializer.hpp:41-62): greedy descent; within a pass
        // the list of the node held at the start of the pass is scanned and the running best
        // (strictly smaller distance) kept, i.e. the first minimum of the list.
        int u = ix.hep;
        if (lane == 0) w.cand_id[0] = u;
        __syncwarp();
        compute_dists<KIND, METRIC, LPR>(ix, w, 1, qsq, lane);
        uint32_t cur = w.cand_key[0];
        cmps += 1;
        __syncwarp();
        for (int level = ix.levels[u]; level > 0; --level) {
            bool changed = true;
            while (changed) {
                changed = false;
                const int32_t *list = ix.lists + ix.loff[u] + (int64_t)(level - 1) * ix.hK;
                int m = 0;
                for (int c0 = 0; c0 < ix.hK; c0 += 32) {
                    const int i = c0 + lane;
                    const int v = i < ix.hK ? __ldg(list + i) : -1;
                    const unsigned endm = __ballot_sync(kFull, v == -1);
                    const int nvalid = endm ? __ffs(endm) - 1 : 32;
                    if (lane < nvalid) w.cand_id[m + lane] = v;
                    m += nvalid;
                    if (endm) break;
                }
                __syncwarp();
                if (m == 0) break;
                compute_dists<KIND, METRIC, LPR>(ix, w, m, qsq, lane);
                cmps += m;
                // first index of the minimum key
                uint32_t bk = 0xffffffffu;
                int bj = 0x7fffffff;
                for (int j = lane; j < m; j += 32) {
                    uint32_t kj = w.cand_key[j];
                    if (kj < bk || (kj == bk && j < bj)) { bk = kj; bj = j; }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    uint32_t ok = __shfl_xor_sync(kFull, bk, o);
                    int oj = __shfl_xor_sync(kFull, bj, o);
                    if (ok < bk || (ok == bk && oj < bj)) { bk = ok; bj = oj; }
                }
                if (bk < cur) {
                    cur = bk;
                    u = w.cand_id[bj];
                    changed = true;
                }
                __syncwarp();
            }
        }
        if (lane == 0) {
            w.cand_id[0] = u;
            w.cand_key[0] = cur;
        }
        __syncwarp();
        merge(w, S, cap, lb, 1, lane, ix);
        bool bad = false;
        visit_all(w, lane == 0, u, bad);
        nvis += 1;
        if (__any_sync(kFull, bad)) overflow = true;
        __syncwarp();
    } else {
        for (int e0 = 0; e0 < ix.nep; e0 += kMaxDegree) {
            const int m = (ix.nep - e0) < kMaxDegree ? (ix.nep - e0) : kMaxDegree;
            for (int j = lane; j < m; j += 32) w.cand_id[j] = __ldg(ix.eps + e0 + j);
            __syncwarp();
            compute_dists<KIND, METRIC, LPR>(ix, w, m, qsq, lane);
            cmps += m;
            merge(w, S, cap, lb, m, lane, ix);
            bool bad = false;
            for (int j0 = 0; j0 < m; j0 += 32) {
                const int j = j0 + lane;
                visit_all(w, j < m, j < m ? w.cand_id[j] : 0, bad);
            }
            nvis += m;
            if (__any_sync(kFull, bad)) overflow = true;
            __syncwarp();
            if (nvis > tlimit) { overflow = true; break; }
        }
    }

    // ---- SearchImpl2 (graph_searcher.hpp:196-224) ----
    const int lim = ef_expand < cap ? ef_expand : cap;
    const bool speculate = (L.prefetch & kSpeculateRow) != 0;
    NextPop np;  // the pop the last merge settled, with its row when it was loaded
    while (!overflow) {
        int32_t u = np.node;
        const int f = np.f >= 0 ? np.f : first_unchecked(w.pid, lb, S < lim ? S : lim, lane, u);
        if (f >= S || f >= lim) break;
        if (nvis + ix.K > tlimit) {
            if constexpr (NCH == 0) {
                if (w.spill && w.epoch == 0) {
                    bool bad = false;
                    migrate_visited(w, lane, bad);
                    tlimit = (1 << w.sbits) - ((1 << w.sbits) >> 3);
                    if (__any_sync(kFull, bad)) { overflow = true; break; }
                }
            }
            if (nvis + ix.K > tlimit) { overflow = true; break; }
        }
        // the pop (neighbor.hpp:398-405): the entry is unexpanded, so its stored id is u itself
        if (lane == 0) w.pid[f] = u | kChecked;
        lb = f + 1;
        ++nexp;
        // adjacency row, stop at the first -1; skip repeats within the row and visited ids
        int32_t r0 = np.r0, r1 = np.r1;
        if (u != np.u) {
            const int32_t *row = ix.adj + (size_t)u * (size_t)ix.K;
            r0 = lane < ix.K ? __ldg(row + lane) : -1;
            r1 = lane + 32 < ix.K ? __ldg(row + 32 + lane) : -1;
        }
        np.f = -1;
        np.u = -1;
        int m = 0;
        const bool staged = NCH > 0 || L.stage_row > 0;
        for (int c0 = 0; c0 < (NCH > 0 ? 32 : ix.K); c0 += 32) {
            const int v = c0 == 0 ? r0 : r1;
            const unsigned endm = __ballot_sync(kFull, v == -1);
            const int nvalid = endm ? __ffs(endm) - 1 : 32;
            const bool valid = lane < nvalid;
            // repeats inside the row: the first occurrence is the one visited (the reference checks
            // and sets the bitset neighbour by neighbour).  The fast form leaves this to the global
            // table, whose inserts already go to the lowest of the lanes holding one id.
            bool first = valid;
            if constexpr (NCH == 0) {
                const unsigned same = __match_any_sync(kFull, v);
                const unsigned vmask = nvalid >= 32 ? kFull : ((1u << nvalid) - 1u);
                first = valid && ((same & vmask & lanemask_lt()) == 0);
            }
            uint8_t *srow = nullptr;
            if (staged) {
                // copy the code row into shared memory now, so that it arrives during the visited check
                srow = w.stage + lane * L.stage_stride;
                if (first) {
                    const uint8_t *c = ix.codes + (size_t)v * (size_t)ix.csize;
#pragma unroll
                    for (int o = 0; o < (NCH > 0 ? 16 * NCH : L.stage_row); o += 16) cp_async16(srow + o, c + o);
                }
                cp_async_commit();
            } else if ((L.prefetch & kPrefetchNeighbours) && first) {
                // start the code row's way in now, so that it overlaps the visited check: the whole row,
                // into L1 when it is at most two lines, else into L2 (32 rows of up to 3 KB would
                // overrun L1)
                const uint8_t *c = ix.codes + (size_t)v * (size_t)ix.csize;
                if (ix.csize <= 256) {
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(c));
                    if (ix.csize > 128) asm volatile("prefetch.global.L1 [%0];" ::"l"(c + 128));
                } else {
                    for (int o = 0; o < ix.csize; o += 128) asm volatile("prefetch.global.L2 [%0];" ::"l"(c + o));
                }
            }
            bool bad = false;
            const bool fresh = NCH > 0 ? visit_global_warp(w, first, v, bad) : visit_all(w, first, v, bad);
            if (__any_sync(kFull, bad)) overflow = true;
            const unsigned nm = __ballot_sync(kFull, fresh);
            const int at = m + __popc(nm & lanemask_lt());
            if constexpr (NCH > 0) {
                // the fresh rows' distances by teams of four lanes: lane (team t, sub s) takes chunk s
                // (and s + 4 when NCH is 8) of fresh row t of each pass of eight, reading the row where
                // its own lane staged it (src), and the team's partials are summed by two shuffles;
                // the integer arithmetic is exact, so the split changes no distance
                const int cnt = __popc(nm);
                if (fresh) w.src[at] = lane;
                cp_async_wait_all();
                __syncwarp();
                const int team = lane >> 2, sub = lane & 3;
                for (int b = 0; b < cnt; b += 8) {
                    const int j = b + team;
                    const int sj = w.src[j & 31] & 31;  // lanes past cnt read a stale, in-range slot
                    const unsigned char *row = w.stage + sj * L.stage_stride;
                    int32_t part = sq_partial_chunk<KIND, METRIC>(reinterpret_cast<const uint4 *>(row)[sub], sub, NCH, w.qc);
                    if (NCH == 8)
                        part += sq_partial_chunk<KIND, METRIC>(reinterpret_cast<const uint4 *>(row)[sub + 4], sub + 4, NCH,
                                                               w.qc);
                    const uint32_t key = key_of(sq_finish<KIND, METRIC, 4>(j < cnt ? part : 0, qsq));
                    if (j < cnt && sub == 0) w.cand_key[j] = key;
                }
                if (fresh) w.cand_id[at] = v;
                __syncwarp();  // the staged rows are read before the next expansion stages others
                m += cnt;
                if (endm) break;
                continue;
            }
            if (staged) {
                // distance of this lane's own neighbour from the staged row (one lane per row)
                cp_async_wait_all();
                if (fresh) {
                    if constexpr (IsIntKind<KIND>::value) {
                        const int32_t part = sq_partial_row<KIND, METRIC>(reinterpret_cast<const uint4 *>(srow),
                                                                          NCH > 0 ? NCH : (L.stage_row >> 4), w.qc);
                        w.cand_key[at] = key_of(sq_finish<KIND, METRIC, 1>(part, qsq));
                    } else if constexpr (NCH == 0) {
                        // the float engine with one lane per row, reading the staged row
                        w.cand_key[at] = key_of(float_dist<KIND, METRIC, 1, true>(srow, ix.dalign >> 4, 0, w.fq, true,
                                                                                ix.sq8p));
                    }
                }
            }
            if (fresh) w.cand_id[at] = v;
            m += __popc(nm);
            if (endm) break;
        }
        __syncwarp();
        nvis += m;
        if (m == 0) continue;
        if (NCH == 0 && !staged) compute_dists<KIND, METRIC, LPR>(ix, w, m, qsq, lane);
        cmps += m;
        // the merge settles the next pop (and, speculating, starts loading its row) before it moves
        // pool entries
        int32_t node0;
        const int f0 = first_unchecked(w.pid, lb, S < lim ? S : lim, lane, node0);
        merge<(NCH > 0)>(w, S, cap, lb, m, lane, ix, &np, speculate, f0, node0, lim);
        if ((L.prefetch & kPrefetchCodes) && np.u >= 0) {
            // the next row has arrived during the merge: pull its neighbours' code rows towards L1
            // for the next expansion (cf. the reference's computer.prefetch, graph_searcher.hpp:212-218)
            const int lines = ix.csize > 128 ? 2 : 1;
            if (np.r0 >= 0) {
                const uint8_t *c = ix.codes + (size_t)np.r0 * (size_t)ix.csize;
                for (int l = 0; l < lines; ++l) asm volatile("prefetch.global.L1 [%0];" ::"l"(c + 128 * l));
            }
            if (np.r1 >= 0) {
                const uint8_t *c = ix.codes + (size_t)np.r1 * (size_t)ix.csize;
                for (int l = 0; l < lines; ++l) asm volatile("prefetch.global.L1 [%0];" ::"l"(c + 128 * l));
            }
        }
        if ((L.prefetch & kPrefetchBuckets) && np.u >= 0 && w.epoch) {
            // the first buckets the next expansion's visited check reads, towards L1 (the warp's own table)
            if (np.r0 >= 0) asm volatile("prefetch.global.L1 [%0];" ::"l"(w.spill + 8 * slot_of(np.r0, w.sbits - 3)));
            if (np.r1 >= 0) asm volatile("prefetch.global.L1 [%0];" ::"l"(w.spill + 8 * slot_of(np.r1, w.sbits - 3)));
        }
    }

    // ---- results ----
    int32_t *oid = bv.out_ids + (size_t)qi * (size_t)bv.out_stride;
    float *odis = bv.out_dis ? bv.out_dis + (size_t)qi * (size_t)bv.out_stride : nullptr;
    if (overflow) {
        for (int j = lane; j < bv.out_stride; j += 32) {
            oid[j] = -1;
            if (odis) odis[j] = __int_as_float(0x7f800000);
        }
        if (lane == 0) {
            bv.status[qi] = 1;
            atomicAdd(bv.overflow, 1u);
            if (bv.cmps) bv.cmps[qi] = cmps;
            if (bv.expansions) bv.expansions[qi] = nexp;
        }
        __syncwarp();
        return;
    }
    if (!refine) {
        // to_sorted (neighbor.hpp:421-428); entries past the pool size are reported as -1/inf
        for (int j = lane; j < bv.out_stride; j += 32) {
            int32_t id = -1;
            float dv = __int_as_float(0x7f800000);
            if (j < kq && j < S) {
                id = w.pid[j] & kIdMask;
                dv = IsIntKind<KIND>::value ? dist_of_key_int(w.pkey[j]) : dist_of_key_float(w.pkey[j]);
            }
            oid[j] = id;
            if (odis) odis[j] = dv;
        }
    } else {
        // Refiner::RefineImpl (refiner.hpp:92-110): FP32 distances of the first reorder_k ids,
        // k smallest by (distance, id), ascending
        const int avail = S < rk ? S : rk;
        int32_t *rid = w.pid;
        float *rdis = reinterpret_cast<float *>(w.pkey);
        for (int j = lane; j < avail; j += 32) rid[j] &= kIdMask;
        __syncwarp();
        // the refiner is FP32Quantizer<metric> with the searcher's metric, even where the first
        // pass compares codes by L2 (SQ4U)
        if (ix.metric == M_IP) refine_dists<M_IP>(ix, rid, rdis, avail, w.fq, lane);
        else refine_dists<M_L2>(ix, rid, rdis, avail, w.fq, lane);
        for (int j = lane; j < avail; j += 32) {
            const float dj = rdis[j];
            const int32_t ij = rid[j];
            int rank = 0;
            // (distance, id) order of Neighbor (neighbor.hpp:205-207); an id that entered the pool
            // twice (a repeated entry point) keeps both copies, ordered by position
            for (int i = 0; i < avail; ++i) {
                const float di = rdis[i];
                const int32_t ii = rid[i];
                rank += (di < dj) || (di == dj && (ii < ij || (ii == ij && i < j)));
            }
            if (rank < kq) {
                oid[rank] = ij;
                if (odis) odis[rank] = dj;
            }
        }
        const int nout = avail < kq ? avail : kq;
        for (int j = nout + lane; j < bv.out_stride; j += 32) {
            oid[j] = -1;
            if (odis) odis[j] = __int_as_float(0x7f800000);
        }
    }
    if (lane == 0) {
        bv.status[qi] = 0;
        if (bv.cmps) bv.cmps[qi] = cmps;
        if (bv.expansions) bv.expansions[qi] = nexp;
    }
    __syncwarp();
}

// Resident 256-thread blocks per SM the register allocation is held to: 64 registers a thread for the
// integer kinds and the 2-byte float rows (FP16 on 1M x 128 at ef 128: 2.67 ms with 128 registers,
// 2.11 ms with 64 — the few spilled words cost less than the resident warps they buy), 128 for the
// other float kinds (E5M2 on 1M x 960, where 1,000 queries fill less than one wave and the latency
// of each query decides: 80 registers spill in the distance loop and took ef 64 from 578 k to 310 k QPS)
template <int KIND>
struct SearchMinBlocks {
    static constexpr int value = IsIntKind<KIND>::value ? 4 : ((KIND == K_FP16 || KIND == K_BF16) ? 4 : 2);
};

template <int KIND, int METRIC, int LPR, int NCH = 0>
__global__ void __launch_bounds__(256, SearchMinBlocks<KIND>::value) search_kernel(IndexView ix, BatchView bv, WarpLayout L) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    unsigned char *ws = smem + (size_t)wib * (size_t)L.total;
    WarpState w;
    w.pkey = reinterpret_cast<uint32_t *>(ws + L.pool_key);
    w.pid = reinterpret_cast<int32_t *>(ws + L.pool_id);
    w.cand_id = reinterpret_cast<int32_t *>(ws + L.cand_id);
    w.cand_key = reinterpret_cast<uint32_t *>(ws + L.cand_key);
    w.acc_ub = reinterpret_cast<int32_t *>(ws + L.acc_ub);
    w.acc_key = reinterpret_cast<uint32_t *>(ws + L.acc_key);
    w.acc_id = reinterpret_cast<int32_t *>(ws + L.acc_id);
    w.fq = reinterpret_cast<float *>(ws + L.fq);
    w.qc = reinterpret_cast<uint32_t *>(ws + L.qc);
    w.stage = ws + L.stage;
    w.src = w.acc_ub;
    const size_t slot = (size_t)blockIdx.x * (blockDim.x >> 5) + wib;
    w.spill = bv.gtab ? bv.gtab + (slot << bv.gtab_bits) : nullptr;
    w.spill_epoch = bv.gtab ? bv.gtab_epoch + slot : nullptr;
    w.sbits = bv.gtab_bits;
    w.shift = bv.gtab_shift;
    w.epoch = 0;
    w.shared_first = L.table_bits > 0;
    w.tab = reinterpret_cast<int32_t *>(ws + L.table);
    w.tbits = L.table_bits;
    while (true) {
        unsigned t = 0;
        if (lane == 0) t = atomicAdd(bv.counter, 1u);
        t = __shfl_sync(kFull, t, 0);
        if (t >= (unsigned)bv.nq) break;
        const int qi = bv.order ? bv.order[t] : (int)t;
        search_one<KIND, METRIC, LPR, NCH>(ix, bv, L, w, qi, lane);
    }
}

// ComputerImpl::operator() for a list of ids (computer.hpp:67-72): one warp per query, the same
// query encoding and distance engines as the search.  refine=1 uses the refine store.
template <int KIND, int METRIC, int LPR>
__global__ void __launch_bounds__(128) distance_kernel(IndexView ix, int refine, const float *queries, int nq,
                                                       const int32_t *ids, int m, double *out, WarpLayout L) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int qi = blockIdx.x * (blockDim.x >> 5) + wib;
    if (qi >= nq) return;
    unsigned char *ws = smem + (size_t)wib * (size_t)L.total;
    WarpState w;
    w.pkey = reinterpret_cast<uint32_t *>(ws + L.pool_key);
    w.pid = reinterpret_cast<int32_t *>(ws + L.pool_id);
    w.cand_id = reinterpret_cast<int32_t *>(ws + L.cand_id);
    w.cand_key = reinterpret_cast<uint32_t *>(ws + L.cand_key);
    w.fq = reinterpret_cast<float *>(ws + L.fq);
    w.qc = reinterpret_cast<uint32_t *>(ws + L.qc);
    const float *q = queries + (size_t)qi * (size_t)ix.d;
    for (int j = lane; j < L.fq_len; j += 32) w.fq[j] = j < ix.d ? q[j] : 0.0f;
    __syncwarp();
    const int32_t qsq = prepare_query<KIND, METRIC>(ix, w, lane);
    for (int c0 = 0; c0 < m; c0 += kMaxDegree) {
        const int mm = (m - c0) < kMaxDegree ? (m - c0) : kMaxDegree;
        for (int j = lane; j < mm; j += 32) w.cand_id[j] = ids[(size_t)qi * m + c0 + j];
        __syncwarp();
        if (refine) {
            float *fo = reinterpret_cast<float *>(w.pkey);
            if (ix.metric == M_IP) refine_dists<M_IP>(ix, w.cand_id, fo, mm, w.fq, lane);
            else refine_dists<M_L2>(ix, w.cand_id, fo, mm, w.fq, lane);
            for (int j = lane; j < mm; j += 32) out[(size_t)qi * m + c0 + j] = (double)fo[j];
        } else {
            compute_dists<KIND, METRIC, LPR>(ix, w, mm, qsq, lane);
            for (int j = lane; j < mm; j += 32) {
                const uint32_t k = w.cand_key[j];
                out[(size_t)qi * m + c0 + j] =
                    IsIntKind<KIND>::value ? (double)dist_of_key_int(k) : (double)dist_of_key_float(k);
            }
        }
        __syncwarp();
    }
}

}  // namespace

}  // namespace gsx
