// NSG / SSG graph construction on the GPU (reference glass/nsg/nsg.hpp:55-104 NSG::Build, bound to
// Python as Index("NSG" | "SSG", ...).build(data), python/bindings.cc:60-87).
//
// Stages, all writing the glass graph layout (N x R int32, -1 padded, one entry point):
//   1. Exact kNN graph of the base set (knn_k neighbours, self excluded, by the fp32 distance below):
//      tensor-core candidate lists, rescored; rows a full list may have cut short are redone by
//      brute force (the reference builds the graph with NN-Descent, nsg/nndescent.hpp; the exact
//      graph is its limit).
//   2. Entry point: the row nearest to the centroid (nsg.hpp:106-127).
//   3. Link (nsg.hpp:160-246): one warp per node runs the reference's search over the kNN graph
//      from the entry point (LinearPool of L entries, nsg.hpp:129-158), keeps the C = R + 100
//      nearest of every row it evaluated plus the node's own kNN row (sync_prune), and prunes them
//      to R with the NSG rule (d(j,k) < d(i,k) occludes) or the SSG angle rule (cos > cos 60deg).
//   4. Reverse links (nsg.hpp:248-315): every edge i -> j offers i to j's list; when the list would
//      exceed R it is pruned with the NSG rule.  The reference inserts the offers one at a time
//      under per-node locks in whatever order its threads reach them; here every node takes all of
//      its offers at once (its own list and the offers, nearest first), so the result does not
//      depend on scheduling.
//   5. Connectivity (nsg.hpp:317-404): breadth-first search from the entry point and attachment of
//      every unreached node to the nearest node with a free slot found by a search from the entry
//      point.  This stage is sequential, like the reference's, and runs on the host.
// Distances are squared L2 in fp32 with a fixed order: four fmaf chains over dimensions j = 4i + t,
// summed (c0 + c1) + (c2 + c3), identical on the device and in the host stage, so the build is
// deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "gsx_host.h"

namespace gsx {

int knn_select(const float *d_base, int64_t N, int32_t d, const float *d_queries, int32_t nq, int32_t k, int32_t ip,
               int min_chunks, int64_t self_base, int fp32_l2, int32_t *d_ids, float *d_dis, int32_t *exact_inputs,
               int32_t *rechecked, cudaStream_t st);

namespace {

constexpr int kLinkWarps = 8;
constexpr int kRevWarps = 8;

__host__ __device__ __forceinline__ float l2_rows(const float *a, const float *b, int d) {
    float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
    int j = 0;
    for (; j + 3 < d; j += 4) {
        const float t0 = a[j] - b[j], t1 = a[j + 1] - b[j + 1], t2 = a[j + 2] - b[j + 2], t3 = a[j + 3] - b[j + 3];
        c0 = fmaf(t0, t0, c0);
        c1 = fmaf(t1, t1, c1);
        c2 = fmaf(t2, t2, c2);
        c3 = fmaf(t3, t3, c3);
    }
    for (; j < d; ++j) {
        const float t = a[j] - b[j];
        const int c = j & 3;
        if (c == 0) c0 = fmaf(t, t, c0);
        else if (c == 1) c1 = fmaf(t, t, c1);
        else c2 = fmaf(t, t, c2);
    }
    return (c0 + c1) + (c2 + c3);
}

// The same sum with 16-byte loads (rows 16-byte aligned, d a multiple of 4).
__device__ __forceinline__ float l2_rows4(const float *a, const float *b, int d) {
    float c0 = 0.0f, c1 = 0.0f, c2 = 0.0f, c3 = 0.0f;
    for (int j = 0; j < d; j += 4) {
        const float4 x = __ldg(reinterpret_cast<const float4 *>(a + j));
        const float4 y = __ldg(reinterpret_cast<const float4 *>(b + j));
        const float t0 = x.x - y.x, t1 = x.y - y.y, t2 = x.z - y.z, t3 = x.w - y.w;
        c0 = fmaf(t0, t0, c0);
        c1 = fmaf(t1, t1, c1);
        c2 = fmaf(t2, t2, c2);
        c3 = fmaf(t3, t3, c3);
    }
    return (c0 + c1) + (c2 + c3);
}

__device__ __forceinline__ float dist_rows(const float *x, int d, bool vec4, int32_t a, int32_t b) {
    const float *ra = x + (size_t)a * d, *rb = x + (size_t)b * d;
    return vec4 ? l2_rows4(ra, rb, d) : l2_rows(ra, rb, d);
}

// -------------------------------------------------------------------------------------------
// entry point: row nearest to the centroid

__global__ void column_sums(const float *__restrict__ x, int64_t N, int d, double *__restrict__ sums) {
    // one block per column group of 32, rows strided over the grid's y dimension
    const int j = blockIdx.x * 32 + (threadIdx.x & 31);
    if (j >= d) return;
    double s = 0.0;
    for (int64_t r = (int64_t)blockIdx.y * (blockDim.x >> 5) + (threadIdx.x >> 5); r < N;
         r += (int64_t)gridDim.y * (blockDim.x >> 5))
        s += (double)x[r * d + j];
    atomicAdd(&sums[j], s);
}

__global__ void centroid_of(const double *__restrict__ sums, int64_t N, int d, float *__restrict__ c) {
    for (int j = threadIdx.x; j < d; j += blockDim.x) c[j] = (float)(sums[j] / (double)N);
}

// key = (distance bits << 32) | row, minimised; distances are >= 0, so the bits order like values
__global__ void nearest_to(const float *__restrict__ x, int64_t N, int d, const float *__restrict__ c,
                           unsigned long long *__restrict__ best) {
    unsigned long long m = ~0ull;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x) {
        const float dd = l2_rows(c, x + r * d, d);
        const unsigned long long key = ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned long long)r;
        m = key < m ? key : m;
    }
    for (int o = 16; o; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
        m = v < m ? v : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMin(best, m);
}

// -------------------------------------------------------------------------------------------
// link: search over the kNN graph + prune (one warp per node)

struct LinkParams {
    const float *x;
    int N, d, vec4;
    const int32_t *knng;
    int K;
    int ep, L, C, R, ssg;
    float threshold;
    const int32_t *nodes;  // nodes to process (nullptr: 0..n_nodes-1)
    int n_nodes;
    int32_t *out_ids;  // N x R
    float *out_dis;
    unsigned long long *vis;  // per warp 2^vis_bits slots: (epoch << 32) | id
    int vis_bits;
    unsigned *counter;
    int32_t *overflow_nodes;
    unsigned *n_overflow;
};

struct LinkWarp {
    int32_t *pid;  // pool ids (bit 31 = expanded), L + 1 entries
    float *pd;
    int32_t *fid;  // the C nearest evaluated rows by (distance, id), C + 1 entries
    float *fd;
    int32_t *rid;  // pruned result, R entries
    float *rd;
    int32_t *edge;  // new neighbours of the expanded node, K entries
    float *ed;
};

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Lanes of a 32-entry piece of a row that come before the row's first -1; sets `stop` when the
// piece holds that -1 (the reference stops reading a row there).
__device__ __forceinline__ unsigned row_prefix(bool in_row, int32_t v, bool &stop) {
    const unsigned inrow = __ballot_sync(0xffffffffu, in_row);
    const unsigned neg = __ballot_sync(0xffffffffu, in_row && v == -1);
    if (!neg) return inrow;
    stop = true;
    const int f = __ffs(neg) - 1;
    return f == 0 ? 0u : (inrow & (0xffffffffu >> (32 - f)));
}

// Visited set: open addressing with linear probing in the warp's own table; entries of earlier
// epochs read as empty.  Returns 1 if u was new, 0 if seen, -1 if the table is too full.
__device__ __forceinline__ int visit(unsigned long long *tab, unsigned mask, int shift, unsigned epoch, int32_t u) {
    const unsigned long long mine = ((unsigned long long)epoch << 32) | (unsigned)u;
    unsigned h = ((unsigned)u * 2654435761u) >> shift;
    for (unsigned probe = 0; probe <= mask; ++probe) {
        unsigned long long cur = __ldcg(&tab[h]);
        while ((unsigned)(cur >> 32) != epoch) {
            const unsigned long long old = atomicCAS(&tab[h], cur, mine);
            if (old == cur) return 1;
            cur = old;
        }
        if ((unsigned)cur == (unsigned)u) return 0;
        h = (h + 1) & mask;
    }
    return -1;
}

__device__ __forceinline__ bool seen(const unsigned long long *tab, unsigned mask, int shift, unsigned epoch,
                                     int32_t u) {
    unsigned h = ((unsigned)u * 2654435761u) >> shift;
    for (unsigned probe = 0; probe <= mask; ++probe) {
        const unsigned long long cur = __ldcg(&tab[h]);
        if ((unsigned)(cur >> 32) != epoch) return false;
        if ((unsigned)cur == (unsigned)u) return true;
        h = (h + 1) & mask;
    }
    return false;
}

// LinearPool::insert (neighbor.hpp:382-396): upper-bound position by distance, rejected when full
// and not nearer than the last entry.
__device__ __forceinline__ void pool_insert(const LinkWarp &w, int &size, int &cur, int cap, int32_t u, float dd,
                                            int lane) {
    if (size == cap && dd >= w.pd[size - 1]) return;
    int lo = 0;
    for (int b = 0; b < size; b += 32) {
        const int i = b + lane;
        lo += __popc(__ballot_sync(0xffffffffu, i < size && w.pd[i] <= dd));
    }
    for (int top = size; top > lo; top -= 32) {
        const int i = top - 1 - lane;
        int32_t a = 0;
        float b = 0.0f;
        if (i >= lo) {
            a = w.pid[i];
            b = w.pd[i];
        }
        __syncwarp();
        if (i >= lo) {
            w.pid[i + 1] = a;
            w.pd[i + 1] = b;
        }
        __syncwarp();
    }
    if (lane == 0) {
        w.pid[lo] = u;
        w.pd[lo] = dd;
    }
    __syncwarp();
    if (size < cap) ++size;
    if (lo < cur) cur = lo;
}

__device__ __forceinline__ bool key_less(float da, int32_t ia, float db, int32_t ib) {
    return da < db || (da == db && ia < ib);
}

// keeps the C smallest (distance, id) pairs, sorted
__device__ __forceinline__ void top_insert(const LinkWarp &w, int &n, int cap, int32_t u, float dd, int lane) {
    if (n == cap && !key_less(dd, u, w.fd[n - 1], w.fid[n - 1])) return;
    int pos = 0;
    for (int b = 0; b < n; b += 32) {
        const int i = b + lane;
        pos += __popc(__ballot_sync(0xffffffffu, i < n && key_less(w.fd[i], w.fid[i], dd, u)));
    }
    for (int top = n; top > pos; top -= 32) {
        const int i = top - 1 - lane;
        int32_t a = 0;
        float b = 0.0f;
        if (i >= pos) {
            a = w.fid[i];
            b = w.fd[i];
        }
        __syncwarp();
        if (i >= pos) {
            w.fid[i + 1] = a;
            w.fd[i + 1] = b;
        }
        __syncwarp();
    }
    if (lane == 0) {
        w.fid[pos] = u;
        w.fd[pos] = dd;
    }
    __syncwarp();
    if (n < cap) ++n;
}

// occlusion of candidate (p, pd) by the kept results (nsg.hpp:208-231)
__device__ __forceinline__ bool occluded(const LinkParams &P, const LinkWarp &w, int nres, int32_t p, float pdist,
                                         bool ssg, int lane) {
    bool occ = false;
    for (int b = 0; b < nres; b += 32) {
        const int t = b + lane;
        bool o = false;
        if (t < nres) {
            const int32_t r = w.rid[t];
            if (r == p) {
                o = true;
            } else {
                const float djk = dist_rows(P.x, P.d, P.vec4, r, p);
                if (ssg) {
                    const float rdist = w.rd[t];
                    const float num = __fsub_rn(__fadd_rn(pdist, rdist), djk);
                    const float cosij = __fdiv_rn(__fdiv_rn(num, 2.0f), __fsqrt_rn(__fmul_rn(pdist, rdist)));
                    o = cosij > P.threshold;
                } else {
                    o = djk < pdist;
                }
            }
        }
        if (__any_sync(0xffffffffu, o)) {
            occ = true;
            break;
        }
    }
    return occ;
}

__global__ void __launch_bounds__(32 * kLinkWarps) nsg_link(LinkParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int L = P.L, C = P.C, R = P.R, K = P.K;
    const size_t per_warp = (size_t)(L + 1) * 8 + (size_t)(C + 1) * 8 + (size_t)R * 8 + (size_t)K * 8;
    unsigned char *base = smem + per_warp * wib;
    LinkWarp w;
    w.pid = reinterpret_cast<int32_t *>(base);
    w.pd = reinterpret_cast<float *>(w.pid + (L + 1));
    w.fid = reinterpret_cast<int32_t *>(w.pd + (L + 1));
    w.fd = reinterpret_cast<float *>(w.fid + (C + 1));
    w.rid = reinterpret_cast<int32_t *>(w.fd + (C + 1));
    w.rd = reinterpret_cast<float *>(w.rid + R);
    w.edge = reinterpret_cast<int32_t *>(w.rd + R);
    w.ed = reinterpret_cast<float *>(w.edge + K);
    const size_t gw = (size_t)blockIdx.x * kLinkWarps + wib;
    unsigned long long *tab = P.vis + (gw << P.vis_bits);
    const unsigned mask = (1u << P.vis_bits) - 1;
    const int shift = 32 - P.vis_bits;
    const int fill_cap = (int)((mask + 1) / 4 * 3);
    unsigned epoch = 0;
    while (true) {
        int item = 0;
        if (lane == 0) item = (int)atomicAdd(P.counter, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= P.n_nodes) break;
        const int32_t q = P.nodes ? P.nodes[item] : item;
        ++epoch;
        bool bad = false;
        int nvis = 0;
        // search_on_graph (nsg.hpp:129-158)
        int size = 0, cur = 0, nfs = 0;
        {
            const float d0 = dist_rows(P.x, P.d, P.vec4, q, P.ep);
            pool_insert(w, size, cur, L, P.ep, d0, lane);
            int r = 0;
            if (lane == 0) r = visit(tab, mask, shift, epoch, P.ep);
            r = __shfl_sync(0xffffffffu, r, 0);
            bad |= r < 0;
            nvis = 1;
            top_insert(w, nfs, C, P.ep, d0, lane);
        }
        while (!bad && cur < size && cur < L) {
            // pop (neighbor.hpp:398-405)
            const int32_t u = w.pid[cur] & 0x7fffffff;
            __syncwarp();
            if (lane == 0) w.pid[cur] |= (int32_t)0x80000000u;
            __syncwarp();
            while (cur < size && (w.pid[cur] & (int32_t)0x80000000u)) ++cur;
            // the row up to its first -1; the unvisited ones in row order
            const int32_t *row = P.knng + (size_t)u * K;
            int n = 0;
            bool stop = false;
            for (int b = 0; b < K && !stop; b += 32) {
                const int j = b + lane;
                const int32_t v = j < K ? row[j] : -1;
                const unsigned valid = row_prefix(j < K, v, stop);
                int r = 0;
                if ((valid >> lane) & 1u) r = visit(tab, mask, shift, epoch, v);
                bad |= __any_sync(0xffffffffu, r < 0);
                const unsigned fresh = __ballot_sync(0xffffffffu, r == 1);
                if (r == 1) w.edge[n + __popc(fresh & lanemask_lt())] = v;
                n += __popc(fresh);
            }
            __syncwarp();
            nvis += n;
            if (bad || nvis > fill_cap) {
                bad = true;
                break;
            }
            for (int i = lane; i < n; i += 32) w.ed[i] = dist_rows(P.x, P.d, P.vec4, q, w.edge[i]);
            __syncwarp();
            for (int i = 0; i < n; ++i) {
                const int32_t v = w.edge[i];
                const float dv = w.ed[i];
                pool_insert(w, size, cur, L, v, dv, lane);
                top_insert(w, nfs, C, v, dv, lane);
            }
        }
        if (bad) {
            if (lane == 0) {
                const unsigned at = atomicAdd(P.n_overflow, 1u);
                P.overflow_nodes[at] = q;
            }
            continue;
        }
        // sync_prune (nsg.hpp:180-246): the node's own kNN row, then the C nearest, pruned to R
        {
            const int32_t *row = P.knng + (size_t)q * K;
            bool stop = false;
            for (int b = 0; b < K && !stop; b += 32) {
                const int j = b + lane;
                const int32_t v = j < K ? row[j] : -1;
                const unsigned valid = row_prefix(j < K, v, stop);
                bool fresh = ((valid >> lane) & 1u) && !seen(tab, mask, shift, epoch, v);
                float dv = 0.0f;
                if (fresh) dv = dist_rows(P.x, P.d, P.vec4, q, v);
                unsigned fm = __ballot_sync(0xffffffffu, fresh);
                while (fm) {
                    const int src = __ffs(fm) - 1;
                    fm &= fm - 1;
                    const int32_t vv = __shfl_sync(0xffffffffu, v, src);
                    const float dd = __shfl_sync(0xffffffffu, dv, src);
                    top_insert(w, nfs, C, vv, dd, lane);
                }
            }
        }
        int nres = 0;
        int start = 0;
        if (nfs > 0 && w.fid[0] == q) start = 1;
        if (start < nfs) {
            if (lane == 0) {
                w.rid[0] = w.fid[start];
                w.rd[0] = w.fd[start];
            }
            __syncwarp();
            nres = 1;
            while (nres < R && ++start < nfs) {
                const int32_t p = w.fid[start];
                const float pdist = w.fd[start];
                if (!occluded(P, w, nres, p, pdist, P.ssg != 0, lane)) {
                    if (lane == 0) {
                        w.rid[nres] = p;
                        w.rd[nres] = pdist;
                    }
                    __syncwarp();
                    ++nres;
                }
            }
        }
        for (int i = lane; i < R; i += 32) {
            P.out_ids[(size_t)q * R + i] = i < nres ? w.rid[i] : -1;
            P.out_dis[(size_t)q * R + i] = i < nres ? w.rd[i] : 0.0f;
        }
        __syncwarp();
    }
}

// -------------------------------------------------------------------------------------------
// reverse links

__global__ void count_in(const int32_t *__restrict__ ids, int64_t n_edges, unsigned *__restrict__ indeg) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_edges; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = ids[e];
        if (v >= 0) atomicAdd(&indeg[v], 1u);
    }
}

// exclusive scan of n counts into off[0..n] (one block per 1024 entries, then the block totals)
__global__ void scan_blocks(const unsigned *__restrict__ in, int64_t n, int64_t *__restrict__ out,
                            int64_t *__restrict__ totals) {
    __shared__ int64_t s[1024];
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    const int64_t v = i < n ? (int64_t)in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int64_t a = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += a;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == 1023) totals[blockIdx.x] = s[1023];
}

__global__ void scan_totals(int64_t *__restrict__ totals, int64_t nb) {
    // one block, sequential over chunks of 1024 with a carry
    __shared__ int64_t s[1024];
    int64_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += 1024) {
        const int64_t i = b0 + threadIdx.x;
        const int64_t v = i < nb ? totals[i] : 0;
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const int64_t a = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : 0;
            __syncthreads();
            s[threadIdx.x] += a;
            __syncthreads();
        }
        if (i < nb) totals[i] = carry + s[threadIdx.x] - v;
        const int64_t blk = s[1023];
        __syncthreads();
        carry += blk;
    }
    if (threadIdx.x == 0) totals[nb] = carry;
}

__global__ void add_totals(int64_t *__restrict__ out, int64_t n, const int64_t *__restrict__ totals) {
    const int64_t i = (int64_t)blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += totals[blockIdx.x];
    if (i == 0) out[n] = totals[gridDim.x];
}

__global__ void fill_in(const int32_t *__restrict__ ids, const float *__restrict__ dis, int64_t n_edges, int R,
                        const int64_t *__restrict__ off, unsigned *__restrict__ fillc, int32_t *__restrict__ src,
                        float *__restrict__ sd) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_edges; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = ids[e];
        if (v < 0) continue;
        const int64_t at = off[v] + atomicAdd(&fillc[v], 1u);
        src[at] = (int32_t)(e / R);
        sd[at] = dis[e];
    }
}

__device__ __forceinline__ unsigned long long dkey(float d, int32_t id) {
    return ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)id;
}

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long m) {
    for (int o = 16; o; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
        m = v < m ? v : m;
    }
    return m;
}

struct RevParams {
    const float *x;
    int N, d, vec4, R;
    const int32_t *ids;  // link lists, N x R
    const float *dis;
    const int64_t *off;  // offers to node j: [off[j], off[j+1])
    int32_t *src;        // offering node (set to -1 when it is already in j's list)
    const float *sd;
    int32_t *out;  // final lists, N x R
};

// One warp per node j: its list and its offers, nearest first, pruned to R with the NSG rule when
// they exceed R (nsg.hpp:248-315); offers already in the list are dropped.
__global__ void __launch_bounds__(32 * kRevWarps) reverse_merge(RevParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int R = P.R;
    int32_t *oid = reinterpret_cast<int32_t *>(smem) + (size_t)wib * 4 * R;
    float *od = reinterpret_cast<float *>(oid + R);
    int32_t *rid = reinterpret_cast<int32_t *>(od + R);
    float *rd = reinterpret_cast<float *>(rid + R);
    LinkParams LP{};
    LP.x = P.x;
    LP.d = P.d;
    LP.vec4 = P.vec4;
    LinkWarp w{};
    w.rid = rid;
    w.rd = rd;
    for (int64_t j = (int64_t)blockIdx.x * kRevWarps + wib; j < P.N; j += (int64_t)gridDim.x * kRevWarps) {
        int nout = 0;
        for (int b = 0; b < R; b += 32) {
            const int i = b + lane;
            const int32_t v = i < R ? P.ids[j * R + i] : -1;
            const float dv = i < R ? P.dis[j * R + i] : 0.0f;
            if (i < R) {
                oid[i] = v;
                od[i] = dv;
            }
            nout += __popc(__ballot_sync(0xffffffffu, i < R && v >= 0));
        }
        __syncwarp();
        const int64_t b0 = P.off[j], b1 = P.off[j + 1];
        int nin = 0;
        for (int64_t e = b0 + lane; e < b1; e += 32) {
            const int32_t s = P.src[e];
            bool dup = false;
            for (int t = 0; t < nout; ++t) dup |= oid[t] == s;
            if (dup) P.src[e] = -1;
            nin += !dup;
        }
        for (int o = 16; o; o >>= 1) nin += __shfl_xor_sync(0xffffffffu, nin, o);
        __syncwarp();
        int nres = 0;
        if (nout + nin <= R) {
            // everything fits: the list, then the offers nearest first
            for (int i = lane; i < nout; i += 32) {
                rid[i] = oid[i];
                rd[i] = od[i];
            }
            nres = nout;
            unsigned long long last = 0;
            bool first = true;
            for (int c = 0; c < nin; ++c) {
                unsigned long long m = ~0ull;
                for (int64_t e = b0 + lane; e < b1; e += 32) {
                    const int32_t s = P.src[e];
                    if (s < 0) continue;
                    const unsigned long long k = dkey(P.sd[e], s);
                    if ((first || k > last) && k < m) m = k;
                }
                m = warp_min64(m);
                if (lane == 0) {
                    rid[nres] = (int32_t)(unsigned)m;
                    rd[nres] = __uint_as_float((unsigned)(m >> 32));
                }
                ++nres;
                last = m;
                first = false;
            }
            __syncwarp();
        } else {
            // union nearest first; the first is kept, the rest pruned against the kept ones
            unsigned long long last = 0;
            bool first = true;
            const int total = nout + nin;
            for (int c = 0; c < total && nres < R; ++c) {
                unsigned long long m = ~0ull;
                for (int i = lane; i < nout; i += 32) {
                    const unsigned long long k = dkey(od[i], oid[i]);
                    if ((first || k > last) && k < m) m = k;
                }
                for (int64_t e = b0 + lane; e < b1; e += 32) {
                    const int32_t s = P.src[e];
                    if (s < 0) continue;
                    const unsigned long long k = dkey(P.sd[e], s);
                    if ((first || k > last) && k < m) m = k;
                }
                m = warp_min64(m);
                last = m;
                first = false;
                const int32_t p = (int32_t)(unsigned)m;
                const float pdist = __uint_as_float((unsigned)(m >> 32));
                if (nres == 0 || !occluded(LP, w, nres, p, pdist, false, lane)) {
                    if (lane == 0) {
                        rid[nres] = p;
                        rd[nres] = pdist;
                    }
                    __syncwarp();
                    ++nres;
                }
            }
        }
        __syncwarp();
        for (int i = lane; i < R; i += 32) P.out[j * R + i] = i < nres ? rid[i] : -1;
        __syncwarp();
    }
}

// -------------------------------------------------------------------------------------------
// connectivity (host): tree_grow / bfs / attach_unlinked, nsg.hpp:317-404

struct HostPool {  // LinearPool<float> (neighbor.hpp:320-433) without its visited set
    std::vector<int32_t> id;
    std::vector<float> dd;
    int size = 0, cur = 0, cap = 0;
    explicit HostPool(int c) : id(c + 1), dd(c + 1), cap(c) {}
    void insert(int32_t u, float d) {
        if (size == cap && d >= dd[size - 1]) return;
        int lo = 0, hi = size;
        while (lo < hi) {
            const int mid = (lo + hi) / 2;
            if (dd[mid] > d) hi = mid;
            else lo = mid + 1;
        }
        std::memmove(&id[lo + 1], &id[lo], (size_t)(size - lo) * 4);
        std::memmove(&dd[lo + 1], &dd[lo], (size_t)(size - lo) * 4);
        id[lo] = u;
        dd[lo] = d;
        if (size < cap) ++size;
        if (lo < cur) cur = lo;
    }
    int32_t pop() {
        id[cur] |= (int32_t)0x80000000u;
        const int pre = cur;
        while (cur < size && (id[cur] & (int32_t)0x80000000u)) ++cur;
        return id[pre] & 0x7fffffff;
    }
    bool has_next() const { return cur < size && cur < cap; }
};

void bfs(const std::vector<int32_t> &g, int R, std::vector<uint8_t> &vis, int32_t root, int64_t &cnt) {
    std::vector<int32_t> qu;
    qu.push_back(root);
    if (!vis[root]) {
        ++cnt;
        vis[root] = 1;
    }
    for (size_t h = 0; h < qu.size(); ++h) {
        const int32_t u = qu[h];
        for (int i = 0; i < R; ++i) {
            const int32_t v = g[(size_t)u * R + i];
            if (v < 0) break;
            if (vis[v]) continue;
            vis[v] = 1;
            ++cnt;
            qu.push_back(v);
        }
    }
}

int tree_grow(const float *x, int64_t N, int d, int R, int L, int32_t ep, std::vector<int32_t> &g, int32_t *attached) {
    std::vector<int32_t> deg(N);
    for (int64_t i = 0; i < N; ++i) {
        int c = 0;
        while (c < R && g[(size_t)i * R + c] >= 0) ++c;
        deg[i] = c;
    }
    std::vector<uint8_t> vis(N, 0);
    int64_t cnt = 0, scan = 0;
    int32_t root = ep;
    int32_t n_att = 0;
    std::vector<uint8_t> seen;
    while (true) {
        bfs(g, R, vis, root, cnt);
        if (cnt >= N) break;
        while (scan < N && vis[scan]) ++scan;
        const int32_t id = (int32_t)scan;
        // search_on_graph from the entry point for `id` over the current graph
        seen.assign(N, 0);
        HostPool pool(L);
        std::vector<std::pair<float, int32_t>> full;
        const float *q = x + (size_t)id * d;
        const float d0 = l2_rows(q, x + (size_t)ep * d, d);
        pool.insert(ep, d0);
        seen[ep] = 1;
        full.push_back({d0, ep});
        while (pool.has_next()) {
            const int32_t u = pool.pop();
            for (int i = 0; i < R; ++i) {
                const int32_t v = g[(size_t)u * R + i];
                if (v < 0) break;
                if (seen[v]) continue;
                seen[v] = 1;
                const float dv = l2_rows(q, x + (size_t)v * d, d);
                pool.insert(v, dv);
                full.push_back({dv, v});
            }
        }
        std::sort(full.begin(), full.end());
        int32_t node = -1;
        for (auto &f : full)
            if (deg[f.second] < R && f.second != id) {
                node = f.second;
                break;
            }
        if (node < 0) {
            // the reference picks a random reached node with a free slot; the first one by id is
            // taken here, so that the build stays deterministic
            for (int64_t i = 0; i < N; ++i)
                if (vis[i] && deg[i] < R && i != id) {
                    node = (int32_t)i;
                    break;
                }
            if (node < 0) return fail(GSX_ERR_STATE, "no node with a free slot to attach node %d", id);
        }
        g[(size_t)node * R + deg[node]] = id;
        deg[node]++;
        root = node;
        ++n_att;
    }
    *attached = n_att;
    return GSX_OK;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

}  // namespace gsx

using namespace gsx;

extern "C" int gsx_graph_build_nsg(const float *data, int64_t N, int32_t d, int32_t R, int32_t L, int32_t use_ssg,
                                   int32_t knn_k, int32_t *knng_out, double *seconds, gsx_graph **out) {
    try {
        if (!data || !out || N < 2 || d <= 0 || R <= 0 || L < 0 || knn_k <= 0)
            return fail(GSX_ERR_INVALID, "bad graph-build arguments");
        if (N > (int64_t)INT32_MAX) return fail(GSX_ERR_INVALID, "N too large");
        if (R > 256 || knn_k > 64) return fail(GSX_ERR_UNSUPPORTED, "R <= 256 and knn_k <= 64 are supported");
        if (d > 128) return fail(GSX_ERR_UNSUPPORTED, "the GPU graph build supports d <= 128 (tensor-core kNN)");
        if (L == 0) L = R + 32;  // nsg.hpp:47
        const int C = R + 100;
        const int K = (int)std::min<int64_t>(knn_k, N - 1);
        int dev = 0, nsm = 0, ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            return fail(GSX_ERR_CUDA, "no CUDA device is visible");
        }
        GSX_CUDA(cudaGetDevice(&dev));
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaStream_t st = nullptr;
        GSX_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        } guard{st};
        double t[5] = {0, 0, 0, 0, 0};
        const double t0 = now_s();
        int rc;
        DevBuf x, knng, cen, sums, best, ids, dis, visb, cnt, ovl, indeg, off, tot, fillc, src, sd, fin;
        if ((rc = x.ensure((size_t)N * d * 4)) || (rc = knng.ensure((size_t)N * K * 4))) return rc;
        GSX_CUDA(cudaMemcpyAsync(x.p, data, (size_t)N * d * 4, cudaMemcpyHostToDevice, st));
        // 1. kNN graph, in query blocks that keep the candidate lists near 1 GB
        const int64_t qblock = 1 << 18;
        int64_t n_re = 0;
        for (int64_t q0 = 0; q0 < N; q0 += qblock) {
            const int nq = (int)std::min<int64_t>(qblock, N - q0);
            int32_t re = 0;
            if ((rc = knn_select(x.as<float>(), N, d, x.as<float>() + q0 * d, nq, K, 0, 16, q0, 1,
                                 knng.as<int32_t>() + q0 * K, nullptr, nullptr, &re, st)))
                return rc;
            n_re += re;
        }
        // 2. entry point
        if ((rc = sums.ensure((size_t)d * 8)) || (rc = cen.ensure((size_t)d * 4)) || (rc = best.ensure(8))) return rc;
        GSX_CUDA(cudaMemsetAsync(sums.p, 0, (size_t)d * 8, st));
        GSX_CUDA(cudaMemsetAsync(best.p, 0xff, 8, st));
        column_sums<<<dim3((d + 31) / 32, 2 * nsm), 256, 0, st>>>(x.as<float>(), N, d, sums.as<double>());
        centroid_of<<<1, 256, 0, st>>>(sums.as<double>(), N, d, cen.as<float>());
        nearest_to<<<4 * nsm, 256, 0, st>>>(x.as<float>(), N, d, cen.as<float>(), best.as<unsigned long long>());
        GSX_CUDA(cudaGetLastError());
        unsigned long long bk = 0;
        GSX_CUDA(cudaMemcpyAsync(&bk, best.p, 8, cudaMemcpyDeviceToHost, st));
        GSX_CUDA(cudaStreamSynchronize(st));
        const int32_t ep = (int32_t)(unsigned)bk;
        if (knng_out) GSX_CUDA(cudaMemcpy(knng_out, knng.p, (size_t)N * K * 4, cudaMemcpyDeviceToHost));
        const double t1 = now_s();
        t[0] = t1 - t0;
        // 3. link
        LinkParams P{};
        P.x = x.as<float>();
        P.N = (int)N;
        P.d = d;
        P.vec4 = (d % 4) == 0;
        P.knng = knng.as<int32_t>();
        P.K = K;
        P.ep = ep;
        P.L = L;
        P.C = C;
        P.R = R;
        P.ssg = use_ssg ? 1 : 0;
        P.threshold = (float)std::cos(60.0 / 180.0 * 3.14159265358979323846264);  // nsg.hpp:40
        if ((rc = ids.ensure((size_t)N * R * 4)) || (rc = dis.ensure((size_t)N * R * 4)) || (rc = cnt.ensure(16)) ||
            (rc = ovl.ensure((size_t)N * 4)))
            return rc;
        P.out_ids = ids.as<int32_t>();
        P.out_dis = dis.as<float>();
        P.counter = cnt.as<unsigned>();
        P.n_overflow = cnt.as<unsigned>() + 1;
        P.overflow_nodes = ovl.as<int32_t>();
        const size_t per_warp = (size_t)(L + 1) * 8 + (size_t)(C + 1) * 8 + (size_t)R * 8 + (size_t)K * 8;
        const size_t link_smem = per_warp * kLinkWarps;
        if (link_smem > 200 * 1024) return fail(GSX_ERR_UNSUPPORTED, "L or R too large for the link kernel");
        GSX_CUDA(cudaFuncSetAttribute(nsg_link, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)link_smem));
        int per_sm = 0;
        GSX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nsg_link, 32 * kLinkWarps, link_smem));
        per_sm = std::max(1, per_sm);
        // pass 1: 2^14-slot visited tables; nodes whose search outgrows them run again with 2^20 slots
        // on fewer warps
        std::vector<int32_t> redo;
        for (int pass = 0; pass < 2; ++pass) {
            const int bits = pass == 0 ? 14 : 20;
            int blocks = pass == 0 ? per_sm * nsm : std::min(per_sm * nsm, std::max(1, (int)((redo.size() + 7) / 8)));
            if (pass == 1) {
                if (redo.empty()) break;
                blocks = std::min(blocks, 32);
            }
            if ((rc = visb.ensure(((size_t)blocks * kLinkWarps) << bits << 3))) return rc;
            GSX_CUDA(cudaMemsetAsync(visb.p, 0, ((size_t)blocks * kLinkWarps) << bits << 3, st));
            GSX_CUDA(cudaMemsetAsync(cnt.p, 0, 8, st));
            P.vis = visb.as<unsigned long long>();
            P.vis_bits = bits;
            DevBuf nodes;
            if (pass == 0) {
                P.nodes = nullptr;
                P.n_nodes = (int)N;
            } else {
                if ((rc = nodes.ensure(redo.size() * 4))) return rc;
                GSX_CUDA(cudaMemcpyAsync(nodes.p, redo.data(), redo.size() * 4, cudaMemcpyHostToDevice, st));
                P.nodes = nodes.as<int32_t>();
                P.n_nodes = (int)redo.size();
            }
            nsg_link<<<blocks, 32 * kLinkWarps, link_smem, st>>>(P);
            GSX_CUDA(cudaGetLastError());
            unsigned hc[2] = {0, 0};
            GSX_CUDA(cudaMemcpyAsync(hc, cnt.p, 8, cudaMemcpyDeviceToHost, st));
            GSX_CUDA(cudaStreamSynchronize(st));
            redo.assign(hc[1], 0);
            if (hc[1]) GSX_CUDA(cudaMemcpy(redo.data(), ovl.p, (size_t)hc[1] * 4, cudaMemcpyDeviceToHost));
            if (pass == 1 && !redo.empty())
                return fail(GSX_ERR_NOMEM, "%zu nodes visited more than 786,432 rows while linking", redo.size());
        }
        visb.release();
        const double t2 = now_s();
        t[1] = t2 - t1;
        // 4. reverse links
        const int64_t n_edges = N * (int64_t)R;
        const int64_t nb = (N + 1023) / 1024;
        if ((rc = indeg.ensure((size_t)N * 4)) || (rc = off.ensure((size_t)(N + 1) * 8)) ||
            (rc = tot.ensure((size_t)(nb + 1) * 8)) || (rc = fillc.ensure((size_t)N * 4)) ||
            (rc = src.ensure((size_t)n_edges * 4)) || (rc = sd.ensure((size_t)n_edges * 4)) ||
            (rc = fin.ensure((size_t)n_edges * 4)))
            return rc;
        GSX_CUDA(cudaMemsetAsync(indeg.p, 0, (size_t)N * 4, st));
        GSX_CUDA(cudaMemsetAsync(fillc.p, 0, (size_t)N * 4, st));
        count_in<<<4 * nsm, 256, 0, st>>>(ids.as<int32_t>(), n_edges, indeg.as<unsigned>());
        scan_blocks<<<(unsigned)nb, 1024, 0, st>>>(indeg.as<unsigned>(), N, off.as<int64_t>(), tot.as<int64_t>());
        scan_totals<<<1, 1024, 0, st>>>(tot.as<int64_t>(), nb);
        add_totals<<<(unsigned)nb, 1024, 0, st>>>(off.as<int64_t>(), N, tot.as<int64_t>());
        fill_in<<<4 * nsm, 256, 0, st>>>(ids.as<int32_t>(), dis.as<float>(), n_edges, R, off.as<int64_t>(),
                                          fillc.as<unsigned>(), src.as<int32_t>(), sd.as<float>());
        GSX_CUDA(cudaGetLastError());
        RevParams Q{};
        Q.x = x.as<float>();
        Q.N = (int)N;
        Q.d = d;
        Q.vec4 = P.vec4;
        Q.R = R;
        Q.ids = ids.as<int32_t>();
        Q.dis = dis.as<float>();
        Q.off = off.as<int64_t>();
        Q.src = src.as<int32_t>();
        Q.sd = sd.as<float>();
        Q.out = fin.as<int32_t>();
        const size_t rev_smem = (size_t)kRevWarps * 4 * R * 4;
        GSX_CUDA(cudaFuncSetAttribute(reverse_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rev_smem));
        reverse_merge<<<8 * nsm, 32 * kRevWarps, rev_smem, st>>>(Q);
        GSX_CUDA(cudaGetLastError());
        std::vector<int32_t> g((size_t)n_edges);
        GSX_CUDA(cudaMemcpyAsync(g.data(), fin.p, (size_t)n_edges * 4, cudaMemcpyDeviceToHost, st));
        GSX_CUDA(cudaStreamSynchronize(st));
        const double t3 = now_s();
        t[2] = t3 - t2;
        // 5. connectivity
        int32_t n_att = 0;
        if ((rc = tree_grow(data, N, d, R, L, ep, g, &n_att))) return rc;
        const double t4 = now_s();
        t[3] = t4 - t3;
        t[4] = t4 - t0;
        auto *gr = new gsx_graph;
        gr->g.N = (int32_t)N;
        gr->g.K = R;
        gr->g.adj.swap(g);
        gr->g.eps.assign(1, ep);
        if ((rc = validate_graph(gr->g))) {
            delete gr;
            return rc;
        }
        if (seconds) {
            for (int i = 0; i < 5; ++i) seconds[i] = t[i];
            seconds[5] = (double)n_att;
            seconds[6] = (double)n_re;
        }
        *out = gr;
        return GSX_OK;
    } GSX_ABI_GUARD("gsx_graph_build_nsg")
}
