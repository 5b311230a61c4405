/* TEST INFRASTRUCTURE ONLY: a CPU restatement of the NSG / SSG graph build, used by the tests as
 * the oracle of the GPU build (pyglass_gb300/csrc/build_kernel.cu); never part of the product.
 *
 * It follows the reference's builder glass/nsg/nsg.hpp stage by stage:
 *   - kNN graph: exact by brute force ((distance, id) order over the fp32 distance below, the row
 *     itself left out) where the reference runs NN-Descent (nsg/nndescent.hpp);
 *   - entry point: the row nearest to the centroid (nsg.hpp:106-127);
 *   - link: search_on_graph over the kNN graph from the entry point with a LinearPool of L entries
 *     (nsg.hpp:129-158, neighbor.hpp:320-433), sync_prune over the C = R + 100 nearest evaluated
 *     rows (nsg.hpp:180-246) with the NSG or the SSG rule;
 *   - reverse links: nsg.hpp:248-315 merged per node in one step (the node's list and all of its
 *     offers, nearest first; pruned with the NSG rule when more than R), as the GPU build does,
 *     instead of the reference's lock-protected insertions in thread order;
 *   - connectivity: tree_grow / bfs / attach_unlinked (nsg.hpp:317-404), with the first reached
 *     node by id where the reference draws a random one.
 * Parity against the reference's own builder is unpinned: its NN-Descent and its reverse-link pass
 * depend on random numbers and thread timing.  Distances are fp32 squared L2 with four fmaf chains
 * over j & 3 summed (c0 + c1) + (c2 + c3), the GPU build's order, so both give identical graphs. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "glass_oracle.h"

static float l2f(const float *a, const float *b, int d) {
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int j = 0; j < d; ++j) {
        const float t = a[j] - b[j];
        c[j & 3] = fmaf(t, t, c[j & 3]);
    }
    return (c[0] + c[1]) + (c[2] + c[3]);
}

typedef struct {
    double d;
    int32_t id;
} dpair;

typedef struct {
    float d;
    int32_t id;
} fpair;

static int dpair_cmp(const void *a, const void *b) {
    const dpair *x = (const dpair *)a, *y = (const dpair *)b;
    if (x->d != y->d) return x->d < y->d ? -1 : 1;
    return x->id < y->id ? -1 : (x->id > y->id);
}

static int fpair_cmp(const void *a, const void *b) {
    const fpair *x = (const fpair *)a, *y = (const fpair *)b;
    if (x->d != y->d) return x->d < y->d ? -1 : 1;
    return x->id < y->id ? -1 : (x->id > y->id);
}

/* (distance, id) order of Neighbor (neighbor.hpp:205-207) */
static int key_less(float da, int32_t ia, float db, int32_t ib) { return da < db || (da == db && ia < ib); }

/* ---- LinearPool<float> (neighbor.hpp:320-433) ------------------------------------------------ */
typedef struct {
    int32_t *id;
    float *d;
    int size, cur, cap;
} lpool;

static void lp_insert(lpool *p, int32_t u, float dist) {
    if (p->size == p->cap && dist >= p->d[p->size - 1]) return;
    int lo = 0, hi = p->size;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (p->d[mid] > dist) hi = mid;
        else lo = mid + 1;
    }
    memmove(p->id + lo + 1, p->id + lo, sizeof(int32_t) * (size_t)(p->size - lo));
    memmove(p->d + lo + 1, p->d + lo, sizeof(float) * (size_t)(p->size - lo));
    p->id[lo] = u;
    p->d[lo] = dist;
    if (p->size < p->cap) p->size++;
    if (lo < p->cur) p->cur = lo;
}

static int32_t lp_pop(lpool *p) {
    p->id[p->cur] |= (int32_t)0x80000000u;
    int pre = p->cur;
    while (p->cur < p->size && (p->id[p->cur] & (int32_t)0x80000000u)) p->cur++;
    return p->id[pre] & 0x7fffffff;
}

/* the C smallest (distance, id) pairs of everything offered */
typedef struct {
    int32_t *id;
    float *d;
    int n, cap;
} topc;

static void tc_insert(topc *t, int32_t u, float dist) {
    if (t->n == t->cap && !key_less(dist, u, t->d[t->n - 1], t->id[t->n - 1])) return;
    int pos = 0;
    while (pos < t->n && key_less(t->d[pos], t->id[pos], dist, u)) ++pos;
    int move = t->n - pos;
    if (t->n == t->cap) --move;
    if (move > 0) {
        memmove(t->id + pos + 1, t->id + pos, sizeof(int32_t) * (size_t)move);
        memmove(t->d + pos + 1, t->d + pos, sizeof(float) * (size_t)move);
    }
    t->id[pos] = u;
    t->d[pos] = dist;
    if (t->n < t->cap) t->n++;
}

/* occlusion test of nsg.hpp:208-231 */
static int occluded(const float *x, int d, const int32_t *rid, const float *rd, int nres, int32_t p, float pd, int ssg,
                    float threshold) {
    for (int t = 0; t < nres; ++t) {
        if (p == rid[t]) return 1;
        const float djk = l2f(x + (size_t)rid[t] * d, x + (size_t)p * d, d);
        if (ssg) {
            const float num = (pd + rd[t]) - djk;
            const float cosij = (num / 2.0f) / sqrtf(pd * rd[t]);
            if (cosij > threshold) return 1;
        } else if (djk < pd) {
            return 1;
        }
    }
    return 0;
}

int go_nsg_build(const float *x, int64_t N, int d, int R, int L, int ssg, int knn_k, const int32_t *knng_in,
                 int32_t ep_in, int32_t *knng_out, int32_t *graph_out, int32_t *ep_out, int32_t *n_attached,
                 int32_t *link_out) {
    if (N < 2 || d <= 0 || R <= 0 || knn_k <= 0) return 1;
    if (L == 0) L = R + 32;
    const int C = R + 100;
    const int K = (int)(knn_k < N - 1 ? knn_k : N - 1);
    const float threshold = (float)cos(60.0 / 180.0 * 3.14159265358979323846264);
    /* kNN graph */
    int32_t *knng = knng_out;
    if (knng_in) {
        memcpy(knng, knng_in, sizeof(int32_t) * (size_t)N * K);
    } else {
#pragma omp parallel
        {
            dpair *all = (dpair *)malloc(sizeof(dpair) * (size_t)N);
#pragma omp for schedule(dynamic, 16)
            for (int64_t q = 0; q < N; ++q) {
                int64_t n = 0;
                for (int64_t r = 0; r < N; ++r) {
                    if (r == q) continue;
                    all[n].d = (double)l2f(x + r * d, x + q * d, d);
                    all[n].id = (int32_t)r;
                    ++n;
                }
                qsort(all, (size_t)n, sizeof(dpair), dpair_cmp);
                for (int j = 0; j < K; ++j) knng[q * K + j] = all[j].id;
            }
            free(all);
        }
    }
    /* entry point */
    int32_t ep = ep_in;
    if (ep < 0) {
        double *sum = (double *)calloc((size_t)d, sizeof(double));
        float *c = (float *)malloc(sizeof(float) * (size_t)d);
        for (int64_t r = 0; r < N; ++r)
            for (int j = 0; j < d; ++j) sum[j] += (double)x[r * d + j];
        for (int j = 0; j < d; ++j) c[j] = (float)(sum[j] / (double)N);
        float best = INFINITY;
        ep = 0;
        for (int64_t r = 0; r < N; ++r) {
            const float dd = l2f(c, x + r * d, d);
            if (dd < best) {
                best = dd;
                ep = (int32_t)r;
            }
        }
        free(sum);
        free(c);
    }
    *ep_out = ep;
    /* link */
    int32_t *lid = (int32_t *)malloc(sizeof(int32_t) * (size_t)N * R);
    float *ldis = (float *)malloc(sizeof(float) * (size_t)N * R);
#pragma omp parallel
    {
        uint8_t *vis = (uint8_t *)malloc((size_t)N);
        int32_t *stamp = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
        for (int64_t i = 0; i < N; ++i) stamp[i] = -1;
        (void)vis;
        lpool p;
        p.id = (int32_t *)malloc(sizeof(int32_t) * (size_t)(L + 1));
        p.d = (float *)malloc(sizeof(float) * (size_t)(L + 1));
        p.cap = L;
        topc t;
        t.id = (int32_t *)malloc(sizeof(int32_t) * (size_t)(C + 1));
        t.d = (float *)malloc(sizeof(float) * (size_t)(C + 1));
        t.cap = C;
        int32_t *rid = (int32_t *)malloc(sizeof(int32_t) * (size_t)R);
        float *rd = (float *)malloc(sizeof(float) * (size_t)R);
#pragma omp for schedule(dynamic, 64)
        for (int64_t q = 0; q < N; ++q) {
            const float *xq = x + q * d;
            p.size = p.cur = 0;
            t.n = 0;
            /* search_on_graph (nsg.hpp:129-158) */
            const float d0 = l2f(xq, x + (size_t)ep * d, d);
            lp_insert(&p, ep, d0);
            stamp[ep] = (int32_t)q;
            tc_insert(&t, ep, d0);
            while (p.cur < p.size && p.cur < L) {
                const int32_t u = lp_pop(&p);
                for (int j = 0; j < K; ++j) {
                    const int32_t v = knng[(size_t)u * K + j];
                    if (v == -1) break;
                    if (stamp[v] == (int32_t)q) continue;
                    stamp[v] = (int32_t)q;
                    const float dv = l2f(xq, x + (size_t)v * d, d);
                    lp_insert(&p, v, dv);
                    tc_insert(&t, v, dv);
                }
            }
            /* sync_prune (nsg.hpp:180-246) */
            for (int j = 0; j < K; ++j) {
                const int32_t v = knng[q * K + j];
                if (v == -1) break;
                if (stamp[v] == (int32_t)q) continue;
                tc_insert(&t, v, l2f(xq, x + (size_t)v * d, d));
            }
            int nres = 0, start = 0;
            if (t.n > 0 && t.id[0] == (int32_t)q) start = 1;
            if (start < t.n) {
                rid[0] = t.id[start];
                rd[0] = t.d[start];
                nres = 1;
                while (nres < R && ++start < t.n) {
                    if (!occluded(x, d, rid, rd, nres, t.id[start], t.d[start], ssg, threshold)) {
                        rid[nres] = t.id[start];
                        rd[nres] = t.d[start];
                        ++nres;
                    }
                }
            }
            for (int i = 0; i < R; ++i) {
                lid[q * R + i] = i < nres ? rid[i] : -1;
                ldis[q * R + i] = i < nres ? rd[i] : 0.0f;
            }
        }
        free(vis);
        free(stamp);
        free(p.id);
        free(p.d);
        free(t.id);
        free(t.d);
        free(rid);
        free(rd);
    }
    /* reverse links, merged per node */
    int64_t *off = (int64_t *)calloc((size_t)N + 1, sizeof(int64_t));
    for (int64_t e = 0; e < N * R; ++e)
        if (lid[e] >= 0) off[lid[e] + 1]++;
    for (int64_t i = 0; i < N; ++i) off[i + 1] += off[i];
    int64_t *fill = (int64_t *)calloc((size_t)N, sizeof(int64_t));
    fpair *offers = (fpair *)malloc(sizeof(fpair) * (size_t)(off[N] > 0 ? off[N] : 1));
    for (int64_t e = 0; e < N * R; ++e) {
        const int32_t v = lid[e];
        if (v < 0) continue;
        offers[off[v] + fill[v]].id = (int32_t)(e / R);
        offers[off[v] + fill[v]].d = ldis[e];
        fill[v]++;
    }
#pragma omp parallel
    {
        fpair *u = (fpair *)malloc(sizeof(fpair) * (size_t)(R + N));
        int32_t *rid = (int32_t *)malloc(sizeof(int32_t) * (size_t)R);
        float *rd = (float *)malloc(sizeof(float) * (size_t)R);
#pragma omp for schedule(dynamic, 64)
        for (int64_t j = 0; j < N; ++j) {
            int nout = 0;
            while (nout < R && lid[j * R + nout] >= 0) ++nout;
            int nin = 0;
            for (int64_t e = off[j]; e < off[j + 1]; ++e) {
                int dup = 0;
                for (int t2 = 0; t2 < nout; ++t2) dup |= lid[j * R + t2] == offers[e].id;
                if (!dup) u[nout + nin++] = offers[e];
            }
            int nres = 0;
            if (nout + nin <= R) {
                for (int i = 0; i < nout; ++i) rid[nres++] = lid[j * R + i];
                qsort(u + nout, (size_t)nin, sizeof(fpair), fpair_cmp);
                for (int i = 0; i < nin; ++i) rid[nres++] = u[nout + i].id;
            } else {
                for (int i = 0; i < nout; ++i) {
                    u[i].id = lid[j * R + i];
                    u[i].d = ldis[j * R + i];
                }
                qsort(u, (size_t)(nout + nin), sizeof(fpair), fpair_cmp);
                for (int i = 0; i < nout + nin && nres < R; ++i) {
                    if (nres == 0 || !occluded(x, d, rid, rd, nres, u[i].id, u[i].d, 0, threshold)) {
                        rid[nres] = u[i].id;
                        rd[nres] = u[i].d;
                        ++nres;
                    }
                }
            }
            for (int i = 0; i < R; ++i) graph_out[j * R + i] = i < nres ? rid[i] : -1;
        }
        free(u);
        free(rid);
        free(rd);
    }
    free(off);
    free(fill);
    free(offers);
    if (link_out) memcpy(link_out, lid, sizeof(int32_t) * (size_t)N * R);
    free(lid);
    free(ldis);
    /* connectivity (nsg.hpp:317-404) */
    int32_t *deg = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    for (int64_t i = 0; i < N; ++i) {
        int c = 0;
        while (c < R && graph_out[i * R + c] >= 0) ++c;
        deg[i] = c;
    }
    uint8_t *vis = (uint8_t *)calloc((size_t)N, 1);
    uint8_t *seen = (uint8_t *)malloc((size_t)N);
    int32_t *qu = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    fpair *full = (fpair *)malloc(sizeof(fpair) * (size_t)N);
    lpool p;
    p.id = (int32_t *)malloc(sizeof(int32_t) * (size_t)(L + 1));
    p.d = (float *)malloc(sizeof(float) * (size_t)(L + 1));
    p.cap = L;
    int64_t cnt = 0, scan = 0;
    int32_t root = ep, att = 0;
    int rc = 0;
    while (1) {
        int64_t h = 0, tl = 0;
        qu[tl++] = root;
        if (!vis[root]) {
            vis[root] = 1;
            ++cnt;
        }
        while (h < tl) {
            const int32_t uu = qu[h++];
            for (int i = 0; i < R; ++i) {
                const int32_t v = graph_out[(size_t)uu * R + i];
                if (v < 0) break;
                if (vis[v]) continue;
                vis[v] = 1;
                ++cnt;
                qu[tl++] = v;
            }
        }
        if (cnt >= N) break;
        while (scan < N && vis[scan]) ++scan;
        const int32_t id = (int32_t)scan;
        memset(seen, 0, (size_t)N);
        p.size = p.cur = 0;
        int64_t nf = 0;
        const float *xq = x + (size_t)id * d;
        const float d0 = l2f(xq, x + (size_t)ep * d, d);
        lp_insert(&p, ep, d0);
        seen[ep] = 1;
        full[nf].id = ep;
        full[nf++].d = d0;
        while (p.cur < p.size && p.cur < L) {
            const int32_t uu = lp_pop(&p);
            for (int i = 0; i < R; ++i) {
                const int32_t v = graph_out[(size_t)uu * R + i];
                if (v < 0) break;
                if (seen[v]) continue;
                seen[v] = 1;
                const float dv = l2f(xq, x + (size_t)v * d, d);
                lp_insert(&p, v, dv);
                full[nf].id = v;
                full[nf++].d = dv;
            }
        }
        qsort(full, (size_t)nf, sizeof(fpair), fpair_cmp);
        int32_t node = -1;
        for (int64_t i = 0; i < nf; ++i)
            if (deg[full[i].id] < R && full[i].id != id) {
                node = full[i].id;
                break;
            }
        if (node < 0) {
            for (int64_t i = 0; i < N; ++i)
                if (vis[i] && deg[i] < R && i != id) {
                    node = (int32_t)i;
                    break;
                }
        }
        if (node < 0) {
            rc = 2;
            break;
        }
        graph_out[(size_t)node * R + deg[node]] = id;
        deg[node]++;
        root = node;
        ++att;
    }
    *n_attached = att;
    free(deg);
    free(vis);
    free(seen);
    free(qu);
    free(full);
    free(p.id);
    free(p.d);
    return rc;
}
