"""The restated NSG / SSG build (oracle/nsg_oracle.c) on the CPU: its kNN graph is exact, it agrees
with a direct Python transcription of glass/nsg/nsg.hpp on small integer data, and on the golden
data it gives the graph the reference's own NSG builder gave (nearly the same edges, the same search
quality)."""

import math
import os

import numpy as np
import pytest

from tests.golden import spec
from tests.helpers import recall, write_glass

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


def _exact_knn(x, k):
    x64 = x.astype(np.float64)
    sq = (x64 * x64).sum(1)
    D = sq[:, None] + sq[None, :] - 2 * x64 @ x64.T
    np.fill_diagonal(D, np.inf)
    ids = np.arange(x.shape[0])
    return np.stack([np.lexsort((ids, D[i]))[:k] for i in range(x.shape[0])]).astype(np.int32)


def test_knn_graph_is_exact(oracle):
    from oracle import pyoracle

    x = np.random.default_rng(3).integers(0, 40, size=(700, 12)).astype(np.float32)
    _, _, kn, _ = pyoracle.nsg_build(x, 16, 0, False, knn_k=24)
    np.testing.assert_array_equal(kn, _exact_knn(x, 24))


# --- a direct transcription of nsg.hpp for integer data (every distance exact in any order) ------


def _py_nsg(x, R, L, ssg, K, knng, ep):
    n = x.shape[0]
    L = L or R + 32
    C = R + 100
    thr = np.float32(math.cos(60.0 / 180.0 * math.pi))
    xi = x.astype(np.int64)

    def dist(a, b):
        return float(((xi[a] - xi[b]) ** 2).sum())

    def search(q, adj, width):  # search_on_graph, nsg.hpp:129-158, LinearPool neighbor.hpp:320-433
        pool, cur, vis, full = [], 0, {ep}, []
        d0 = dist(q, ep)
        pool.append([d0, ep, False])
        full.append((d0, ep))
        while cur < len(pool) and cur < L:
            pool[cur][2] = True
            u = pool[cur][1]
            while cur < len(pool) and pool[cur][2]:
                cur += 1
            for j in range(width):
                v = int(adj[u][j])
                if v == -1:
                    break
                if v in vis:
                    continue
                vis.add(v)
                dv = dist(q, v)
                full.append((dv, v))
                if len(pool) == L and dv >= pool[-1][0]:
                    continue
                lo = sum(1 for e in pool if e[0] <= dv)
                pool.insert(lo, [dv, v, False])
                del pool[L:]
                cur = min(cur, lo)
        return vis, full

    def occl(res, p, pd, use_ssg):
        for r, rd in res:
            if p == r:
                return True
            djk = dist(r, p)
            if use_ssg:
                num = np.float32(pd + rd - djk)
                c = (num / np.float32(2.0)) / np.sqrt(np.float32(pd) * np.float32(rd))
                if c > thr:
                    return True
            elif djk < pd:
                return True
        return False

    lists = []
    for q in range(n):  # link + sync_prune, nsg.hpp:160-246
        vis, full = search(q, knng, K)
        for v in knng[q]:
            if v == -1:
                break
            if int(v) not in vis:
                full.append((dist(q, int(v)), int(v)))
        full = sorted(full)[:C]
        start = 1 if full[0][1] == q else 0
        res = [(full[start][1], full[start][0])] if start < len(full) else []
        while res and len(res) < R and start + 1 < len(full):
            start += 1
            d, p = full[start]
            if not occl(res, p, d, ssg):
                res.append((p, d))
        lists.append(res)
    offers = [[] for _ in range(n)]  # reverse links, merged per node
    for q in range(n):
        for v, d in lists[q]:
            offers[v].append((d, q))
    graph = np.full((n, R), -1, np.int32)
    for j in range(n):
        mine = {v for v, _ in lists[j]}
        extra = sorted(o for o in offers[j] if o[1] not in mine)
        if len(lists[j]) + len(extra) <= R:
            row = [v for v, _ in lists[j]] + [v for _, v in extra]
        else:
            union = sorted([(d, v) for v, d in lists[j]] + extra)
            res = [(union[0][1], union[0][0])]
            for d, p in union[1:]:
                if len(res) == R:
                    break
                if not occl(res, p, d, False):
                    res.append((p, d))
            row = [v for v, _ in res]
        graph[j, : len(row)] = row
    deg = (graph >= 0).sum(1)  # tree_grow, nsg.hpp:317-404
    reached = np.zeros(n, bool)
    root, att = ep, 0
    while True:
        queue = [root]
        reached[root] = True
        while queue:
            u = queue.pop(0)
            for v in graph[u]:
                if v < 0:
                    break
                if not reached[v]:
                    reached[v] = True
                    queue.append(int(v))
        if reached.all():
            break
        nid = int(np.argmin(reached))
        _, full = search(nid, graph, R)
        node = next((v for _, v in sorted(full) if deg[v] < R and v != nid), None)
        if node is None:
            node = next(i for i in range(n) if reached[i] and deg[i] < R and i != nid)
        graph[node, deg[node]] = nid
        deg[node] += 1
        root = node
        att += 1
    return graph, att


@pytest.mark.parametrize("ssg", [False, True])
@pytest.mark.parametrize("R,L", [(8, 0), (12, 20)])
def test_matches_python_transcription(oracle, ssg, R, L):
    from oracle import pyoracle

    x = np.random.default_rng(5 + R).integers(0, 16, size=(260, 6)).astype(np.float32)
    g, ep, kn, att = pyoracle.nsg_build(x, R, L, ssg, knn_k=20)
    want, watt = _py_nsg(x, R, L, ssg, 20, kn, ep)
    np.testing.assert_array_equal(g, want)
    assert att == watt


def _connected_from(g, ep):
    seen = np.zeros(g.shape[0], bool)
    seen[ep] = True
    frontier = [ep]
    while frontier:
        nxt = g[frontier].ravel()
        nxt = np.unique(nxt[nxt >= 0])
        nxt = nxt[~seen[nxt]]
        seen[nxt] = True
        frontier = list(nxt)
    return seen.all()


def test_golden_data_matches_reference_builder(oracle, tmp_path):
    """tests/golden/nsg_d100.glass was written by the reference's NSG builder (R 16, L 40, FP32) on
    the same rows: the restated build shares ~98% of its edges and searches as well."""
    from oracle import pyoracle

    x, q = spec.base(), spec.queries()
    g, ep, _, _ = pyoracle.nsg_build(x, 16, 40, False)
    ref = pyoracle.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass")).adjacency()
    inter = union = 0
    for i in range(x.shape[0]):
        a, b = set(ref[i][ref[i] >= 0]), set(g[i][g[i] >= 0])
        inter += len(a & b)
        union += len(a | b)
    assert inter / union > 0.97
    assert (g >= 0).sum(1).max() <= 16 and _connected_from(g, ep)
    for row in g:
        v = row[row >= 0]
        assert len(np.unique(v)) == len(v) and (row[len(v):] == -1).all()
    D = ((q[:, None, :].astype(np.float64) - x[None, :, :]) ** 2).sum(-1)
    gt = np.argsort(D, axis=1, kind="stable")[:, :10]
    path = str(tmp_path / "oracle_nsg_d100.glass")
    write_glass(path, g, [ep])
    for ef in (16, 40):
        r_ref = pyoracle.Searcher(pyoracle.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass")), x, "L2", "FP32")
        r_new = pyoracle.Searcher(pyoracle.Graph(path), x, "L2", "FP32")
        r_ref.set_ef(ef)
        r_new.set_ef(ef)
        a = recall(r_ref.batch_search(q, 10)[0], gt, 10)
        b = recall(r_new.batch_search(q, 10)[0], gt, 10)
        assert b >= a - 0.02, (ef, a, b)
