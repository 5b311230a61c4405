"""Small helpers shared by the tests (graph files written from numpy, recall)."""

import numpy as np


def write_glass(path, adj, eps, hnsw=None):
    """Writes a glass-format graph (glass/graph.hpp:240-253); hnsw = (K, ep, per-node lists)."""
    adj = np.ascontiguousarray(adj, dtype=np.int32)
    with open(path, "wb") as f:
        np.array([len(eps)], np.int32).tofile(f)
        np.asarray(eps, np.int32).tofile(f)
        np.array(adj.shape, np.int32).tofile(f)
        adj.tofile(f)
        if hnsw is not None:
            hk, ep, lists = hnsw
            np.array([adj.shape[0], hk, ep], np.int32).tofile(f)
            for lst in lists:
                lst = np.asarray(lst, np.int32)
                np.array([lst.size], np.int32).tofile(f)
                lst.tofile(f)


def knn_graph(x, K, rng, drop=0.3, dup=0.05):
    """A fixed-degree graph from exact neighbours with random truncation (-1 padding) and a few
    repeated ids inside rows, to exercise the row handling of the searchers."""
    n = x.shape[0]
    sq = (x * x).sum(1)
    d = sq[:, None] + sq[None, :] - 2 * x @ x.T
    np.fill_diagonal(d, np.inf)
    nn = np.argsort(d, axis=1)[:, :K].astype(np.int32)
    adj = nn.copy()
    for i in range(n):
        if rng.random() < drop:
            adj[i, rng.integers(1, K):] = -1
        if rng.random() < dup:
            a, b = rng.integers(0, K, size=2)
            if adj[i, a] != -1 and adj[i, b] != -1:
                adj[i, b] = adj[i, a]
    return adj


def recall(ids, gt, k):
    return float(np.mean([len(np.intersect1d(ids[i, :k], gt[i, :k])) for i in range(ids.shape[0])])) / k


def oracle_graph(oracle, glass, path, fmt):
    """The oracle reads glass and NSG files itself; other formats are converted through the library's
    loader."""
    if fmt in ("glass", "nsg"):
        return oracle.Graph(path, fmt)
    import os
    import tempfile

    tmp = os.path.join(tempfile.mkdtemp(), "g.glass")
    glass.Graph(path, fmt).save(tmp)
    return oracle.Graph(tmp)
