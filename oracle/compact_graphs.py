"""Writes the NSG-format twin (K, entry point, then per node: count + ids; glass/graph.hpp:354-379)
of a glass graph without HNSW levels.  Rows padded with -1 take a count instead of the padding, so
the benchmark graphs travel in about half the bytes; the searchers load either file.

    python oracle/compact_graphs.py data/clusters1m.glass [...]
"""

import sys

import numpy as np


def compact(path: str) -> str:
    with open(path, "rb") as f:
        nep = int(np.fromfile(f, np.int32, 1)[0])
        eps = np.fromfile(f, np.int32, nep)
        n, k = (int(x) for x in np.fromfile(f, np.int32, 2))
        adj = np.fromfile(f, np.int32, n * k).reshape(n, k)
        if f.read(1):
            raise ValueError(f"{path} has HNSW levels; the NSG format cannot hold them")
    if nep != 1:
        raise ValueError("the NSG format holds exactly one entry point")
    valid = adj != -1
    counts = np.where(valid.all(1), k, np.argmin(valid, axis=1)).astype(np.int32)
    out = path[: -len(".glass")] + ".nsg"
    with open(out, "wb") as f:
        np.array([k, eps[0]], np.int32).tofile(f)
        rows = np.empty(int(counts.sum()) + n, np.int32)
        pos = 0
        for i in range(n):
            c = counts[i]
            rows[pos] = c
            rows[pos + 1 : pos + 1 + c] = adj[i, :c]
            pos += 1 + c
        rows.tofile(f)
    return out


if __name__ == "__main__":
    for p in sys.argv[1:]:
        print(compact(p))
