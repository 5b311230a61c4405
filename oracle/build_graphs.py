"""Builds the benchmark graphs with the reference's own CPU builders (oracle/_ref).

Graph construction is not part of the GPU path: the reference's HNSW/NSG builders write the
glass graph file (glass/graph.hpp:106-119) that both the GPU searcher and the CPU oracle read.
Output: data/<workload>.glass plus data/<workload>.json (data checksums, build time).  Run where
the reference checkout exists (GLASS_REFERENCE_DIR); the files travel with the repository snapshot.
``--gt`` instead writes data/<workload>_gt.npy: the exact top-100 ids of the workload's queries by
brute force on the CPU (used by the benchmark's reference arm for its recall).

    python oracle/build_graphs.py clusters1m [gauss10k ...]
    python oracle/build_graphs.py --gt clusters1m
"""

import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from pyglass_gb300 import datasets  # noqa: E402


def ground_truth(name: str, k: int = 100, chunk: int = 256) -> None:
    """Exact k nearest base rows of every query by squared L2 (ties by id), in float64 from a float32
    GEMM shortlist of 4k candidates per query re-ranked exactly."""
    import numpy as np

    w = datasets.WORKLOADS[name]
    base, queries = w["base"](), w["queries"]()
    bsq = (base.astype(np.float64) ** 2).sum(1).astype(np.float32)
    out = np.empty((queries.shape[0], k), np.int32)
    t = time.time()
    for s in range(0, queries.shape[0], chunk):
        q = queries[s:s + chunk]
        d = bsq[None, :] - 2.0 * (q @ base.T)
        cand = np.argpartition(d, 4 * k, axis=1)[:, : 4 * k]
        for i in range(q.shape[0]):
            c = cand[i]
            ex = ((base[c].astype(np.float64) - q[i].astype(np.float64)) ** 2).sum(1)
            out[s + i] = c[np.lexsort((c, ex))[:k]]
    np.save(os.path.join(ROOT, "data", f"{name}_gt.npy"), out)
    mpath = os.path.join(ROOT, "data", f"{name}.json")
    meta = json.load(open(mpath)) if os.path.exists(mpath) else {}
    meta.update(gt_base_checksum=datasets.checksum(base), gt_query_checksum=datasets.checksum(queries), gt_k=k,
                gt_seconds=time.time() - t)
    with open(mpath, "w") as f:
        json.dump(meta, f, indent=1)
    print(json.dumps({"ground_truth": name, "k": k, "seconds": meta["gt_seconds"]}))


def main(names):
    pyoracle.build(ref=True)
    os.makedirs(os.path.join(ROOT, "data"), exist_ok=True)
    for name in names:
        w = datasets.WORKLOADS[name]
        base = w["base"]()
        queries = w["queries"]()
        itype, R, L, bq = w["index"]
        path = os.path.join(ROOT, "data", f"{name}.glass")
        t = time.time()
        pyoracle.RefGlass.build_graph(itype, base, w["metric"], bq, R, L, path)
        meta = dict(workload=name, desc=w["desc"], index=[itype, R, L, bq], metric=w["metric"],
                    base_checksum=datasets.checksum(base), query_checksum=datasets.checksum(queries),
                    build_seconds=time.time() - t)
        with open(os.path.join(ROOT, "data", f"{name}.json"), "w") as f:
            json.dump(meta, f, indent=1)
        print(json.dumps(meta))


if __name__ == "__main__":
    args = sys.argv[1:]
    if args and args[0] == "--gt":
        for n in args[1:]:
            ground_truth(n)
    else:
        main(args or ["gauss10k", "clusters1m"])
