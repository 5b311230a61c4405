"""Builds the benchmark graphs with the reference's own CPU builders (oracle/_ref).

Graph construction is not part of the GPU path: the reference's HNSW/NSG builders write the
glass graph file (glass/graph.hpp:106-119) that both the GPU searcher and the CPU oracle read.
Output: data/<workload>.glass plus data/<workload>.json (data checksums, build time).  Run here,
where the reference checkout exists; the files travel with the repository snapshot.

    python oracle/build_graphs.py clusters1m [gauss10k ...]
"""

import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from pyglass_gb300 import datasets  # noqa: E402


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
    main(sys.argv[1:] or ["gauss10k", "clusters1m"])
