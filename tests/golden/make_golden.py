"""Generates the golden fixtures of the parity suite from the UNMODIFIED reference.

Needs the reference checkout (oracle/_ref is compiled from it by oracle/Makefile).  Writes:
  tests/golden/{hnsw,nsg}_d100.glass  graphs built by the reference's HNSW and NSG builders
  tests/golden/golden.npz              reference outputs: codes digests, calibrator parameters,
                                       query->row distances and search results (ids, dis, cmps)
The inputs are regenerated from seeds (pyglass_gb300.datasets, identical bytes on x86 and
aarch64), so only graphs and outputs are stored.

    python tests/golden/make_golden.py [--rebuild-graphs]
"""

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from tests.golden import spec  # noqa: E402


def main():
    pyoracle.build(ref=True)
    R = pyoracle.RefGlass
    base0, queries = spec.base(), spec.queries()
    # the reference's FP16 encoder reads past the last row when d is not a multiple of 16
    # (fp32_to_fp16 over the rounded-up row length): give it a zero row there, which is what the
    # oracle and the GPU encode, so that the fixtures do not depend on memory past the array
    bz = np.zeros((base0.shape[0] + 1, base0.shape[1]), np.float32)
    bz[:-1] = base0
    base = bz[:-1]
    for name, (itype, Rdeg, L) in spec.GRAPHS.items():
        path = os.path.join(HERE, f"{name}.glass")
        # the builders are multi-threaded and not deterministic: keep the committed graphs, so that
        # adding cases does not change the existing ones
        if not os.path.exists(path) or "--rebuild-graphs" in sys.argv:
            R.build_graph(itype, base, "L2", "FP32", Rdeg, L, path)
    out = {}
    rng = np.random.default_rng(5)
    ids = rng.integers(0, base.shape[0], size=(spec.NQ_DIST, 40)).astype(np.int32)
    out["dist_ids"] = ids
    for quant, metric in spec.QUANTS:
        codes, params = R.encode(quant, metric, base)
        out[f"codes_sha/{quant}/{metric}"] = np.frombuffer(hashlib.sha256(codes.tobytes()).digest(), np.uint8)
        out[f"params/{quant}/{metric}"] = params
        d, _ = R.query_distances(quant, metric, base, queries[: spec.NQ_DIST], ids)
        out[f"dist/{quant}/{metric}"] = d
        if quant in ("SQ8U", "SQ4U", "SQ2U", "SQ8", "SQ4UA", "SQ1"):
            d, _ = R.query_distances("FP32", metric, base, queries[: spec.NQ_DIST], ids)
            out[f"dist/FP32/{metric}"] = d
    for case in spec.search_cases():
        g, quant, metric, refine, ef, k, mode = case
        s = R.Searcher(os.path.join(HERE, f"{g}.glass"), base, metric, quant, refine)
        s.set_ef(ef)
        q = queries[: spec.NQ_SEARCH]
        if mode == "batch":
            ids_, dis_ = s.batch_search(q, k)
            cm = np.array([s.get_last_search_dist_cmps()])
        else:
            res = [s.search(q[i], k) for i in range(q.shape[0])]
            ids_ = np.stack([r[0] for r in res])
            dis_ = np.stack([r[1] for r in res])
            cm = np.array([-1.0])
        key = spec.case_key(case)
        out[f"ids/{key}"] = ids_
        out[f"dis/{key}"] = dis_
        out[f"cmps/{key}"] = cm
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
