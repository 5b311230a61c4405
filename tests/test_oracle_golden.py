"""The CPU oracle against the golden outputs of the compiled reference (bit-exact)."""

import hashlib
import os

import numpy as np
import pytest

from tests.golden import spec

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("quant,metric", spec.QUANTS)
def test_codes_params_distances(oracle, golden, quant, metric):
    base, q = spec.base(), spec.queries()[: spec.NQ_DIST]
    qz = oracle.Quant(quant, metric, base)
    assert hashlib.sha256(qz.codes.tobytes()).digest() == golden[f"codes_sha/{quant}/{metric}"].tobytes()
    np.testing.assert_array_equal(qz.params, golden[f"params/{quant}/{metric}"])
    d = qz.distances(q, golden["dist_ids"])
    if (quant, metric) in spec.FLOAT_TOLERANT:
        np.testing.assert_allclose(d, golden[f"dist/{quant}/{metric}"], rtol=spec.RTOL, atol=0)
    else:
        np.testing.assert_array_equal(d, golden[f"dist/{quant}/{metric}"])  # bit-exact, floats included


@pytest.mark.parametrize("case", list(spec.search_cases()), ids=spec.case_key)
def test_search(oracle, golden, case):
    g, quant, metric, refine, ef, k, mode = case
    graph = oracle.Graph(os.path.join(GOLDEN_DIR, f"{g}.glass"))
    s = oracle.Searcher(graph, spec.base(), metric, quant, refine)
    s.set_ef(ef)
    q = spec.queries()[: spec.NQ_SEARCH]
    key = spec.case_key(case)
    if mode == "batch":
        ids, dis = s.batch_search(q, k)
        assert s.get_last_search_dist_cmps() == golden[f"cmps/{key}"][0]
    else:
        res = [s.search(q[i], k) for i in range(q.shape[0])]
        ids, dis = np.stack([r[0] for r in res]), np.stack([r[1] for r in res])
    np.testing.assert_array_equal(ids, golden[f"ids/{key}"])
    if (quant, metric) in spec.FLOAT_TOLERANT:
        np.testing.assert_allclose(dis, golden[f"dis/{key}"], rtol=spec.RTOL, atol=0)
    else:
        np.testing.assert_array_equal(dis, golden[f"dis/{key}"])


def test_nsg_reader_equals_glass_reader(oracle, tmp_path):
    """The oracle's NSG-format reader (Graph::load_nsg, glass/graph.hpp:224-246) gives the graph the
    glass reader gives for the same rows: the compact twin oracle/compact_graphs.py writes."""
    import shutil

    from oracle import compact_graphs

    src = tmp_path / "g.glass"
    shutil.copy(os.path.join(GOLDEN_DIR, "nsg_d100.glass"), src)
    twin = compact_graphs.compact(str(src))
    a, b = oracle.Graph(str(src)), oracle.Graph(twin, "nsg")
    assert (a.N, a.K) == (b.N, b.K)
    np.testing.assert_array_equal(a.adjacency(), b.adjacency())
    assert a._g.eps[0] == b._g.eps[0]
    with pytest.raises(ValueError):
        oracle.Graph(twin, "diskann")
