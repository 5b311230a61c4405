"""Live comparison of the oracle with the compiled reference on fresh inputs (runs only where the
reference checkout exists, i.e. where oracle/_ref could be built)."""

import os

import numpy as np
import pytest

from pyglass_gb300 import datasets


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        try:
            oracle.build(ref=True)
        except Exception:
            pass
    if not oracle.ref_available():
        pytest.skip("reference checkout not available on this host")
    return oracle.RefGlass


@pytest.mark.parametrize("quant", ["SQ8U", "SQ4U", "E5M2", "FP32", "FP16", "BF16", "SQ2U", "SQ8", "SQ4UA", "SQ1"])
@pytest.mark.parametrize("metric", ["L2", "IP"])
def test_encode_and_distances(oracle, ref, quant, metric):
    base = datasets.cluster_mixture(2000, d=72, n_clusters=16, seed=21)
    q = datasets.cluster_mixture(8, d=72, n_clusters=16, seed=21, stream=1)
    codes, params = ref.encode(quant, metric, base)
    qz = oracle.Quant(quant, metric, base)
    # FP16 with d % 16 != 0: the reference fills a row's padding from the floats after the row, and for
    # the last row reads past the end of the data array (undefined contents); that row is left out
    last = base.shape[0] - 1 if quant == "FP16" else base.shape[0]
    np.testing.assert_array_equal(codes[:last], qz.codes[:last])
    np.testing.assert_array_equal(params, qz.params)
    ids = np.random.default_rng(1).integers(0, last, size=(8, 50)).astype(np.int32)
    rd, rq = ref.query_distances(quant, metric, base, q, ids)
    if (quant, metric) == ("SQ8", "L2"):
        # a float kernel the reference's -Ofast build rounds differently in this stand-alone copy than
        # in its search loop (which the oracle follows): floating-point tolerance
        np.testing.assert_allclose(rd, qz.distances(q, ids), rtol=1e-5, atol=0)
    else:
        np.testing.assert_array_equal(rd, qz.distances(q, ids))
    oq = qz.encode_queries(q)
    if quant == "SQ8":
        oq = oq[:, : 4 * qz.dalign]  # the oracle appends the calibrator arrays to the fp32 query
    np.testing.assert_array_equal(rq[:, : oq.shape[1]], oq)


def test_search_nsg_clusters(oracle, ref, tmp_path):
    base = datasets.cluster_mixture(4000, d=32, n_clusters=32, seed=22)
    q = datasets.cluster_mixture(80, d=32, n_clusters=32, seed=22, stream=1)
    path = str(tmp_path / "g.glass")
    ref.build_graph("NSG", base, "L2", "SQ8U", 24, 40, path)
    g = oracle.Graph(path)
    cases = [("SQ4U", "FP32", "L2"), ("SQ8U", "", "L2"), ("FP32", "", "L2"), ("FP16", "", "L2"), ("BF16", "", "IP"),
             ("SQ2U", "FP32", "L2"), ("SQ4UA", "FP32", "L2"), ("SQ1", "FP32", "IP"), ("SQ4U", "FP16", "L2")]
    for quant, refine, metric in cases:
        rs = ref.Searcher(path, base, metric, quant, refine)
        os_ = oracle.Searcher(g, base, metric, quant, refine)
        for ef, k in [(10, 10), (32, 5), (64, 10)]:
            rs.set_ef(ef)
            os_.set_ef(ef)
            ri, rdis = rs.batch_search(q, k)
            oi, odis = os_.batch_search(q, k)
            np.testing.assert_array_equal(ri, oi)
            np.testing.assert_array_equal(rdis, odis)
            assert rs.get_last_search_dist_cmps() == os_.get_last_search_dist_cmps()
