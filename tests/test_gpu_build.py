"""GPU NSG / SSG graph build (pyglass_gb300/csrc/build_kernel.cu) against the restated build
(oracle/nsg_oracle.c): identical kNN graph, entry point and final graph on integer data (where every
distance is exact in any order); identical final graph on float data given the same kNN graph and
entry point (fp32 distances in one fixed order on both sides); reference-level search quality on
the golden data; and the graph invariants at 100,000 rows."""

import os

import numpy as np
import pytest

from tests.golden import spec
from tests.helpers import recall

pytestmark = pytest.mark.gpu

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


def _build(glass, x, kind, R, L, knn_k=64):
    idx = glass.Index(kind, "L2", "FP32", R, L)
    g = idx.build(x, knn_k=knn_k, keep_knn=True)
    return g, idx


def _adj(glass, g, tmp_path):
    """adjacency and entry point of a Graph, read back through a saved glass file"""
    from oracle import pyoracle

    path = str(tmp_path / "g.glass")
    g.save(path)
    og = pyoracle.Graph(path)
    eps = np.ctypeslib.as_array(og._g.eps, shape=(og._g.nep,)).copy()
    return og.adjacency(), int(eps[0])


def _connected_from(g, ep):
    seen = np.zeros(g.shape[0], bool)
    seen[ep] = True
    frontier = np.array([ep])
    while frontier.size:
        nxt = g[frontier].ravel()
        nxt = np.unique(nxt[nxt >= 0])
        nxt = nxt[~seen[nxt]]
        seen[nxt] = True
        frontier = nxt
    return bool(seen.all())


@pytest.mark.parametrize("kind", ["NSG", "SSG"])
@pytest.mark.parametrize("n,d,R,L", [(3000, 32, 16, 0), (2500, 30, 24, 40), (1200, 7, 8, 0)])
def test_integer_data_matches_oracle(glass, oracle, tmp_path, kind, n, d, R, L):
    from oracle import pyoracle

    x = np.random.default_rng(n + d).integers(0, 16, size=(n, d)).astype(np.float32)
    g, idx = _build(glass, x, kind, R, L)
    adj, ep = _adj(glass, g, tmp_path)
    want, wep, wkn, watt = pyoracle.nsg_build(x, R, L, kind == "SSG")
    np.testing.assert_array_equal(idx.knn_graph, wkn)
    assert ep == wep
    np.testing.assert_array_equal(adj, want)
    assert idx.stages()["attached"] == watt


@pytest.mark.parametrize("n", [2, 3, 65, 150])
def test_small_sets_match_oracle(glass, oracle, tmp_path, n):
    """Fewer rows than candidate slots: every row's kNN list comes from the brute-force pass."""
    from oracle import pyoracle

    x = np.random.default_rng(n).integers(0, 16, size=(n, 16)).astype(np.float32)
    g, idx = _build(glass, x, "NSG", 8, 0)
    adj, ep = _adj(glass, g, tmp_path)
    want, wep, wkn, watt = pyoracle.nsg_build(x, 8, 0, False)
    np.testing.assert_array_equal(idx.knn_graph, wkn)
    assert ep == wep
    np.testing.assert_array_equal(adj, want)


def test_rows_sorted_by_cluster_match_oracle(glass, oracle, tmp_path):
    """Rows stored cluster by cluster put a row's nearest neighbours into one 64-column half of the
    tensor-core tiles, more than its 16-entry candidate list holds: those rows must be found and
    redone by brute force."""
    from oracle import pyoracle

    rng = np.random.default_rng(4)
    centers = rng.integers(0, 200, size=(30, 24))
    x = np.concatenate([np.clip(c + rng.integers(-3, 4, size=(100, 24)), 0, 255) for c in centers]).astype(np.float32)
    g, idx = _build(glass, x, "SSG", 16, 0)
    assert idx.stages()["knn_rows_rechecked"] > 0
    adj, ep = _adj(glass, g, tmp_path)
    want, wep, wkn, watt = pyoracle.nsg_build(x, 16, 0, True)
    np.testing.assert_array_equal(idx.knn_graph, wkn)
    assert ep == wep
    np.testing.assert_array_equal(adj, want)


@pytest.mark.parametrize("kind", ["NSG", "SSG"])
def test_float_data_matches_oracle(glass, oracle, tmp_path, kind):
    from oracle import pyoracle

    x = np.random.default_rng(7).standard_normal((4000, 64)).astype(np.float32)
    g, idx = _build(glass, x, kind, 24, 0)
    adj, ep = _adj(glass, g, tmp_path)
    # the kNN graph is the exact one (fp32 distances, (distance, id) order; fp64 agrees but for
    # near-ties)
    x64 = x.astype(np.float64)
    sq = (x64 * x64).sum(1)
    D = sq[:, None] + sq[None, :] - 2 * x64 @ x64.T
    np.fill_diagonal(D, np.inf)
    rows = np.arange(0, 4000, 7)
    exact = np.stack([np.argsort(D[i], kind="stable")[:64] for i in rows])
    assert np.mean(np.all(idx.knn_graph[rows] == exact, axis=1)) > 0.99
    # the oracle's own kNN graph (same fp32 order) equals the GPU's; link / reverse / connectivity
    # are bit-identical given the same entry point
    want, wep, wkn, watt = pyoracle.nsg_build(x, 24, 0, kind == "SSG", ep=ep)
    np.testing.assert_array_equal(idx.knn_graph, wkn)
    assert wep == ep
    np.testing.assert_array_equal(adj, want)
    assert idx.stages()["attached"] == watt


def test_golden_data_search_quality(glass, tmp_path):
    """On the golden rows the GPU-built NSG (R 16, L 40) searches as well as the reference's own."""
    x, q = spec.base(), spec.queries()
    g, _ = _build(glass, x, "NSG", 16, 40)
    path = str(tmp_path / "gpu_nsg.glass")
    g.save(path)
    D = ((q[:, None, :].astype(np.float64) - x[None, :, :]) ** 2).sum(-1)
    gt = np.argsort(D, axis=1, kind="stable")[:, :10]
    for ef in (16, 40):
        rr = []
        for p in (os.path.join(GOLDEN_DIR, "nsg_d100.glass"), path):
            s = glass.Searcher(glass.Graph(p), x, "L2", "FP32")
            s.set_ef(ef)
            rr.append(recall(s.batch_search(q, 10)[0], gt, 10))
        assert rr[1] >= rr[0] - 0.02, (ef, rr)


def test_build_graph_writes_a_loadable_file(glass, tmp_path):
    x = np.random.default_rng(1).standard_normal((2000, 16)).astype(np.float32)
    path = str(tmp_path / "b.glass")
    secs = glass.build_graph("SSG", x, path, "L2", "FP32", 12, 0)
    assert secs > 0
    n, k, nep, h = glass.Graph(path).info()
    assert (n, k, nep, h) == (2000, 12, 1, False)
    with pytest.raises(RuntimeError, match="not built on the GPU"):
        glass.Index("HNSW", "L2", "FP32", 16, 0)
    with pytest.raises(RuntimeError, match="FP32"):
        glass.Index("NSG", "L2", "SQ8U", 16, 0)
    with pytest.raises(RuntimeError, match="d <= 128"):
        glass.Index("NSG", "L2").build(np.zeros((100, 200), np.float32))


def test_100k_rows_invariants(glass, tmp_path):
    # rows near a 12-dimensional subspace: a single-entry NSG navigates them well (on a few
    # well-separated clusters it does not, whatever builds it)
    rng = np.random.default_rng(2)
    w = rng.standard_normal((12, 48)).astype(np.float32)
    x = rng.standard_normal((100_000, 12)).astype(np.float32) @ w + 0.05 * rng.standard_normal((100_000, 48)).astype(np.float32)
    q = rng.standard_normal((200, 12)).astype(np.float32) @ w + 0.05 * rng.standard_normal((200, 48)).astype(np.float32)
    g, idx = _build(glass, x, "NSG", 32, 0)
    st = idx.stages()
    adj, ep = _adj(glass, g, tmp_path)
    deg = (adj >= 0).sum(1)
    assert deg.max() <= 32 and deg.min() >= 1
    for row in adj[::997]:
        v = row[row >= 0]
        assert len(np.unique(v)) == len(v) and (row[len(v):] == -1).all()
    assert _connected_from(adj, ep)
    s = glass.Searcher(g, x, "L2", "FP32")
    s.set_ef(64)
    ids, _ = s.batch_search(q, 10)
    q64, x64 = q.astype(np.float64), x.astype(np.float64)
    D = (q64 * q64).sum(1)[:, None] + (x64 * x64).sum(1)[None, :] - 2 * q64 @ x64.T
    gt = np.argsort(D, axis=1)[:, :10]
    assert recall(ids, gt, 10) > 0.8
    assert st["total_s"] < 60
