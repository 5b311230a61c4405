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


@pytest.mark.parametrize("fmt", ["glass", "nsg", "diskann", "hnswlib"])
def test_graph_loaders_match_the_reference(ref, glass, tmp_path, fmt):
    """Each graph format read by the library's loader (gsx_graph_load) gives the entry points and
    the -1 padded adjacency that the reference's Graph<int>::load gives for the same file."""
    import ctypes as C

    from tests.helpers import write_glass
    from tests.test_abi import _adj, _info, _load, _write_hnswlib

    rng = np.random.default_rng(17)
    N, K = 300, 12
    rows = [list(rng.choice(N, size=int(rng.integers(0, K + 1)), replace=False).astype(int)) for _ in range(N)]
    rows[5] = list(rng.choice(N, size=K, replace=False).astype(int))  # a full row
    ep = 42
    p = str(tmp_path / f"g.{fmt}")
    if fmt == "glass":
        adj = np.full((N, K), -1, np.int32)
        for i, r in enumerate(rows):
            adj[i, : len(r)] = r
        write_glass(p, adj, [ep, 7])
    elif fmt in ("nsg", "diskann"):
        body = b"".join(np.array([len(r)] + r, np.int32).tobytes() for r in rows)
        with open(p, "wb") as f:
            if fmt == "nsg":  # glass/graph.hpp:219-245
                np.array([K, ep], np.int32).tofile(f)
            else:  # glass/graph.hpp:155-182
                np.array([24 + len(body)], np.uint64).tofile(f)
                np.array([K, ep], np.int32).tofile(f)
                np.array([0], np.uint64).tofile(f)
            f.write(body)
    else:
        _write_hnswlib(p, rows, K, ep)
    want_eps, want_adj = ref.load_graph(p, fmt)
    lib = C.CDLL(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pyglass_gb300",
                              "libglass_gb300.so"))
    rc, h = _load(lib, p, fmt)
    assert rc == 0
    n, k, nep, _ = _info(lib, h)
    assert (n, k) == want_adj.shape and nep == want_eps.size
    np.testing.assert_array_equal(_adj(lib, h, n, k), want_adj)
    got_eps = np.zeros(nep, np.int32)
    lib.gsx_graph_eps.argtypes = [C.c_void_p, C.c_void_p]
    assert lib.gsx_graph_eps(h, got_eps.ctypes.data) == 0
    np.testing.assert_array_equal(got_eps, want_eps)
    lib.gsx_graph_destroy.argtypes = [C.c_void_p]
    lib.gsx_graph_destroy(h)


def _workload_graph(name):
    """(glass path, base, queries) of a benchmark workload whose reference-built graph is present
    under data/ (made by oracle/build_graphs.py), else skip."""
    import json

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = os.path.join(root, "data", f"{name}.glass")
    meta = os.path.join(root, "data", f"{name}.json")
    if not (os.path.exists(path) and os.path.exists(meta)):
        pytest.skip(f"data/{name}.glass not present (built by oracle/build_graphs.py)")
    w = datasets.WORKLOADS[name]
    base = w["base"]()
    if datasets.checksum(base) != json.load(open(meta))["base_checksum"]:
        pytest.skip(f"{name}: base rows differ from the ones the graph was built on")
    return path, base, w["queries"]()


@pytest.mark.parametrize("name, cases", [
    # 960-d low-rank rows, HNSW R=32 L=200 (upper levels exercised): E5M2 and SQ8U, L2
    ("lowrank100k", [("E5M2", "", "L2"), ("SQ8U", "", "L2")]),
    # 768-d unit vectors, NSG R=48 L=100, inner product: SQ4U first pass with FP32 rerank, and FP16
    ("sphere200k", [("SQ4U", "FP32", "IP"), ("FP16", "", "IP")]),
    # 1M x 128 clusters, NSG R=32 L=50: the benchmark searcher
    ("clusters1m", [("SQ4U", "FP32", "L2")]),
])
def test_search_on_workload_graphs(oracle, ref, name, cases):
    """The oracle's searches equal the compiled reference's (ids, distances, distance counts) on the
    reference-built graphs of the workload shapes, at several ef and k in {10, 100}."""
    path, base, queries = _workload_graph(name)
    q = queries[:64]
    g = oracle.Graph(path)
    for quant, refine, metric in cases:
        rs = ref.Searcher(path, base, metric, quant, refine)
        os_ = oracle.Searcher(g, base, metric, quant, refine)
        for ef, k in [(64, 10), (128, 100)]:
            rs.set_ef(ef)
            os_.set_ef(ef)
            ri, rdis = rs.batch_search(q, k)
            oi, odis = os_.batch_search(q, k)
            np.testing.assert_array_equal(ri, oi, err_msg=f"{quant}/{refine}/{metric} ef={ef} k={k}")
            np.testing.assert_array_equal(rdis, odis, err_msg=f"{quant}/{refine}/{metric} ef={ef} k={k}")
            assert rs.get_last_search_dist_cmps() == os_.get_last_search_dist_cmps()
        # the single-query form (expansion limit max(k, ef)) on a few queries
        rs.set_ef(32)
        os_.set_ef(32)
        for i in range(4):
            a, b = rs.search(q[i], 10), os_.search(q[i], 10)
            np.testing.assert_array_equal(a[0], b[0])
            np.testing.assert_array_equal(a[1], b[1])
        del rs, os_


@pytest.mark.parametrize("K", [5, 32, 48])
@pytest.mark.parametrize("quant,metric,refine", [("SQ4U", "L2", "FP32"), ("SQ8U", "IP", ""), ("E5M2", "L2", ""),
                                                 ("FP32", "IP", ""), ("FP16", "L2", ""), ("BF16", "IP", ""),
                                                 ("SQ2U", "L2", "FP32"), ("SQ4UA", "IP", "FP32"), ("SQ1", "IP", "FP32"),
                                                 ("SQ8", "IP", "FP16"), ("SQ8", "L2", "")])
def test_edge_graphs_match_the_reference(oracle, ref, tmp_path, K, quant, metric, refine):
    """The edge graphs the GPU parity suite runs against the oracle (rows cut short by -1, repeated
    ids inside rows, several entry points with a repeat; same seeds and shapes), searched by the
    compiled reference: the oracle gives its ids, distances and distance counts, so the GPU's
    equality with the oracle on these graphs is equality with the reference.

    Two reference behaviours are undefined and are kept out of the comparison: (1) a pool that ends
    with fewer entries than requested leaves stale memory in the reference's output (neighbor.hpp:
    421-428), and under a refiner those stale ids are rescored and can rank among the results, so a
    query is compared only where its pool filled (its distance count, which equals the pool size
    below capacity, reaches the requested count); (2) FP16 encoding reads the floats after the last
    row (d not a multiple of 16), so the reference is given a buffer whose next row is zeros, which
    is what the oracle encodes there."""
    from tests.helpers import knn_graph, write_glass

    rng = np.random.default_rng(K)
    x = rng.standard_normal((1500, 40)).astype(np.float32)
    q = rng.standard_normal((70, 40)).astype(np.float32)
    adj = knn_graph(x, K, rng)
    p = str(tmp_path / "g.glass")
    write_glass(p, adj, [0, 17, 17, 900])
    xz = np.zeros((x.shape[0] + 1, x.shape[1]), np.float32)  # a zero row after the data
    xz[:-1] = x
    rs = ref.Searcher(p, xz[:-1], metric, quant, refine)
    os_ = oracle.Searcher(oracle.Graph(p), x, metric, quant, refine)
    tol = (quant, metric) == ("SQ8", "L2")  # the reference's -Ofast copies of this kernel differ by 1-2 ulp

    def same(a_ids, a_dis, b_ids, b_dis, cmps, k, msg):
        # requested count: k, or up to 3k under a refiner (reorder_k = k x refine factor)
        want = 3 * k if refine else k
        for i in range(b_ids.shape[0]):
            n = int(cmps[i])
            if refine and n < want:
                continue
            m = min(n, k)
            np.testing.assert_array_equal(a_ids[i, :m], b_ids[i, :m], err_msg=f"{msg} query {i}")
            if tol:
                np.testing.assert_allclose(a_dis[i, :m], b_dis[i, :m], rtol=1e-5, atol=0)
            else:
                np.testing.assert_array_equal(a_dis[i, :m], b_dis[i, :m], err_msg=f"{msg} query {i}")

    for ef, k in [(1, 1), (12, 10), (64, 7), (5, 20)]:
        rs.set_ef(ef)
        os_.set_ef(ef)
        ri, rd = rs.batch_search(q, k)
        oi, od = os_.batch_search(q, k)
        same(ri, rd, oi, od, os_.last_cmps, k, f"batch ef={ef} k={k}")
        assert rs.get_last_search_dist_cmps() == os_.get_last_search_dist_cmps()
        for i in range(3):
            a, b = rs.search(q[i], k), os_.search(q[i], k)
            same(a[0][None], a[1][None], b[0][None], b[1][None], os_.last_cmps, k, f"single ef={ef} k={k}")


@pytest.mark.parametrize("quant,metric,refine", [("SQ4U", "L2", "FP32"), ("FP16", "IP", ""), ("SQ8U", "L2", "")])
def test_large_pools_match_the_reference(oracle, ref, quant, metric, refine):
    """Pools of 129..256 entries (ef up to 250, k = 100 with reorder_k 150) on the reference-built
    NSG fixture: the cases of the GPU's large-pool parity test, oracle against reference."""
    from tests.golden import spec

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = os.path.join(root, "tests", "golden", "nsg_d100.glass")
    base, q = spec.base(), spec.queries()
    bz = np.zeros((base.shape[0] + 1, base.shape[1]), np.float32)  # FP16 reads the row after the last: zeros
    bz[:-1] = base
    rs = ref.Searcher(p, bz[:-1], metric, quant, refine)
    os_ = oracle.Searcher(oracle.Graph(p), base, metric, quant, refine)
    for ef, k in [(200, 10), (250, 100), (129, 100), (64, 100)]:
        rs.set_ef(ef)
        os_.set_ef(ef)
        ri, rd = rs.batch_search(q, k)
        oi, od = os_.batch_search(q, k)
        np.testing.assert_array_equal(ri, oi, err_msg=f"ef={ef} k={k}")
        np.testing.assert_array_equal(rd, od, err_msg=f"ef={ef} k={k}")
        assert rs.get_last_search_dist_cmps() == os_.get_last_search_dist_cmps()


def test_mixed_ef_and_k_match_the_reference(oracle, ref):
    """Per-query ef and k in one batch (the batched form the GPU takes, e.g. ef in {8..64}, k in
    {1, 10, 25}): each query's result equals the reference's SearchBatch run with that query's ef
    and k, since the reference has a single ef per call."""
    from tests.golden import spec

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = os.path.join(root, "tests", "golden", "hnsw_d100.glass")
    base, q = spec.base(), spec.queries()
    rng = np.random.default_rng(3)
    ef = rng.choice([8, 16, 32, 64], size=q.shape[0]).astype(np.int32)
    k = rng.choice([1, 10, 25], size=q.shape[0]).astype(np.int32)
    os_ = oracle.Searcher(oracle.Graph(p), base, "L2", "SQ4U", "FP32")
    oi, od = os_.batch_search(q, int(k.max()), ef_per_query=ef, k_per_query=k)
    rs = ref.Searcher(p, base, "L2", "SQ4U", "FP32")
    for e in np.unique(ef):
        for kk in np.unique(k):
            sel = np.where((ef == e) & (k == kk))[0]
            if sel.size == 0:
                continue
            rs.set_ef(int(e))
            ri, rd = rs.batch_search(q[sel], int(kk))
            np.testing.assert_array_equal(oi[sel, :kk], ri, err_msg=f"ef={e} k={kk}")
            np.testing.assert_array_equal(od[sel, :kk], rd, err_msg=f"ef={e} k={kk}")
            assert (oi[sel, kk:] == -1).all()


@pytest.mark.parametrize("ssg", [False, True])
@pytest.mark.parametrize("n,d,R,L", [(1500, 32, 16, 40), (3000, 64, 24, 0), (800, 7, 8, 24)])
def test_nsg_link_step_matches_the_reference(oracle, ref, n, d, R, L, ssg):
    """The link step of the NSG build (per node: search_on_graph over the kNN graph from the entry
    point, then sync_prune with the NSG or the SSG rule; nsg.hpp:129-246) run by the oracle and by the
    reference's own NSG code on the same kNN graph and entry point gives the same pruned forward
    graph.  Integer-valued rows keep every squared distance exact in fp32, so the reference's
    AVX-512 sums and the oracle's equal bit for bit.  (The kNN graph itself is NN-Descent in the
    reference, random; the reverse-link and connectivity passes depend on thread timing and random
    draws there.  The GPU build equals the oracle in every stage.)"""
    x = datasets.cluster_mixture(n, d=d, n_clusters=24, seed=31)
    g, ep, knng, _, link = oracle.nsg_build(x, R, L, ssg=ssg, return_link=True)
    want = ref.nsg_link(x, R, L, ssg, knng, ep)
    np.testing.assert_array_equal(link, want)
    assert (link[:, 0] >= 0).all()


@pytest.mark.parametrize("n,d,seed", [(1500, 32, 31), (800, 7, 31), (20000, 128, 2), (5000, 100, 7)])
def test_nsg_entry_point_matches_the_reference(oracle, ref, n, d, seed):
    """The build's entry point (the row nearest the centroid, NSG::Init, nsg.hpp:106-127): the
    oracle's equals the reference's on integer rows (exact centroid sums) and on float rows."""
    # a ring stands in for the kNN graph: only the entry point is compared
    ring = np.stack([(np.arange(n) + 1) % n, (np.arange(n) + 2) % n], axis=1).astype(np.int32)
    x = datasets.cluster_mixture(n, d=d, n_clusters=24, seed=seed)
    assert oracle.nsg_build(x, 16, 40, knn_k=2, knng=ring)[1] == ref.nsg_entry_point(x)
    y = datasets.gaussian(n, d, seed=seed)
    assert oracle.nsg_build(y, 16, 40, knn_k=2, knng=ring)[1] == ref.nsg_entry_point(y)
