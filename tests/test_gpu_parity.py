"""Parity of the GPU search path with the reference (golden fixtures) and with the oracle.

Integer SQ distances and, because the device reproduces the reference's accumulation order,
FP32/E5M2 distances too are compared for exact equality; search results (ids, distances,
distance counts) must be identical.  The golden fixtures come from the compiled reference
(tests/golden/make_golden.py)."""

import ctypes as C
import hashlib
import os

import numpy as np
import pytest

from tests.golden import spec
from tests.helpers import knn_graph, write_glass

pytestmark = pytest.mark.gpu
GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_cache = {}


def searcher(gpu, g, quant, metric, refine=""):
    key = (g, quant, metric, refine)
    if key not in _cache:
        graph = gpu.Graph(os.path.join(GOLDEN_DIR, f"{g}.glass"))
        _cache[key] = gpu.Searcher(graph, spec.base(), metric, quant, refine)
    return _cache[key]


@pytest.mark.parametrize("quant,metric", spec.SEARCHABLE)
def test_codes_and_calibration(gpu, golden, quant, metric):
    s = searcher(gpu, "nsg_d100", quant, metric)
    cs, params = s.calibration()
    codes = s.code_rows(spec.N)
    assert hashlib.sha256(codes.tobytes()).digest() == golden[f"codes_sha/{quant}/{metric}"].tobytes()
    np.testing.assert_array_equal(np.array(params, np.float32), golden[f"params/{quant}/{metric}"])


@pytest.mark.parametrize("quant,metric", spec.SEARCHABLE)
def test_distances_bit_exact(gpu, golden, quant, metric):
    refine = "FP32" if quant in ("SQ8U", "SQ4U", "SQ2U", "SQ8", "SQ4UA", "SQ1") else ""
    s = searcher(gpu, "nsg_d100", quant, metric, refine)
    q = spec.queries()[: spec.NQ_DIST]
    d = s.distances(q, golden["dist_ids"])
    if (quant, metric) in spec.FLOAT_TOLERANT:
        np.testing.assert_allclose(d, golden[f"dist/{quant}/{metric}"], rtol=spec.RTOL, atol=0)
    else:
        np.testing.assert_array_equal(d, golden[f"dist/{quant}/{metric}"])
    if refine:
        d = s.distances(q, golden["dist_ids"], refine=True)
        np.testing.assert_array_equal(d, golden[f"dist/FP32/{metric}"])


@pytest.mark.parametrize("case", list(spec.search_cases()), ids=spec.case_key)
def test_search_matches_reference(gpu, golden, case):
    g, quant, metric, refine, ef, k, mode = case
    s = searcher(gpu, g, quant, metric, refine)
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


@pytest.mark.parametrize("K", [5, 32, 48])
@pytest.mark.parametrize("quant,metric,refine", [("SQ4U", "L2", "FP32"), ("SQ8U", "IP", ""), ("E5M2", "L2", ""),
                                                 ("FP32", "IP", ""), ("FP16", "L2", ""), ("BF16", "IP", ""),
                                                 ("SQ2U", "L2", "FP32"), ("SQ4UA", "IP", "FP32"), ("SQ1", "IP", "FP32"),
                                                 ("SQ8", "IP", "FP16"), ("SQ8", "L2", "")])
def test_edge_graphs_match_oracle(gpu, oracle, tmp_path, K, quant, metric, refine):
    """Rows cut short by -1, repeated ids inside rows, several entry points with a repeat."""
    rng = np.random.default_rng(K)
    x = rng.standard_normal((1500, 40)).astype(np.float32)
    q = rng.standard_normal((70, 40)).astype(np.float32)
    adj = knn_graph(x, K, rng)
    eps = [0, 17, 17, 900]
    p = str(tmp_path / "g.glass")
    write_glass(p, adj, eps)
    gs = gpu.Searcher(gpu.Graph(p), x, metric, quant, refine)
    os_ = oracle.Searcher(oracle.Graph(p), x, metric, quant, refine)
    for ef, k in [(1, 1), (12, 10), (64, 7), (5, 20)]:
        gs.set_ef(ef)
        os_.set_ef(ef)
        gi, gd = gs.batch_search(q, k)
        oi, od = os_.batch_search(q, k)
        np.testing.assert_array_equal(gi, oi)
        np.testing.assert_array_equal(gd, od)
        assert gs.get_last_search_dist_cmps() == os_.get_last_search_dist_cmps()
        for i in range(3):
            a, b = gs.search(q[i], k), os_.search(q[i], k)
            np.testing.assert_array_equal(a[0], b[0])
            np.testing.assert_array_equal(a[1], b[1])


def test_mixed_ef_and_k(gpu, oracle):
    s = searcher(gpu, "hnsw_d100", "SQ4U", "L2", "FP32")
    o = oracle.Searcher(oracle.Graph(os.path.join(GOLDEN_DIR, "hnsw_d100.glass")), spec.base(), "L2", "SQ4U", "FP32")
    q = spec.queries()
    rng = np.random.default_rng(3)
    ef = rng.choice([8, 16, 32, 64], size=q.shape[0]).astype(np.int32)
    k = rng.choice([1, 10, 25], size=q.shape[0]).astype(np.int32)
    gi, gd = s.batch_search_mixed(q, ef, k)
    oi, od = o.batch_search(q, int(k.max()), ef_per_query=ef, k_per_query=k)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gd, od)


@pytest.mark.parametrize("spill_bits", [0, 7])
def test_visited_table_overflow_is_exact(gpu, oracle, spill_bits):
    """A 128-slot shared table (96 visits) overflows: the visited set moves to the warp's global
    spill table and the search goes on; with a 128-slot spill table too, the query is re-run by the
    host with a table sized for the whole graph.  Either way the results are exact."""
    s = searcher(gpu, "nsg_d100", "SQ8U", "L2")
    o = oracle.Searcher(oracle.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass")), spec.base(), "L2", "SQ8U")
    q = spec.queries()
    try:
        s.set_tuning(warps_per_block=4, table_bits=7, lanes_per_row=1, prefetch=1, spill_bits=spill_bits)
        s.set_ef(64)
        o.set_ef(64)
        gi, gd = s.batch_search(q, 10)
        oi, od = o.batch_search(q, 10)
        np.testing.assert_array_equal(gi, oi)
        np.testing.assert_array_equal(gd, od)
        assert s.get_last_search_dist_cmps() == o.get_last_search_dist_cmps()
    finally:
        s.set_tuning(0, 0, 0, 2, 0)


def test_tuning_variants_agree(gpu, golden):
    s = searcher(gpu, "hnsw_d100", "SQ8U", "IP")
    s.set_ef(40)
    q = spec.queries()
    ref_ids, ref_dis = s.batch_search(q, 10)
    try:
        for wpb in (1, 2, 8):
            for lpr in (1, 2, 4):
                for prefetch in (0, 1, 2, 3, 4, 7, 8, 12, 34, 35):  # 8: code rows not staged; 32: buckets
                    for bits in (0, 1, 9):  # automatic, global table only, 512 shared slots
                        s.set_tuning(warps_per_block=wpb, table_bits=bits, lanes_per_row=lpr, prefetch=prefetch,
                                     spill_bits=0)
                        ids, dis = s.batch_search(q, 10)
                        np.testing.assert_array_equal(ids, ref_ids)
                        np.testing.assert_array_equal(dis, ref_dis)
    finally:
        s.set_tuning(0, 0, 0, 2, 0)


def test_optimize_keeps_results(gpu):
    s = searcher(gpu, "nsg_d100", "SQ4U", "L2", "FP32")
    s.set_ef(32)
    q = spec.queries()
    a = s.batch_search(q, 10)
    s.optimize()
    t = s.get_tuning()
    assert t["warps_per_block"] in (2, 4, 8)
    b = s.batch_search(q, 10)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    # a visited-table size optimize picked at ef 32 (it may be one below the automatic size) gives way
    # to the automatic size of larger pools: the device batch, which re-runs nothing, answers every
    # query at ef 256 as the host batch does
    torch = pytest.importorskip("torch")
    s.set_ef(256)
    hi, hd = s.batch_search(q, 10)
    dq = torch.from_numpy(q).cuda()
    di = torch.empty((q.shape[0], 10), dtype=torch.int32, device="cuda")
    dd = torch.empty((q.shape[0], 10), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    s.batch_search_device(dq.data_ptr(), q.shape[0], 10, di.data_ptr(), dd.data_ptr(), kmax=10)
    torch.cuda.synchronize()
    assert s.overflow_count() == 0
    np.testing.assert_array_equal(di.cpu().numpy(), hi)
    np.testing.assert_array_equal(dd.cpu().numpy(), hd)
    s.set_tuning(0, 0, 0, 2, 0)


def test_edge_inputs(gpu):
    s = searcher(gpu, "nsg_d100", "SQ8U", "L2")
    s.set_ef(16)
    ids, dis = s.batch_search(np.zeros((0, spec.D), np.float32), 10)
    assert ids.shape == (0, 10)
    with pytest.raises(RuntimeError, match="dimension"):
        s.batch_search(np.zeros((2, spec.D + 1), np.float32), 10)
    with pytest.raises(RuntimeError):
        s.batch_search(np.zeros((2, spec.D), np.float32), 0)
    with pytest.raises(RuntimeError, match="capacity"):
        s.batch_search(np.zeros((1, spec.D), np.float32), 5000)
    with pytest.raises(RuntimeError):
        s.set_ef(0)
    g = gpu.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass"))
    with pytest.raises(RuntimeError, match="rows"):
        gpu.Searcher(g, spec.base()[:100], "L2", "SQ8U")
    with pytest.raises(RuntimeError, match="outside"):
        gpu.Searcher(gpu.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass")), spec.base(), "L2", "PQ8")


def test_fewer_results_than_k(gpu, oracle, tmp_path):
    """A graph whose reachable part is smaller than k: missing entries are -1 / inf."""
    x = np.random.default_rng(9).standard_normal((40, 16)).astype(np.float32)
    adj = np.full((40, 4), -1, np.int32)
    adj[0, :2] = [1, 2]
    p = str(tmp_path / "tiny.glass")
    write_glass(p, adj, [0])
    s = gpu.Searcher(gpu.Graph(p), x, "L2", "FP32")
    ids, dis = s.batch_search(x[:3], 5)
    assert (ids[:, 3:] == -1).all() and np.isinf(dis[:, 3:]).all()
    o = oracle.Searcher(oracle.Graph(p), x, "L2", "FP32")
    oi, od = o.batch_search(x[:3], 5)
    np.testing.assert_array_equal(ids, oi)


def test_device_pointer_batch(gpu):
    torch = pytest.importorskip("torch")
    s = searcher(gpu, "hnsw_d100", "E5M2", "L2")
    s.set_ef(32)
    q = spec.queries()
    hi, hd = s.batch_search(q, 10)
    dq = torch.from_numpy(q).cuda()
    di = torch.empty((q.shape[0], 10), dtype=torch.int32, device="cuda")
    dd = torch.empty((q.shape[0], 10), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    s.batch_search_device(dq.data_ptr(), q.shape[0], 10, di.data_ptr(), dd.data_ptr(), kmax=10)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(di.cpu().numpy(), hi)
    np.testing.assert_array_equal(dd.cpu().numpy(), hd)


def test_plain_c_abi(gpu):
    """One search driven through the C ABI with ctypes, as a non-Python host would call it."""
    lib = C.CDLL(os.path.join(ROOT, "pyglass_gb300", "libglass_gb300.so"))
    vp = C.c_void_p
    lib.gsx_graph_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
    lib.gsx_searcher_create.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.POINTER(vp)]
    lib.gsx_searcher_set_data.argtypes = [vp, C.c_void_p, C.c_int32, C.c_int32]
    lib.gsx_searcher_set_ef.argtypes = [vp, C.c_int32]
    lib.gsx_searcher_search_batch.argtypes = [vp, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    lib.gsx_searcher_destroy.argtypes = [vp]
    lib.gsx_graph_destroy.argtypes = [vp]
    g, s = vp(), vp()
    assert lib.gsx_graph_load(os.path.join(GOLDEN_DIR, "nsg_d100.glass").encode(), b"glass", C.byref(g)) == 0
    assert lib.gsx_searcher_create(g, b"L2", b"SQ4U", b"FP32", 0, C.byref(s)) == 0
    base = spec.base()
    assert lib.gsx_searcher_set_data(s, base.ctypes.data, base.shape[0], base.shape[1]) == 0
    assert lib.gsx_searcher_set_ef(s, 16) == 0
    q = spec.queries()
    ids = np.zeros((q.shape[0], 10), np.int32)
    dis = np.zeros((q.shape[0], 10), np.float32)
    assert lib.gsx_searcher_search_batch(s, q.ctypes.data, q.shape[0], 10, ids.ctypes.data, dis.ctypes.data) == 0
    lib.gsx_searcher_destroy(s)
    lib.gsx_graph_destroy(g)
    ref = searcher(gpu, "nsg_d100", "SQ4U", "L2", "FP32")
    ref.set_ef(16)
    np.testing.assert_array_equal(ids, ref.batch_search(q, 10)[0])


def test_sq1_searcher_needs_ip(gpu):
    """The reference builds SQ1 searchers for the IP metric only (graph_searcher.hpp:362-369)."""
    graph = gpu.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass"))
    with pytest.raises(RuntimeError, match="IP metric only"):
        gpu.Searcher(graph, spec.base(), "L2", "SQ1")


@pytest.mark.parametrize("quant,metric,refine", [("SQ4U", "L2", "FP32"), ("FP16", "IP", ""), ("SQ8U", "L2", "")])
def test_large_pools_match_oracle(gpu, oracle, quant, metric, refine):
    """Pools of 129..256 entries (ef up to 250; k = 100 with the 1.5x refine gives reorder_k 150): the
    register merge's two-block path, against the oracle."""
    s = searcher(gpu, "nsg_d100", quant, metric, refine)
    o = oracle.Searcher(oracle.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass")), spec.base(), metric, quant, refine)
    q = spec.queries()
    for ef, k in [(200, 10), (250, 100), (129, 100), (64, 100)]:
        s.set_ef(ef)
        o.set_ef(ef)
        gi, gd = s.batch_search(q, k)
        oi, od = o.batch_search(q, k)
        np.testing.assert_array_equal(gi, oi)
        np.testing.assert_array_equal(gd, od)
        assert s.get_last_search_dist_cmps() == o.get_last_search_dist_cmps()
