"""Parity on the other workload shapes: the GPU searcher equals the oracle on reference-built
graphs of each config (the 960-d and 768-d sets at reduced size: 100k and 200k base rows)."""

import json
import os

import numpy as np
import pytest

from pyglass_gb300 import datasets
from tests.helpers import oracle_graph

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load(name):
    found = datasets.graph_file(name, ROOT)
    if found is None:
        pytest.skip(f"data/{name}.glass not present (built by oracle/build_graphs.py)")
    path, fmt = found
    meta = json.load(open(os.path.join(ROOT, "data", f"{name}.json")))
    w = datasets.WORKLOADS[name]
    base, q = w["base"](), w["queries"]()
    if datasets.checksum(base) != meta["base_checksum"]:
        pytest.skip(f"{name}: this host generates different base rows than the host that built the graph")
    return (path, fmt), base, q


def test_gauss10k_hnsw_sq8u_single_query_calls(gpu, oracle):
    """10,000 x 128 N(0,1), HNSW R=32 L=50, SQ8U, ef=32, k=10, one query per call."""
    path, base, q = load("gauss10k")
    s = gpu.Searcher(gpu.Graph(*path), base, "L2", "SQ8U")
    o = oracle.Searcher(oracle_graph(oracle, gpu, *path), base, "L2", "SQ8U")
    s.set_ef(32)
    o.set_ef(32)
    for i in range(0, q.shape[0], 5):
        a, b = s.search(q[i], 10), o.search(q[i], 10)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    gi, gd = s.batch_search(q, 10)
    oi, od = o.batch_search(q, 10)
    np.testing.assert_array_equal(gi, oi)
    assert s.get_last_search_dist_cmps() == o.get_last_search_dist_cmps()


@pytest.mark.parametrize("quant", ["E5M2", "SQ8U"])
def test_lowrank960_hnsw_mixed_ef_k(gpu, oracle, quant):
    """960-d low-rank data, HNSW R=32 L=200; per-query ef in {64,128,256} and k in {10,100}."""
    path, base, q = load("lowrank100k")
    q = q[:300]
    rng = np.random.default_rng(11)
    ef = rng.choice([64, 128, 256], size=q.shape[0]).astype(np.int32)
    k = rng.choice([10, 100], size=q.shape[0]).astype(np.int32)
    s = gpu.Searcher(gpu.Graph(*path), base, "L2", quant)
    s.set_ef(256)
    s.optimize()
    gi, gd = s.batch_search_mixed(q, ef, k)
    o = oracle.Searcher(oracle_graph(oracle, gpu, *path), base, "L2", quant)
    oi, od = o.batch_search(q, 100, ef_per_query=ef, k_per_query=k)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gd, od)


def test_sphere768_nsg_ip_sq4u_refine(gpu, oracle):
    """768-d unit vectors, NSG R=48 L=100, inner product, SQ4U first pass + FP32 rerank."""
    path, base, q = load("sphere200k")
    q = q[:400]
    s = gpu.Searcher(gpu.Graph(*path), base, "IP", "SQ4U", "FP32")
    o = oracle.Searcher(oracle_graph(oracle, gpu, *path), base, "IP", "SQ4U", "FP32")
    for ef in (32, 128, 256):
        s.set_ef(ef)
        o.set_ef(ef)
        gi, gd = s.batch_search(q, 10)
        oi, od = o.batch_search(q, 10)
        np.testing.assert_array_equal(gi, oi)
        np.testing.assert_array_equal(gd, od)


def test_lowrank1m_hnsw_e5m2_full_size(gpu, oracle):
    """Full size: 1,000,000 x 960 low-rank data, HNSW R=32 L=200, E5M2, mixed ef/k; 100 queries
    against the oracle, sortedness and id validity for all 1,000."""
    path, base, q = load("lowrank1m")
    rng = np.random.default_rng(5)
    ef = rng.choice([64, 128, 256], size=q.shape[0]).astype(np.int32)
    k = rng.choice([10, 100], size=q.shape[0]).astype(np.int32)
    s = gpu.Searcher(gpu.Graph(*path), base, "L2", "E5M2")
    s.set_ef(256)
    gi, gd = s.batch_search_mixed(q, ef, k)
    o = oracle.Searcher(oracle_graph(oracle, gpu, *path), base, "L2", "E5M2")
    sample = np.arange(0, q.shape[0], 10)
    oi, od = o.batch_search(q[sample], 100, ef_per_query=ef[sample], k_per_query=k[sample])
    np.testing.assert_array_equal(gi[sample], oi)
    np.testing.assert_array_equal(gd[sample], od)
    for i in range(q.shape[0]):
        row = gd[i, : k[i]]
        assert np.all(np.diff(row) >= 0) and np.all(gi[i, : k[i]] >= 0)


def test_sphere2m_nsg_ip_full_size(gpu, oracle):
    """Full size: 2,000,000 x 768 unit vectors, NSG R=48 L=100, IP, SQ4U + FP32 rerank."""
    path, base, q = load("sphere2m")
    s = gpu.Searcher(gpu.Graph(*path), base, "IP", "SQ4U", "FP32")
    o = oracle.Searcher(oracle_graph(oracle, gpu, *path), base, "IP", "SQ4U", "FP32")
    s.set_ef(64)
    o.set_ef(64)
    gi, gd = s.batch_search(q, 10)
    sample = np.arange(0, q.shape[0], 50)
    oi, od = o.batch_search(q[sample], 10)
    np.testing.assert_array_equal(gi[sample], oi)
    np.testing.assert_array_equal(gd[sample], od)
    assert np.all(np.diff(gd, axis=1) >= 0)
