"""Seeded random cases, oracle against the compiled reference: random graphs (random degree, rows
cut short by -1, repeated ids in rows, one to four entry points with repeats), random data shapes
(d from 1 to 130, so every padding rule is hit), every searcher the reference builds, random ef and
k (including k > ef and ef = 1), batch and single-query forms.  Ids, distances and distance counts
must be equal (runs where the reference checkout exists).

The reference's undefined behaviours stay out, as in the other comparisons: a query whose pool
ends with fewer entries than requested (stale output memory, rescored by a refiner), and FP16
encoding past the last row (the reference gets a zero row there, which the oracle encodes); SQ8
L2 distances are held to 1e-5 relative (the reference's -Ofast copies of that kernel differ by an
ulp or two)."""

import numpy as np
import pytest

from tests.golden import spec
from tests.helpers import write_glass

CASES = 100


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


def random_graph(rng, n):
    K = int(rng.integers(1, 65))
    adj = rng.integers(0, n, size=(n, K)).astype(np.int32)
    for i in range(n):
        if rng.random() < 0.3:
            adj[i, rng.integers(0, K):] = -1  # a row cut short (possibly empty)
        if K > 1 and rng.random() < 0.1:
            a, b = rng.integers(0, K, size=2)
            if adj[i, a] != -1 and adj[i, b] != -1:
                adj[i, b] = adj[i, a]  # a repeated id inside the row
    nep = int(rng.integers(1, 5))
    eps = list(rng.integers(0, n, size=nep))
    if nep > 1 and rng.random() < 0.5:
        eps[-1] = eps[0]  # a repeated entry point
    return adj, [int(e) for e in eps]


@pytest.mark.parametrize("case", range(CASES))
def test_random_case(oracle, ref, tmp_path, case):
    rng = np.random.default_rng(1000 + case)
    n = int(rng.integers(50, 1500))
    d = int(rng.integers(1, 131))
    quant, metric, refine = spec.SEARCHERS[int(rng.integers(0, len(spec.SEARCHERS)))]
    if rng.random() < 0.5:
        x = rng.standard_normal((n, d)).astype(np.float32)
    else:
        x = np.rint(rng.uniform(0, 255, size=(n, d))).astype(np.float32)
    q = (x[rng.integers(0, n, size=20)] + rng.standard_normal((20, d)).astype(np.float32)).astype(np.float32)
    adj, eps = random_graph(rng, n)
    p = str(tmp_path / "g.glass")
    write_glass(p, adj, eps)
    # zeros after the data for the reference's FP16 encoder, which reads up to 15 floats past the
    # last row (its 16-wide loop over the rounded-up row length)
    xz = np.zeros((n + 16 // d + 1, d), np.float32)
    xz[:n] = x
    rs = ref.Searcher(p, xz[:n], metric, quant, refine)
    os_ = oracle.Searcher(oracle.Graph(p), x, metric, quant, refine)
    tol = (quant, metric) == ("SQ8", "L2")
    what = f"case {case}: n={n} d={d} K={adj.shape[1]} eps={eps} {quant}/{metric}/{refine or '-'}"

    factor = oracle.REFINE_FACTOR[quant] if os_.refine is not None else 1.0

    def requested(k):
        # entries the pool must hold: reorder_k = (int)(k * factor) under a refiner (refiner.hpp:46)
        return int(np.float32(k) * np.float32(factor))

    def check(a_i, a_d, b_i, b_d, cmps, k, msg):
        want = requested(k)
        for i in range(b_i.shape[0]):
            c = int(cmps[i])
            if want != k and c < want:
                continue
            m = min(c, k)
            np.testing.assert_array_equal(a_i[i, :m], b_i[i, :m], err_msg=f"{what} {msg} query {i}")
            if tol:
                np.testing.assert_allclose(a_d[i, :m], b_d[i, :m], rtol=1e-5, atol=0, err_msg=f"{what} {msg}")
            else:
                np.testing.assert_array_equal(a_d[i, :m], b_d[i, :m], err_msg=f"{what} {msg} query {i}")

    for _ in range(3):
        ef = int(rng.choice([1, 2, int(rng.integers(3, 300))]))
        k = int(rng.integers(1, 121))
        rs.set_ef(ef)
        os_.set_ef(ef)
        ri, rd = rs.batch_search(q, k)
        oi, od = os_.batch_search(q, k)
        check(ri, rd, oi, od, os_.last_cmps, k, f"batch ef={ef} k={k}")
        if requested(k) == k or (os_.last_cmps >= requested(k)).all():
            assert rs.get_last_search_dist_cmps() == os_.get_last_search_dist_cmps(), f"{what} ef={ef} k={k}"
        for i in range(2):
            a, b = rs.search(q[i], k), os_.search(q[i], k)
            check(a[0][None], a[1][None], b[0][None], b[1][None], os_.last_cmps, k, f"single ef={ef} k={k}")


def random_hnsw(rng, n):
    """Random HNSW upper levels in the glass layout (HNSWInitializer.hpp:64-86): geometric levels,
    each list of hK ids drawn among the nodes present on that level, cut short by -1; the entry point
    is a node of the top level."""
    hK = int(rng.integers(1, 17))
    levels = np.minimum(rng.geometric(0.5, size=n) - 1, 5)
    top = int(levels.max())
    ep = int(rng.choice(np.where(levels == top)[0]))
    by_level = {lv: np.where(levels >= lv)[0] for lv in range(1, top + 1)}
    lists = []
    for u in range(n):
        flat = []
        for lv in range(1, int(levels[u]) + 1):
            cand = by_level[lv]
            row = list(rng.choice(cand, size=hK).astype(int))
            cut = int(rng.integers(0, hK + 1))
            row = row[:cut] + [-1] * (hK - cut)
            flat += row
        lists.append(np.array(flat, np.int32))
    return hK, ep, lists


@pytest.mark.parametrize("case", range(30))
def test_random_hnsw_case(oracle, ref, tmp_path, case):
    """Random graphs with random HNSW upper levels: the greedy descent (HNSWInitializer::initialize)
    and the search after it, oracle against reference."""
    rng = np.random.default_rng(5000 + case)
    n = int(rng.integers(50, 1200))
    d = int(rng.integers(1, 100))
    quant, metric, refine = [c for c in spec.SEARCHERS if not c[2]][int(rng.integers(0, 13))]
    x = rng.standard_normal((n, d)).astype(np.float32)
    q = rng.standard_normal((15, d)).astype(np.float32)
    adj, _ = random_graph(rng, n)
    hnsw = random_hnsw(rng, n)
    p = str(tmp_path / "h.glass")
    write_glass(p, adj, [hnsw[1]], hnsw=hnsw)
    xz = np.zeros((n + 16 // d + 1, d), np.float32)
    xz[:n] = x
    rs = ref.Searcher(p, xz[:n], metric, quant, refine)
    os_ = oracle.Searcher(oracle.Graph(p), x, metric, quant, refine)
    tol = (quant, metric) == ("SQ8", "L2")
    for ef, k in [(int(rng.integers(1, 200)), int(rng.integers(1, 50))), (1, 1)]:
        rs.set_ef(ef)
        os_.set_ef(ef)
        ri, rd = rs.batch_search(q, k)
        oi, od = os_.batch_search(q, k)
        for i in range(q.shape[0]):
            # the upper-level descent's distances count but do not enter the pool, so the pool size is
            # read from the oracle's output: its entries past the pool are -1 (the reference's stale)
            m = int((oi[i] >= 0).sum())
            np.testing.assert_array_equal(ri[i, :m], oi[i, :m], err_msg=f"case {case} {quant}/{metric} ef={ef} k={k}")
            if tol:
                np.testing.assert_allclose(rd[i, :m], od[i, :m], rtol=1e-5, atol=0)
            else:
                np.testing.assert_array_equal(rd[i, :m], od[i, :m], err_msg=f"case {case} ef={ef} k={k}")
        assert rs.get_last_search_dist_cmps() == os_.get_last_search_dist_cmps()
