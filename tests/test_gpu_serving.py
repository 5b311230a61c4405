"""The serving loop: requests of mixed sizes, k and ef submitted while others are on the GPU give
exactly the results they give alone."""

import os
import threading

import numpy as np
import pytest

from tests.golden import spec

pytestmark = pytest.mark.gpu
GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def searcher(gpu):
    return gpu.Searcher(gpu.Graph(os.path.join(GOLDEN_DIR, "nsg_d100.glass")), spec.base(), "L2", "SQ4U", "FP32")


def test_results_alone_equal_results_in_the_mix(gpu, searcher):
    rng = np.random.default_rng(7)
    q = np.concatenate([spec.queries(), spec.base()[:400]])  # 460 distinct queries
    reqs = []
    pos = 0
    while pos < q.shape[0]:
        n = int(min(q.shape[0] - pos, np.exp(rng.uniform(0, np.log(64)))))
        reqs.append((pos, n, int(rng.choice([1, 10, 40])), int(rng.choice([8, 16, 48, 96]))))
        pos += n
    # alone: each request by itself through the synchronous batched API
    alone = []
    for p0, n, k, ef in reqs:
        ids, dis = searcher.batch_search_mixed(q[p0:p0 + n], np.full(n, ef, np.int32), np.full(n, k, np.int32))
        alone.append((ids, dis))
    # in the mix: everything submitted from a producer thread while a consumer waits
    srv = gpu.Server(searcher, capacity=256, kmax=40, efmax=96, streams=3)
    tickets = [None] * len(reqs)

    def produce():
        for i, (p0, n, k, ef) in enumerate(reqs):
            tickets[i] = srv.submit(q[p0:p0 + n], k, ef)

    th = threading.Thread(target=produce)
    th.start()
    th.join()
    lat = []
    for i, (p0, n, k, ef) in enumerate(reqs):
        ids, dis, ms = srv.wait(tickets[i], n, k, timeout_ms=60000)
        np.testing.assert_array_equal(ids, alone[i][0])
        np.testing.assert_array_equal(dis, alone[i][1])
        lat.append(ms)
    done, queued, running = srv.stats()
    assert done == q.shape[0] and queued == 0
    assert min(lat) >= 0.0
    srv.close()


def test_limits_and_timeouts(gpu, searcher):
    srv = gpu.Server(searcher, capacity=64, kmax=10, efmax=32, streams=2)
    assert srv.capacity() == 64
    q = spec.queries()
    with pytest.raises(RuntimeError, match="exceeds"):
        srv.submit(q[:60].repeat(2, axis=0), 10, 16)  # 120 queries > 64 slots
    with pytest.raises(RuntimeError, match="limits"):
        srv.submit(q[:2], 11, 16)
    t = srv.submit(q[:50], 10, 32)
    try:
        srv.wait(t, 50, 10, timeout_ms=0)  # may or may not be finished yet
    except RuntimeError as e:
        assert "not finished" in str(e)
        ids, dis, _ = srv.wait(t, 50, 10, timeout_ms=60000)
        assert ids.shape == (50, 10)
    with pytest.raises(RuntimeError, match="unknown ticket"):
        srv.wait(987654, 1, 10, timeout_ms=10)
    srv.close()


def test_poisson_driver(gpu, searcher):
    srv = gpu.Server(searcher, capacity=512, kmax=40, efmax=96, streams=4)
    q = np.concatenate([spec.queries(), spec.base()[:500]])
    lat, sizes, wall = srv.drive_poisson(q, 300, 3000.0, 1, 64, [1, 10, 40], [8, 32, 96], seed=3)
    assert lat.shape == (300,) and sizes.min() >= 1 and sizes.max() <= 64
    assert np.all(lat > 0) and wall > 0
    done, queued, running = srv.stats()
    assert done == int(sizes.sum()) and queued == 0
    with pytest.raises(RuntimeError, match="load-driver"):
        srv.drive_poisson(q, 10, 100.0, 1, 1000, [10], [32])  # size_max above the admitted slots
    srv.close()
