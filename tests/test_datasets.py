"""The synthetic workload generators are deterministic and have the stated shapes/ranges."""

import numpy as np

from pyglass_gb300 import datasets


def test_cluster_mixture_is_integer_valued():
    x = datasets.cluster_mixture(3000, d=16, n_clusters=8, seed=2)
    assert x.dtype == np.float32 and x.shape == (3000, 16)
    assert np.all(x == np.rint(x)) and x.min() >= 0 and x.max() <= 255
    assert datasets.checksum(x) == datasets.checksum(datasets.cluster_mixture(3000, d=16, n_clusters=8, seed=2))


def test_streams_differ_and_shapes():
    a = datasets.gaussian(10, 8, seed=1)
    b = datasets.gaussian(10, 8, seed=1, stream=1)
    assert not np.array_equal(a, b)
    y = datasets.low_rank(100, d=64, rank=8, seed=3)
    assert y.shape == (100, 64)
    z = datasets.normalized_mixture(100, d=32, n_clusters=4, seed=4)
    np.testing.assert_allclose(np.linalg.norm(z, axis=1), 1.0, rtol=1e-5)
