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


def test_generator_bytes_are_pinned():
    """The first rows of every workload generator hash to fixed values, so a numpy whose random
    streams or float reductions differ from the build host's is caught here (the benchmark graphs
    under data/ record the full-size checksums they were built from, and the GPU tests skip a
    workload whose rows differ)."""
    assert datasets.checksum(datasets.cluster_mixture(5000)) == "616f3532b8760553"
    assert datasets.checksum(datasets.cluster_mixture(2000, stream=1)) == "534f519677ca8cf3"
    assert datasets.checksum(datasets.gaussian(1000, 128, seed=1)) == "a067f7f3a779c815"
    assert datasets.checksum(datasets.low_rank(2000, 960, seed=3)) == "b1be06207028329f"
    assert datasets.checksum(datasets.normalized_mixture(2000, 768, seed=4)) == "55f41e05b3a1ce26"
