"""Seeded synthetic stand-ins for the benchmark workloads of the graph-search path.

The reference measures on ann-benchmarks HDF5 sets (python/ann_dataset/dataset.py:68-88) that are
not available offline; these generators produce inputs with the shapes and value distributions
of the named workloads instead.  numpy's PCG64 streams are identical on x86 and aarch64, so the
same call returns the same bytes on every host; ``checksum`` lets a caller verify that.
"""

from __future__ import annotations

import hashlib

import numpy as np

_CHUNK = 100_000


def gaussian(n: int, d: int, seed: int, stream: int = 0) -> np.ndarray:
    """n x d i.i.d. N(0,1) float32 rows."""
    rng = np.random.default_rng([seed, stream])
    return rng.standard_normal((n, d), dtype=np.float32)


def cluster_mixture(n: int, d: int = 128, n_clusters: int = 1024, sigma: float = 12.0, seed: int = 2,
                    stream: int = 0) -> np.ndarray:
    """Gaussian-mixture rows: centers uniform in [0,128]^d (shared by every stream of a seed),
    per-dimension sigma, rounded and clipped to the integers 0..255, stored float32."""
    centers = np.random.default_rng([seed, 999]).uniform(0.0, 128.0, size=(n_clusters, d))
    rng = np.random.default_rng([seed, stream])
    out = np.empty((n, d), np.float32)
    for s in range(0, n, _CHUNK):
        m = min(_CHUNK, n - s)
        lab = rng.integers(0, n_clusters, size=m)
        x = centers[lab] + rng.normal(0.0, sigma, size=(m, d))
        out[s:s + m] = np.clip(np.rint(x), 0, 255)
    return out


def low_rank(n: int, d: int = 960, rank: int = 32, noise: float = 0.05, seed: int = 3, stream: int = 0) -> np.ndarray:
    """x = W z + e with z ~ N(0, I_rank), W (d x rank) ~ N(0, 1/rank) shared per seed, e zero-mean noise
    of standard deviation `noise` (a scaled sum of four uniforms)."""
    w = np.random.default_rng([seed, 999]).normal(0.0, 1.0 / np.sqrt(rank), size=(d, rank)).astype(np.float32)
    rng = np.random.default_rng([seed, stream])
    out = np.empty((n, d), np.float32)
    step = 10_000
    for s in range(0, n, step):
        m = min(step, n - s)
        z = rng.standard_normal((m, rank), dtype=np.float32)
        # noise: a sum of four uniforms, centred and scaled to sd `noise` (built from integer-derived
        # doubles only, so every host produces the same bytes)
        u = rng.random((4, m, d))
        acc = (u[0] + u[1] + u[2] + u[3] - 2.0) * (np.sqrt(3.0) * noise)
        # elementwise float64 products summed in a fixed order: a BLAS product would round
        # differently on different hosts
        for r in range(rank):
            acc += z[:, r:r + 1].astype(np.float64) * w[:, r].astype(np.float64)
        out[s:s + m] = acc
    return out


def normalized_mixture(n: int, d: int = 768, n_clusters: int = 4096, sigma: float = 0.3, seed: int = 4,
                       stream: int = 0) -> np.ndarray:
    """Unit-length rows of a Gaussian mixture (centers ~ N(0, I), within-cluster sigma).

    Every random value is built from integer-derived uniforms by correctly rounded arithmetic alone,
    so x86 and aarch64 hosts produce the same bytes: a normal deviate is a centred, scaled sum of four
    uniforms (numpy's ziggurat samplers call libm's exp and log, whose last bits differ between hosts,
    and a flipped accept/reject decision desynchronises the stream), and the row norms are sums of
    float64 squares taken column by column in a fixed order (a float32 ``np.linalg.norm`` reduces in
    SIMD-width-dependent order)."""

    def normals(rng, shape):
        u = rng.random((4,) + shape)
        return (u[0] + u[1] + u[2] + u[3] - 2.0) * np.sqrt(3.0)

    centers = normals(np.random.default_rng([seed, 999]), (n_clusters, d))
    rng = np.random.default_rng([seed, stream])
    out = np.empty((n, d), np.float32)
    step = 20_000
    for s in range(0, n, step):
        m = min(step, n - s)
        lab = rng.integers(0, n_clusters, size=m)
        xt = np.ascontiguousarray((centers[lab] + normals(rng, (m, d)) * sigma).T)
        ss = np.zeros(m)
        for j in range(d):
            ss += xt[j] * xt[j]
        out[s:s + m] = (xt / np.sqrt(ss)).T.astype(np.float32)
    return out


# name -> (base generator, query generator, description).  Queries use stream 1 of the same seed.
WORKLOADS = {
    "gauss10k": dict(base=lambda: gaussian(10_000, 128, seed=1), queries=lambda: gaussian(1_000, 128, seed=1, stream=1),
                     index=("HNSW", 32, 50, "FP32"), metric="L2",
                     desc="10,000 x 128 N(0,1), HNSW R=32 L=50, 1,000 queries"),
    "clusters1m": dict(base=lambda: cluster_mixture(1_000_000), queries=lambda: cluster_mixture(10_000, stream=1),
                       index=("NSG", 32, 50, "SQ8U"), metric="L2",
                       desc="1,000,000 x 128 from 1,024 clusters (sigma 12, integers 0..255), NSG R=32 L=50 "
                            "(build quant SQ8U), 10,000 queries"),
    # reduced-size versions of the 960-d low-rank (HNSW R=32 L=200) and 768-d normalised (NSG
    # R=48 L=100, inner product) workloads, used as parity cases
    "lowrank100k": dict(base=lambda: low_rank(100_000, 960, seed=3), queries=lambda: low_rank(1_000, 960, seed=3, stream=1),
                        index=("HNSW", 32, 200, "SQ8U"), metric="L2",
                        desc="100,000 x 960 low-rank (x = Wz + e, rank 32, noise 0.05), HNSW R=32 L=200, 1,000 queries"),
    "lowrank1m": dict(base=lambda: low_rank(1_000_000, 960, seed=3), queries=lambda: low_rank(1_000, 960, seed=3, stream=1),
                      index=("HNSW", 32, 200, "SQ8U"), metric="L2",
                      desc="1,000,000 x 960 low-rank (x = Wz + e, rank 32, noise 0.05), HNSW R=32 L=200, 1,000 queries"),
    "sphere2m": dict(base=lambda: normalized_mixture(2_000_000, 768, seed=4),
                     queries=lambda: normalized_mixture(10_000, 768, seed=4, stream=1),
                     index=("NSG", 48, 100, "SQ8U"), metric="IP",
                     desc="2,000,000 x 768 unit vectors from 4,096 clusters (sigma 0.3), NSG R=48 L=100 (L2 build), "
                          "10,000 queries, inner product"),
    "sphere200k": dict(base=lambda: normalized_mixture(200_000, 768, seed=4),
                       queries=lambda: normalized_mixture(2_000, 768, seed=4, stream=1),
                       index=("NSG", 48, 100, "SQ8U"), metric="IP",
                       desc="200,000 x 768 unit vectors from 4,096 clusters (sigma 0.3), NSG R=48 L=100 (L2 build), "
                            "2,000 queries, inner product"),
}


def graph_file(name: str, root: str) -> tuple[str, str] | None:
    """(path, format) of a workload's graph under root/data: the glass file, else its compact
    NSG-format twin; None when neither exists."""
    import os

    for ext, fmt in ((".glass", "glass"), (".nsg", "nsg")):
        p = os.path.join(root, "data", name + ext)
        if os.path.exists(p):
            return p, fmt
    return None


def checksum(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]
