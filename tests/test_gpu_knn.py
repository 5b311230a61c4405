"""The tensor-core exact-kNN ground truth against a brute-force CPU recompute."""

import numpy as np
import pytest

from pyglass_gb300 import datasets

pytestmark = pytest.mark.gpu


def brute(base, q, k, ip):
    if ip:
        d = -(q.astype(np.float64) @ base.astype(np.float64).T)
    else:
        d = ((q.astype(np.float64)[:, None, :] - base.astype(np.float64)[None, :, :]) ** 2).sum(-1)
    idx = np.argsort(d, axis=1, kind="stable")[:, :k]
    return idx, np.take_along_axis(d, idx, 1)


def run(gpu, base, q, k, ip):
    torch = pytest.importorskip("torch")
    b = torch.from_numpy(base).cuda()
    qq = torch.from_numpy(q).cuda()
    ids = torch.empty((q.shape[0], k), dtype=torch.int32, device="cuda")
    dis = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    exact = gpu.knn_exact(b.data_ptr(), base.shape[0], base.shape[1], qq.data_ptr(), q.shape[0], k, ip,
                          ids.data_ptr(), dis.data_ptr())
    return exact, ids.cpu().numpy(), dis.cpu().numpy()


@pytest.mark.parametrize("n,d", [(3000, 128), (5000, 100), (777, 64)])
def test_integer_data_single_exact_pass(gpu, n, d):
    base = datasets.cluster_mixture(n, d=d, n_clusters=16, seed=31)
    q = datasets.cluster_mixture(300, d=d, n_clusters=16, seed=31, stream=1)
    exact, ids, dis = run(gpu, base, q, 10, False)
    assert exact
    want_ids, want_d = brute(base, q, 10, False)
    np.testing.assert_allclose(dis, want_d, rtol=0, atol=0)  # integer data: exact distances
    # ties in distance may order ids differently from a stable CPU sort only among equal distances
    for i in range(q.shape[0]):
        assert set(ids[i][dis[i] < want_d[i, -1]]) == set(want_ids[i][want_d[i] < want_d[i, -1]])


@pytest.mark.parametrize("ip", [False, True])
def test_float_data_split_passes(gpu, ip):
    base = datasets.gaussian(20000, 96, seed=32)
    q = datasets.gaussian(256, 96, seed=32, stream=1)
    exact, ids, dis = run(gpu, base, q, 16, ip)
    assert not exact
    want_ids, want_d = brute(base, q, 16, ip)
    np.testing.assert_array_equal(ids, want_ids)
    np.testing.assert_allclose(dis, want_d, rtol=1e-6, atol=1e-5)


def test_rejects_unsupported_shapes(gpu):
    torch = pytest.importorskip("torch")
    x = torch.zeros((10, 200), device="cuda")
    o = torch.zeros((10, 4), dtype=torch.int32, device="cuda")
    with pytest.raises(RuntimeError, match="d <= 128"):
        gpu.knn_exact(x.data_ptr(), 10, 200, x.data_ptr(), 10, 4, False, o.data_ptr(), o.data_ptr())
    with pytest.raises(RuntimeError, match="k must be"):
        gpu.knn_exact(x.data_ptr(), 10, 100, x.data_ptr(), 10, 17, False, o.data_ptr(), o.data_ptr())
