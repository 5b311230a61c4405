"""The CUDA-graph form of the device batch (gsx_searcher_capture_batch / gsx_batch_graph_launch):
a captured batch, replayed after its query buffer is refilled in place, returns exactly what the
device batch entry point returns for the same queries (the same kernels and arithmetic; only the
launch path and the scratch storage differ)."""

import os

import numpy as np
import pytest

from pyglass_gb300 import datasets
from tests.golden import spec

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GRAPH = os.path.join(ROOT, "tests", "golden", "nsg_d100.glass")


def searcher(gpu, quant="SQ4U", refine="FP32", ef=48):
    s = gpu.Searcher(gpu.Graph(GRAPH), spec.base(), "L2", quant, refine)
    s.set_ef(ef)
    return s


def device_batch(torch, s, q, k, ef_per=None, k_per=None, kmax=None):
    kmax = kmax or k
    dq = torch.from_numpy(q).cuda()
    ids = torch.full((q.shape[0], kmax), -7, dtype=torch.int32, device="cuda")
    dis = torch.zeros((q.shape[0], kmax), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    s.batch_search_device(dq.data_ptr(), q.shape[0], k, ids.data_ptr(), dis.data_ptr(),
                          ef_per=0 if ef_per is None else ef_per.data_ptr(),
                          k_per=0 if k_per is None else k_per.data_ptr(), kmax=kmax)
    torch.cuda.synchronize()
    return ids.cpu().numpy(), dis.cpu().numpy()


def test_replays_match_the_device_batch(gpu):
    torch = pytest.importorskip("torch")
    s = searcher(gpu)
    k = 10
    a = np.concatenate([spec.queries(), spec.base()[:200]])
    b = datasets.gaussian(a.shape[0], spec.D, seed=11, stream=5)
    want_a, want_b = device_batch(torch, s, a, k), device_batch(torch, s, b, k)
    assert (want_a[0] >= 0).all() and (want_b[0] >= 0).all()
    dq = torch.from_numpy(a).cuda()
    ids = torch.full((a.shape[0], k), -7, dtype=torch.int32, device="cuda")
    dis = torch.zeros((a.shape[0], k), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    g = s.capture_batch_device(dq.data_ptr(), a.shape[0], k, ids.data_ptr(), dis.data_ptr())
    # the capture call ran the batch once
    np.testing.assert_array_equal(ids.cpu().numpy(), want_a[0])
    np.testing.assert_array_equal(dis.cpu().numpy(), want_a[1])
    for rnd, (q, want) in enumerate([(b, want_b), (a, want_a), (a, want_a), (b, want_b)]):
        dq.copy_(torch.from_numpy(q))
        ids.fill_(-7)
        dis.zero_()
        torch.cuda.synchronize()
        g.launch()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ids.cpu().numpy(), want[0], err_msg=f"replay {rnd}")
        np.testing.assert_array_equal(dis.cpu().numpy(), want[1], err_msg=f"replay {rnd}")
        assert g.overflow_count() == 0
    g.close()
    with pytest.raises(RuntimeError):
        g.launch()


def test_large_mixed_batch_on_a_caller_stream(gpu):
    """More queries than resident warps (the batch-order kernels are part of the graph), per-query
    ef and k on the device, replays on a stream of the caller's."""
    torch = pytest.importorskip("torch")
    s = searcher(gpu, "SQ8U", "", 48)
    nq, kmax = 12000, 20
    q = datasets.gaussian(nq, spec.D, seed=11, stream=6)
    rng = np.random.default_rng(5)
    efp = torch.from_numpy(rng.choice(np.array([16, 32, 48], np.int32), nq)).cuda()
    kp = torch.from_numpy(rng.choice(np.array([10, 20], np.int32), nq)).cuda()
    want = device_batch(torch, s, q, kmax, efp, kp, kmax)
    dq = torch.from_numpy(q).cuda()
    ids = torch.full((nq, kmax), -7, dtype=torch.int32, device="cuda")
    dis = torch.zeros((nq, kmax), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    g = s.capture_batch_device(dq.data_ptr(), nq, kmax, ids.data_ptr(), dis.data_ptr(), ef_per=efp.data_ptr(),
                               k_per=kp.data_ptr(), kmax=kmax)
    st = torch.cuda.Stream()
    for rnd in range(2):
        ids.fill_(-7)
        dis.zero_()
        torch.cuda.synchronize()
        g.launch(st.cuda_stream)
        st.synchronize()
        # a query's first k entries are its results (k from its own k_per)
        mask = np.arange(kmax)[None, :] < kp.cpu().numpy()[:, None]
        np.testing.assert_array_equal(ids.cpu().numpy()[mask], want[0][mask], err_msg=f"replay {rnd}")
        np.testing.assert_array_equal(dis.cpu().numpy()[mask], want[1][mask], err_msg=f"replay {rnd}")
        assert g.overflow_count() == 0
    g.close()


def test_capture_rejects_bad_arguments(gpu):
    torch = pytest.importorskip("torch")
    s = searcher(gpu)
    buf = torch.zeros((4, spec.D), dtype=torch.float32, device="cuda")
    out = torch.zeros((4, 10), dtype=torch.int32, device="cuda")
    with pytest.raises(RuntimeError):
        s.capture_batch_device(buf.data_ptr(), 0, 10, out.data_ptr(), out.data_ptr())
    with pytest.raises(RuntimeError):
        s.capture_batch_device(buf.data_ptr(), 4, 0, out.data_ptr(), out.data_ptr())
