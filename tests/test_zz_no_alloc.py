"""The allocation-free batched search (gsx_searcher_search_batch_noalloc), driven through the C ABI
the way a caller that may not allocate device memory would use it (an engine whose device memory is
all handed to its own pool, or a latency path that cannot take an allocation's synchronisation): it
must return what the allocating device entry point returns, on two calls in a row over the same
shared scratch, leave the driver's free memory unchanged, report the queries a too-small visited
table left unanswered, and give the calling thread its current device back."""

import ctypes as C
import os

import numpy as np
import pytest

from tests.golden import spec

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GRAPH = os.path.join(ROOT, "tests", "golden", "nsg_d100.glass")


class Tuning(C.Structure):
    _fields_ = [("warps_per_block", C.c_int32), ("table_bits", C.c_int32), ("lanes_per_row", C.c_int32),
                ("prefetch", C.c_int32), ("spill_bits", C.c_int32)]


@pytest.fixture(scope="module")
def abi(gpu):
    lib = C.CDLL(os.path.join(ROOT, "pyglass_gb300", "libglass_gb300.so"))
    vp = C.c_void_p
    lib.gsx_last_error.restype = C.c_char_p
    lib.gsx_graph_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(vp)]
    lib.gsx_graph_destroy.argtypes = [vp]
    lib.gsx_searcher_create.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.POINTER(vp)]
    lib.gsx_searcher_set_data.argtypes = [vp, vp, C.c_int32, C.c_int32]
    lib.gsx_searcher_set_ef.argtypes = [vp, C.c_int32]
    lib.gsx_searcher_search_batch_device.argtypes = [vp, vp, C.c_int32, C.c_int32, vp, vp, C.c_int32, vp, vp, vp, vp,
                                                     vp]
    lib.gsx_searcher_search_batch_noalloc.argtypes = [vp, vp, C.c_int32, C.c_int32, vp, vp, vp]
    lib.gsx_searcher_noalloc_overflow_count.argtypes = [vp, C.POINTER(C.c_uint32)]
    lib.gsx_searcher_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    lib.gsx_searcher_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
    lib.gsx_searcher_destroy.argtypes = [vp]
    g, s = vp(), vp()
    assert lib.gsx_graph_load(GRAPH.encode(), b"glass", C.byref(g)) == 0, lib.gsx_last_error()
    assert lib.gsx_searcher_create(g, b"L2", b"SQ4U", b"FP32", 0, C.byref(s)) == 0, lib.gsx_last_error()
    lib.gsx_graph_destroy(g)
    base = spec.base()
    assert lib.gsx_searcher_set_data(s, base.ctypes.data, base.shape[0], base.shape[1]) == 0, lib.gsx_last_error()
    assert lib.gsx_searcher_set_ef(s, 48) == 0
    yield lib, s
    lib.gsx_searcher_destroy(s)


def test_noalloc_matches_device_entry_point_twice(abi):
    torch = pytest.importorskip("torch")
    lib, s = abi
    k = 10
    q = torch.from_numpy(np.concatenate([spec.queries(), spec.base()[:200]])).cuda()
    nq = q.shape[0]
    ref_ids = torch.full((nq, k), -7, dtype=torch.int32, device="cuda")
    ref_dis = torch.zeros((nq, k), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.gsx_searcher_search_batch_device(s, q.data_ptr(), nq, k, None, None, k, ref_ids.data_ptr(),
                                              ref_dis.data_ptr(), None, None, None)
    assert rc == 0, lib.gsx_last_error()
    torch.cuda.synchronize()
    assert (ref_ids >= 0).all()
    for call in range(2):
        ids = torch.full((nq, k), -7, dtype=torch.int32, device="cuda")
        dis = torch.zeros((nq, k), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.gsx_searcher_search_batch_noalloc(s, q.data_ptr(), nq, k, ids.data_ptr(), dis.data_ptr(), None)
        assert rc == 0, lib.gsx_last_error()
        torch.cuda.synchronize()
        # exact equality: the same kernel arithmetic, only the scratch storage differs
        np.testing.assert_array_equal(ids.cpu().numpy(), ref_ids.cpu().numpy(), err_msg=f"call {call}")
        np.testing.assert_array_equal(dis.cpu().numpy(), ref_dis.cpu().numpy(), err_msg=f"call {call}")
        n = C.c_uint32(99)
        assert lib.gsx_searcher_noalloc_overflow_count(s, C.byref(n)) == 0, lib.gsx_last_error()
        assert n.value == 0


def test_noalloc_allocates_nothing(abi):
    """After a first call on the device (which looks up the fixed array's address), further calls
    leave the driver's free device memory exactly where it was."""
    torch = pytest.importorskip("torch")
    lib, s = abi
    k = 10
    q = torch.from_numpy(spec.queries()).cuda()
    nq = q.shape[0]
    ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dis = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    assert lib.gsx_searcher_search_batch_noalloc(s, q.data_ptr(), nq, k, ids.data_ptr(), dis.data_ptr(), None) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert lib.gsx_searcher_search_batch_noalloc(s, q.data_ptr(), nq, k, ids.data_ptr(), dis.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_overflow_is_reported(abi):
    """A 128-slot shared-memory table (at most 96 visits) over a range of ef: the queries whose
    visited sets outgrow it come back as all -1 / +inf, the count call says how many, and every
    other query equals the allocating entry point's answer (which moves an outgrown set to a larger
    table and answers every query).  Some ef in the range leaves part of the batch unanswered."""
    torch = pytest.importorskip("torch")
    lib, s = abi
    t0 = Tuning()
    assert lib.gsx_searcher_get_tuning(s, C.byref(t0)) == 0
    t = Tuning(t0.warps_per_block, 7, t0.lanes_per_row, t0.prefetch, t0.spill_bits)
    assert lib.gsx_searcher_set_tuning(s, C.byref(t)) == 0, lib.gsx_last_error()
    k = 10
    q = torch.from_numpy(np.concatenate([spec.queries(), spec.base()[:200]])).cuda()
    nq = q.shape[0]
    counts = []
    try:
        for ef in (2, 4, 8, 16, 32, 64):
            assert lib.gsx_searcher_set_ef(s, ef) == 0
            ref_ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
            ref_dis = torch.empty((nq, k), dtype=torch.float32, device="cuda")
            rc = lib.gsx_searcher_search_batch_device(s, q.data_ptr(), nq, k, None, None, k, ref_ids.data_ptr(),
                                                      ref_dis.data_ptr(), None, None, None)
            assert rc == 0, lib.gsx_last_error()
            ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
            dis = torch.empty((nq, k), dtype=torch.float32, device="cuda")
            rc = lib.gsx_searcher_search_batch_noalloc(s, q.data_ptr(), nq, k, ids.data_ptr(), dis.data_ptr(), None)
            assert rc == 0, lib.gsx_last_error()
            torch.cuda.synchronize()
            n = C.c_uint32(12345)
            assert lib.gsx_searcher_noalloc_overflow_count(s, C.byref(n)) == 0, lib.gsx_last_error()
            gi, gd = ids.cpu().numpy(), dis.cpu().numpy()
            ri, rd = ref_ids.cpu().numpy(), ref_dis.cpu().numpy()
            lost = gi[:, 0] == -1
            assert int(lost.sum()) == n.value, f"ef={ef}"
            assert (gi[lost] == -1).all() and np.isinf(gd[lost]).all(), f"ef={ef}"
            assert (ri[:, 0] >= 0).all(), f"ef={ef}"
            np.testing.assert_array_equal(gi[~lost], ri[~lost], err_msg=f"ef={ef}")
            np.testing.assert_array_equal(gd[~lost], rd[~lost], err_msg=f"ef={ef}")
            counts.append(n.value)
    finally:
        assert lib.gsx_searcher_set_tuning(s, C.byref(t0)) == 0
        assert lib.gsx_searcher_set_ef(s, 48) == 0
    assert any(0 < c < nq for c in counts), counts
    assert counts[-1] > 0, counts


def test_noalloc_keeps_the_callers_device(abi):
    torch = pytest.importorskip("torch")
    lib, s = abi
    before = torch.cuda.current_device()
    q = torch.from_numpy(spec.queries()[:8]).cuda()
    ids = torch.empty((8, 10), dtype=torch.int32, device="cuda")
    assert lib.gsx_searcher_search_batch_noalloc(s, q.data_ptr(), 8, 10, ids.data_ptr(), None, None) == 0
    torch.cuda.synchronize()
    assert torch.cuda.current_device() == before


def test_noalloc_rejects_too_many_queries(abi):
    lib, s = abi
    rc = lib.gsx_searcher_search_batch_noalloc(s, C.c_void_p(16), 65537, 10, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == 1
    assert b"65536" in lib.gsx_last_error()
