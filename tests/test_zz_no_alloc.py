"""The allocation-free batched search (gsx_searcher_search_batch_noalloc), driven through the C ABI
the way a caller that may not allocate device memory would use it: it must return what the
allocating device entry point returns, on two calls in a row over the same shared scratch."""

import ctypes as C
import os

import numpy as np
import pytest

from tests.golden import spec

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GRAPH = os.path.join(ROOT, "tests", "golden", "nsg_d100.glass")


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


def test_noalloc_rejects_too_many_queries(abi):
    lib, s = abi
    rc = lib.gsx_searcher_search_batch_noalloc(s, C.c_void_p(16), 65537, 10, C.c_void_p(16), C.c_void_p(16), None)
    assert rc == 1
    assert b"65536" in lib.gsx_last_error()
