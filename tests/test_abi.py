"""CPU checks of the C ABI: the library loads, exports every declared entry point, and its
host-side logic (graph files, argument checks, error codes) works without a GPU."""

import ctypes as C
import os
import re

import numpy as np
import pytest

from tests.helpers import write_glass

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "glass_gb300.h")


@pytest.fixture(scope="module")
def lib(glass):
    return C.CDLL(os.path.join(ROOT, "pyglass_gb300", "libglass_gb300.so"))


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"\b(gsx_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(lib):
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def _load(lib, path, fmt="glass"):
    lib.gsx_graph_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]
    h = C.c_void_p()
    rc = lib.gsx_graph_load(path.encode(), fmt.encode(), C.byref(h))
    return rc, h


def _info(lib, h):
    lib.gsx_graph_info.argtypes = [C.c_void_p] + [C.POINTER(C.c_int32)] * 4
    v = [C.c_int32() for _ in range(4)]
    assert lib.gsx_graph_info(h, *[C.byref(x) for x in v]) == 0
    return [x.value for x in v]


def _adj(lib, h, N, K):
    out = np.zeros((N, K), np.int32)
    lib.gsx_graph_adjacency.argtypes = [C.c_void_p, C.c_void_p]
    assert lib.gsx_graph_adjacency(h, out.ctypes.data) == 0
    return out


def test_glass_roundtrip_with_hnsw_levels(lib, tmp_path):
    rng = np.random.default_rng(0)
    N, K = 50, 8
    adj = rng.integers(-1, N, size=(N, K)).astype(np.int32)
    lists = [np.zeros(0, np.int32) for _ in range(N)]
    lists[3] = np.array([7, 9, -1, -1], np.int32)  # node 3 on level 1, hK = 4
    lists[7] = np.array([3, -1, -1, -1], np.int32)
    lists[9] = np.array([3, 7, -1, -1], np.int32)
    p = str(tmp_path / "a.glass")
    write_glass(p, adj, [3], hnsw=(4, 3, lists))
    rc, h = _load(lib, p)
    assert rc == 0
    assert _info(lib, h) == [N, K, 1, 1]
    np.testing.assert_array_equal(_adj(lib, h, N, K), adj)
    q = str(tmp_path / "b.glass")
    lib.gsx_graph_save.argtypes = [C.c_void_p, C.c_char_p]
    assert lib.gsx_graph_save(h, q.encode()) == 0
    assert open(p, "rb").read() == open(q, "rb").read()
    lib.gsx_graph_destroy.argtypes = [C.c_void_p]
    lib.gsx_graph_destroy(h)


def test_reference_graph_fixture_loads(lib):
    rc, h = _load(lib, os.path.join(ROOT, "tests", "golden", "hnsw_d100.glass"))
    assert rc == 0
    N, K, nep, hn = _info(lib, h)
    assert (N, K, hn) == (3000, 16, 1)


def test_nsg_and_diskann_formats(lib, tmp_path):
    rows = [[1, 2], [0], [0, 1, 3], []]
    K, ep = 3, 2
    p = str(tmp_path / "g.nsg")
    with open(p, "wb") as f:  # graph.hpp:354-379
        np.array([K, ep], np.int32).tofile(f)
        for r in rows:
            np.array([len(r)] + r, np.int32).tofile(f)
    rc, h = _load(lib, p, "nsg")
    assert rc == 0
    assert _info(lib, h)[:3] == [4, 3, 1]
    want = np.full((4, 3), -1, np.int32)
    for i, r in enumerate(rows):
        want[i, : len(r)] = r
    np.testing.assert_array_equal(_adj(lib, h, 4, 3), want)
    p2 = str(tmp_path / "g.diskann")
    body = b"".join(np.array([len(r)] + r, np.int32).tobytes() for r in rows)
    with open(p2, "wb") as f:  # graph.hpp:289-316
        np.array([24 + len(body)], np.uint64).tofile(f)
        np.array([K, ep], np.int32).tofile(f)
        np.array([0], np.uint64).tofile(f)
        f.write(body)
    rc, h2 = _load(lib, p2, "diskann")
    assert rc == 0
    np.testing.assert_array_equal(_adj(lib, h2, 4, 3), want)


def _write_hnswlib(path, rows, maxM0, ep, max_level=0, d=4):
    """An hnswlib index file as the reference's loader reads it (glass/graph.hpp:184-217): header
    fields it skips are written as zeros; each level-0 element is a 32-bit link count, maxM0
    links, the vector and its 8-byte label."""
    size_per = 4 * (maxM0 + 1) + 4 * d + 8
    with open(path, "wb") as f:
        np.array([0, len(rows), len(rows), size_per, 0, 0], np.uint64).tofile(f)
        np.array([max_level, ep], np.int32).tofile(f)
        np.array([maxM0, maxM0], np.uint64).tofile(f)  # maxM, maxM0
        f.write(bytes(24))  # M, mult, ef_construction
        for i, r in enumerate(rows):
            links = np.full(maxM0, 123456, np.int32)  # unused slots hold junk; only the count matters
            links[: len(r)] = r
            np.array([len(r)], np.int32).tofile(f)
            links.tofile(f)
            np.full(d, 0.5, np.float32).tofile(f)
            np.array([i], np.uint64).tofile(f)


def test_hnswlib_level0_format(lib, tmp_path):
    rng = np.random.default_rng(3)
    N, maxM0 = 40, 6
    rows = [list(rng.choice(N, size=int(rng.integers(0, maxM0 + 1)), replace=False).astype(int)) for _ in range(N)]
    p = str(tmp_path / "g.hnswlib")
    _write_hnswlib(p, rows, maxM0, ep=7)
    rc, h = _load(lib, p, "hnswlib")
    assert rc == 0
    assert _info(lib, h)[:3] == [N, maxM0, 1]
    want = np.full((N, maxM0), -1, np.int32)
    for i, r in enumerate(rows):
        want[i, : len(r)] = r
    np.testing.assert_array_equal(_adj(lib, h, N, maxM0), want)
    # a file with upper levels: the reference stops with "Not supported"; here it is an error code
    p2 = str(tmp_path / "multi.hnswlib")
    _write_hnswlib(p2, rows, maxM0, ep=7, max_level=2)
    rc, _ = _load(lib, p2, "hnswlib")
    assert rc == 7  # GSX_ERR_UNSUPPORTED
    # a count larger than the row holds is rejected instead of read past the row
    p3 = str(tmp_path / "bad.hnswlib")
    _write_hnswlib(p3, [[1, 2]] + rows[1:], maxM0, ep=0)
    with open(p3, "r+b") as f:
        f.seek(96)  # first element's link count
        np.array([maxM0 + 1], np.int32).tofile(f)
    rc, _ = _load(lib, p3, "hnswlib")
    assert rc == 1


def test_malformed_graphs_are_rejected(lib, tmp_path):
    p = str(tmp_path / "bad.glass")
    write_glass(p, np.array([[1, 5], [0, -1]], np.int32), [0])  # id 5 >= N
    rc, _ = _load(lib, p)
    assert rc == 1
    lib.gsx_last_error.restype = C.c_char_p
    assert b"out of range" in lib.gsx_last_error()
    rc, _ = _load(lib, str(tmp_path / "missing.glass"))
    assert rc == 5
    rc, _ = _load(lib, p, "unknown-format")
    assert rc == 1
    # an HNSW neighbour that does not exist on the level it is listed on
    p3 = str(tmp_path / "bad_hnsw.glass")
    lists = [np.zeros(0, np.int32), np.array([0, -1], np.int32)]
    write_glass(p3, np.array([[1], [0]], np.int32), [1], hnsw=(2, 1, lists))
    rc, _ = _load(lib, p3)
    assert rc == 1


def test_degree_limit(lib, tmp_path):
    p = str(tmp_path / "wide.glass")
    write_glass(p, np.zeros((2, 65), np.int32), [0])
    rc, _ = _load(lib, p)
    assert rc == 7  # GSX_ERR_UNSUPPORTED


def test_python_surface(glass):
    for name in ["Graph", "Searcher", "set_num_threads"]:
        assert hasattr(glass, name)
    g = glass.Graph(os.path.join(ROOT, "tests", "golden", "nsg_d100.glass"))
    assert g.info()[:2] == (3000, 16)
    glass.set_num_threads(4)


def test_no_device_is_an_error_not_a_fallback(glass):
    if glass.device_count() > 0:
        pytest.skip("a GPU is visible")
    g = glass.Graph(os.path.join(ROOT, "tests", "golden", "nsg_d100.glass"))
    with pytest.raises(RuntimeError, match="no CUDA device"):
        glass.Searcher(g, np.zeros((3000, 100), np.float32), "L2", "SQ8U")


def test_compact_nsg_twin_roundtrip(glass, tmp_path):
    """oracle/compact_graphs.py writes the NSG-format twin of a glass graph; the library loads it
    back to the same adjacency, and saving that gives the original glass file byte for byte."""
    from oracle import compact_graphs

    src = os.path.join(ROOT, "tests", "golden", "nsg_d100.glass")
    dst = str(tmp_path / "g.glass")
    open(dst, "wb").write(open(src, "rb").read())
    twin = compact_graphs.compact(dst)
    again = str(tmp_path / "again.glass")
    glass.Graph(twin, "nsg").save(again)
    assert open(again, "rb").read() == open(src, "rb").read()


_HOSTILE = r"""
import ctypes as C, sys
lib = C.CDLL(sys.argv[1])
lib.gsx_graph_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]
lib.gsx_graph_create.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]
h = C.c_void_p()
for path, fmt in zip(sys.argv[2::2], sys.argv[3::2]):
    print(path.rsplit("/", 1)[-1], lib.gsx_graph_load(path.encode(), fmt.encode(), C.byref(h)), flush=True)
one = (C.c_int32 * 1)(0)
print("create", lib.gsx_graph_create(one, 1 << 30, 1 << 30, one, 1, C.byref(h)), flush=True)
"""


def test_hostile_headers_are_errors_not_allocations(lib, tmp_path):
    """Header fields that claim more rows, wider rows or longer lists than the file holds are
    rejected before anything is allocated for them (a malformed file must not exhaust host memory
    or end the process)."""
    import subprocess
    import sys

    files = []

    def add(name, fmt, *arrays):
        p = str(tmp_path / name)
        with open(p, "wb") as f:
            for a in arrays:
                a.tofile(f)
        files.extend([p, fmt])

    i32, u64 = np.int32, np.uint64
    add("huge_n.glass", "glass", np.array([1, 0, 1 << 30, 48], i32))               # 200 GB of rows, 16-byte file
    add("huge_nk.glass", "glass", np.array([1, 0, 1 << 30, 1 << 30], i32))         # N*K overflows 32 bits
    add("wide.nsg", "nsg", np.array([1 << 30, 0, 1, 0], i32))                      # K = 2^30
    add("wide.diskann", "diskann", np.array([40], u64), np.array([1 << 30, 0], i32), np.array([0], u64),
        np.array([1, 0], i32))
    add("huge.hnswlib", "hnswlib", np.array([0, (1 << 31) - 1, 0, 1 << 40, 0, 0], u64), np.array([0, 0], i32),
        np.array([32, 32], u64), np.zeros(24, np.uint8))
    adj = np.array([[1], [0]], i32)
    add("huge_levels.glass", "glass", np.array([1, 0, 2, 1], i32), adj.ravel(), np.array([2, 1, 0], i32),
        np.array([1 << 30], i32))                                                  # one node claims 2^30 list entries
    lib_path = os.path.join(ROOT, "pyglass_gb300", "libglass_gb300.so")
    r = subprocess.run([sys.executable, "-c", _HOSTILE, lib_path, *files], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, f"crashed: {r.stdout[-500:]} {r.stderr[-1500:]}"
    got = dict(line.split() for line in r.stdout.splitlines())
    for name in ("huge_n.glass", "huge.hnswlib", "huge_levels.glass"):
        assert got[name] == "1", (name, got[name])      # GSX_ERR_INVALID: the file does not hold what it claims
    for name in ("huge_nk.glass", "wide.nsg", "wide.diskann"):
        assert got[name] == "7", (name, got[name])      # GSX_ERR_UNSUPPORTED: degree above 64
    assert got["create"] == "7"
