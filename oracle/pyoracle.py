"""ctypes access to the two CPU oracle libraries (TEST INFRASTRUCTURE ONLY).

* ``Oracle`` wraps ``_build/libglass_oracle.so``: our C restatement of the reference search path
  (``oracle/glass_oracle.c``).  It runs everywhere gcc does, including the GPU host.
* ``RefGlass`` wraps ``_ref/libglass_ref.so``: the unmodified reference compiled from its own
  headers by ``oracle/Makefile`` (only where the reference checkout exists).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this module.  The
product package never imports it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libglass_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libglass_ref.so")


def reference_dir() -> str | None:
    """The pyglass checkout the reference driver is compiled from: the GLASS_REFERENCE_DIR
    environment variable (the build entry point sets it on a host that has the checkout), or None."""
    d = os.environ.get("GLASS_REFERENCE_DIR")
    return d if d and os.path.isdir(os.path.join(d, "glass")) else None

KIND = {"FP32": 0, "FP16": 1, "BF16": 2, "E5M2": 3, "SQ8U": 4, "SQ8": 5, "SQ4U": 7, "SQ4UA": 8, "SQ2U": 11, "SQ1": 12}
METRIC = {"L2": 0, "IP": 1}
# get_refine_factor (glass/searcher/graph_searcher.hpp:227-238) for the quantizers in scope
REFINE_FACTOR = {"SQ8U": 1.5, "SQ8": 1.5, "SQ4U": 1.5, "SQ4UA": 1.5, "SQ2U": 3.0, "SQ1": 3.0, "E5M2": 1.0, "FP32": 1.0, "FP16": 1.0, "BF16": 1.0}

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(ref: bool | None = None) -> None:
    """Compiles the oracle (always) and the reference driver (when the reference is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    src = reference_dir()
    if ref is None:
        ref = src is not None
    if ref:
        if src is None:
            raise RuntimeError("the reference driver needs GLASS_REFERENCE_DIR (a pyglass checkout)")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={src}"], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


class _GoGraph(C.Structure):
    _fields_ = [
        ("N", C.c_int32), ("K", C.c_int32), ("adj", C.POINTER(C.c_int32)),
        ("nep", C.c_int32), ("eps", C.POINTER(C.c_int32)),
        ("has_hnsw", C.c_int32), ("hK", C.c_int32), ("hep", C.c_int32),
        ("levels", C.POINTER(C.c_int32)), ("loff", C.POINTER(C.c_int64)), ("lists", C.POINTER(C.c_int32)),
    ]


class _GoIndex(C.Structure):
    _fields_ = [
        ("g", C.POINTER(_GoGraph)), ("kind", C.c_int), ("metric", C.c_int), ("d", C.c_int),
        ("dalign", C.c_int), ("csize", C.c_int), ("p", C.c_float * 2), ("codes", C.c_void_p),
        ("has_refine", C.c_int), ("refine_factor", C.c_float), ("r_dalign", C.c_int), ("r_codes", C.c_void_p),
        ("r_kind", C.c_int), ("pp", C.c_void_p),
    ]


_lib = None


def _oracle_lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        lib = C.CDLL(ORACLE_SO)
        lib.go_layout.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.go_train.argtypes = [C.c_int, C.c_int, _f32p, C.c_int64, C.c_int, _f32p]
        lib.go_encode.argtypes = [C.c_int, C.c_int, _f32p, _f32p, C.c_int64, C.c_int, _u8p]
        lib.go_encode_query.argtypes = [C.c_int, C.c_int, _f32p, _f32p, C.c_int, C.c_void_p]
        lib.go_encode_query.restype = C.c_int
        lib.go_query_distances.argtypes = [C.c_int, C.c_int, _f32p, C.c_int, _f32p, C.c_int64, _u8p, _i32p,
                                           C.c_int, _f64p]
        lib.go_graph_load.argtypes = [C.c_char_p, C.POINTER(_GoGraph)]
        lib.go_graph_load_nsg.argtypes = [C.c_char_p, C.POINTER(_GoGraph)]
        lib.go_graph_free.argtypes = [C.POINTER(_GoGraph)]
        lib.go_search.argtypes = [C.POINTER(_GoIndex), _f32p, C.c_int64, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                  C.c_int, _i32p, _f32p, _i64p, C.c_int]
        lib.go_nsg_build.argtypes = [_f32p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                     C.c_int32, _i32p, _i32p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                     C.c_void_p]
        lib.go_nsg_build.restype = C.c_int
        _lib = lib
    return _lib


def layout(quant: str, d: int) -> tuple[int, int]:
    da, cs = C.c_int(), C.c_int()
    _oracle_lib().go_layout(KIND[quant], d, C.byref(da), C.byref(cs))
    return da.value, cs.value


class Quant:
    """A trained quantizer of the restatement: params + codes of the base rows."""

    def __init__(self, quant: str, metric: str, data: np.ndarray):
        lib = _oracle_lib()
        data = np.ascontiguousarray(data, dtype=np.float32)
        self.quant, self.metric = quant, metric
        self.kind, self.m = KIND[quant], METRIC[metric]
        self.n, self.d = data.shape
        self.dalign, self.csize = layout(quant, self.d)
        self.params = np.zeros(2 * self.dalign if quant == "SQ8" else 2, np.float32)
        lib.go_train(self.kind, self.m, data, self.n, self.d, self.params)
        self.codes = np.zeros((self.n, self.csize), np.uint8)
        lib.go_encode(self.kind, self.m, self.params, data, self.n, self.d, self.codes)

    def encode_queries(self, q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.d)
        width = {"SQ8U": self.csize, "SQ4U": self.csize, "SQ2U": self.csize, "SQ1": self.csize, "SQ4UA": self.dalign,
                 "SQ8": 12 * self.dalign}.get(self.quant, 4 * self.dalign)
        out = np.zeros((q.shape[0], width), np.uint8)
        for i in range(q.shape[0]):
            _oracle_lib().go_encode_query(self.kind, self.m, self.params, q[i], self.d, out[i].ctypes.data)
        return out

    def distances(self, q: np.ndarray, ids: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.d)
        ids = np.ascontiguousarray(ids, dtype=np.int32).reshape(q.shape[0], -1)
        out = np.zeros(ids.shape, np.float64)
        _oracle_lib().go_query_distances(self.kind, self.m, self.params, self.d, q, q.shape[0], self.codes, ids,
                                         ids.shape[1], out)
        return out


class Graph:
    """A graph file in the glass format (with HNSW levels) or the NSG format."""

    def __init__(self, path: str, fmt: str = "glass"):
        self._g = _GoGraph()
        load = {"glass": _oracle_lib().go_graph_load, "nsg": _oracle_lib().go_graph_load_nsg}.get(fmt)
        if load is None:
            raise ValueError(f"the oracle reads glass and nsg graph files, not {fmt!r}")
        rc = load(path.encode(), C.byref(self._g))
        if rc != 0:
            raise IOError(f"cannot load {fmt} graph {path} ({rc})")
        self.N, self.K = self._g.N, self._g.K

    def adjacency(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._g.adj, shape=(self.N, self.K)).copy()

    def __del__(self):
        if getattr(self, "_g", None) is not None and _lib is not None:
            _lib.go_graph_free(C.byref(self._g))


class Searcher:
    """The restated glass.Searcher: batch_search/search with the reference's semantics."""

    def __init__(self, graph: Graph, data: np.ndarray, metric: str, quantizer: str, refine_quant: str = ""):
        data = np.ascontiguousarray(data, dtype=np.float32)
        if quantizer == "SQ1" and metric != "IP":
            raise ValueError("SQ1 searchers exist for IP only (graph_searcher.hpp:362-369)")
        self.graph = graph
        self.q = Quant(quantizer, metric, data)
        self.ef = 32
        self._ix = _GoIndex()
        self._ix.g = C.pointer(graph._g)
        self._ix.kind, self._ix.metric, self._ix.d = self.q.kind, self.q.m, self.q.d
        self._ix.dalign, self._ix.csize = self.q.dalign, self.q.csize
        self._ix.p[0], self._ix.p[1] = float(self.q.params[0]), float(self.q.params[1])
        self._ix.codes = self.q.codes.ctypes.data
        self._ix.pp = self.q.params.ctypes.data
        self.refine = None
        # make_refiner (graph_searcher.hpp:240-254): FP16 -> FP16 store; FP32 or a name the quantizer
        # map does not know -> FP32 store; any other known quantizer name -> no refiner
        known = {"FP32", "FP16", "BF16", "E5M2", "SQ8U", "SQ8", "SQ6", "SQ4U", "SQ4UA", "SQ4", "SQ8P", "SQ1",
                 "SQ2U", "PQ8"}
        if refine_quant and (refine_quant in ("FP16", "FP32") or refine_quant not in known):
            rq = "FP16" if refine_quant == "FP16" else "FP32"
            self.refine = Quant(rq, metric, data)
            self._ix.has_refine = 1
            self._ix.refine_factor = REFINE_FACTOR[quantizer]
            self._ix.r_dalign = self.refine.dalign
            self._ix.r_codes = self.refine.codes.ctypes.data
            self._ix.r_kind = KIND[rq]
        self.last_cmps = None

    def set_ef(self, ef: int) -> None:
        self.ef = int(ef)

    def _run(self, q, k, single, ef_per_query=None, k_per_query=None, num_threads=0):
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.q.d)
        nq = q.shape[0]
        kmax = int(k if k_per_query is None else max(k, int(np.max(k_per_query))))
        ids = np.zeros((nq, kmax), np.int32)
        dis = np.zeros((nq, kmax), np.float32)
        cmps = np.zeros(nq, np.int64)
        efa = None if ef_per_query is None else np.ascontiguousarray(ef_per_query, dtype=np.int32)
        ka = None if k_per_query is None else np.ascontiguousarray(k_per_query, dtype=np.int32)
        _oracle_lib().go_search(C.byref(self._ix), q, nq, int(k), self.ef,
                                None if efa is None else efa.ctypes.data, None if ka is None else ka.ctypes.data,
                                int(single), ids, dis, cmps, int(num_threads))
        self.last_cmps = cmps
        return ids, dis

    def batch_search(self, q, k, num_threads=0, ef_per_query=None, k_per_query=None):
        return self._run(q, k, 0, ef_per_query, k_per_query, num_threads)

    def search(self, q, k):
        ids, dis = self._run(q, k, 1, num_threads=1)
        return ids[0], dis[0]

    def get_last_search_dist_cmps(self) -> float:
        return float(self.last_cmps.mean()) if self.last_cmps is not None else 0.0


def nsg_build(data: np.ndarray, R: int, L: int = 0, ssg: bool = False, knn_k: int = 64, knng=None, ep: int = -1,
              return_link: bool = False):
    """The restated NSG / SSG build (oracle/nsg_oracle.c): returns (graph N x R, entry point, kNN
    graph, nodes attached by the connectivity pass), plus the pruned forward graph of the link step
    (before reverse links) when return_link is set.  knng / ep, when given, replace the oracle's own
    kNN graph / entry point."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, d = data.shape
    k = min(knn_k, n - 1)
    kn = np.zeros((n, k), np.int32)
    kin = None
    if knng is not None:
        kin = np.ascontiguousarray(knng, dtype=np.int32)
        assert kin.shape == (n, k)
    g = np.zeros((n, R), np.int32)
    ep_out, att = C.c_int32(), C.c_int32()
    link = np.zeros((n, R), np.int32) if return_link else None
    rc = _oracle_lib().go_nsg_build(data, n, d, R, L, 1 if ssg else 0, knn_k,
                                    kin.ctypes.data if kin is not None else None, int(ep), kn, g,
                                    C.byref(ep_out), C.byref(att), link.ctypes.data if return_link else None)
    if rc != 0:
        raise RuntimeError(f"oracle NSG build failed ({rc})")
    if return_link:
        return g, ep_out.value, kn, att.value, link
    return g, ep_out.value, kn, att.value


_ref = None


def _ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError("oracle/_ref/libglass_ref.so not built (needs the reference checkout)")
        lib = C.CDLL(REF_SO)
        lib.ref_set_num_threads.argtypes = [C.c_int]
        lib.ref_build_graph.argtypes = [C.c_char_p, _f32p, C.c_int, C.c_int, C.c_char_p, C.c_char_p, C.c_int,
                                        C.c_int, C.c_char_p]
        lib.ref_build_graph.restype = C.c_double
        lib.ref_searcher_create.argtypes = [C.c_char_p, _f32p, C.c_int, C.c_int, C.c_char_p, C.c_char_p, C.c_char_p]
        lib.ref_searcher_create.restype = C.c_void_p
        lib.ref_searcher_set_ef.argtypes = [C.c_void_p, C.c_int]
        lib.ref_searcher_search.argtypes = [C.c_void_p, _f32p, C.c_int, _i32p, _f32p]
        lib.ref_searcher_search_batch.argtypes = [C.c_void_p, _f32p, C.c_int, C.c_int, _i32p, _f32p]
        lib.ref_searcher_dist_cmps.argtypes = [C.c_void_p]
        lib.ref_searcher_dist_cmps.restype = C.c_double
        lib.ref_searcher_destroy.argtypes = [C.c_void_p]
        lib.ref_nsg_link.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _i32p, C.c_int, C.c_int,
                                     _i32p]
        lib.ref_nsg_link.restype = C.c_int
        lib.ref_nsg_init.argtypes = [_f32p, C.c_int, C.c_int]
        lib.ref_nsg_init.restype = C.c_int
        lib.ref_graph_open.argtypes = [C.c_char_p, C.c_char_p]
        lib.ref_graph_open.restype = C.c_void_p
        lib.ref_graph_info.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.ref_graph_copy.argtypes = [C.c_void_p, _i32p, _i32p]
        lib.ref_graph_close.argtypes = [C.c_void_p]
        lib.ref_code_size.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        lib.ref_encode.argtypes = [C.c_char_p, C.c_char_p, _f32p, C.c_int, C.c_int, _u8p, _f32p]
        lib.ref_query_distances.argtypes = [C.c_char_p, C.c_char_p, _f32p, C.c_int, C.c_int, _f32p, C.c_int, _i32p,
                                            C.c_int, _f64p, C.c_void_p, C.c_int]
        _ref = lib
    return _ref


class RefGlass:
    """The unmodified reference (compiled here) behind a small functional API."""

    @staticmethod
    def set_num_threads(n: int) -> None:
        _ref_lib().ref_set_num_threads(int(n))

    @staticmethod
    def build_graph(index_type, data, metric, quant, R, L, path) -> float:
        data = np.ascontiguousarray(data, dtype=np.float32)
        return _ref_lib().ref_build_graph(index_type.encode(), data, data.shape[0], data.shape[1], metric.encode(),
                                          quant.encode(), int(R), int(L), path.encode())

    @staticmethod
    def nsg_link(data, R, L, ssg, knng, ep):
        """The reference NSG's per-node link step (search_on_graph + sync_prune) over a given kNN
        graph and entry point, FP32 distances: the pruned forward graph, N x R, -1 padded."""
        data = np.ascontiguousarray(data, dtype=np.float32)
        knng = np.ascontiguousarray(knng, dtype=np.int32)
        out = np.zeros((data.shape[0], R), np.int32)
        rc = _ref_lib().ref_nsg_link(data, data.shape[0], data.shape[1], int(R), int(L), 1 if ssg else 0, knng,
                                     knng.shape[1], int(ep), out)
        if rc != 0:
            raise RuntimeError("reference link step failed")
        return out

    @staticmethod
    def nsg_entry_point(data):
        """The reference NSG's entry point: the row nearest the centroid (NSG::Init)."""
        data = np.ascontiguousarray(data, dtype=np.float32)
        return int(_ref_lib().ref_nsg_init(data, data.shape[0], data.shape[1]))

    @staticmethod
    def load_graph(path, fmt="glass"):
        """(entry points, N x K adjacency) of a graph file as the reference's loader reads it."""
        lib = _ref_lib()
        h = lib.ref_graph_open(path.encode(), fmt.encode())
        n, k, nep = C.c_int(), C.c_int(), C.c_int()
        lib.ref_graph_info(h, C.byref(n), C.byref(k), C.byref(nep))
        eps = np.zeros(nep.value, np.int32)
        adj = np.zeros((n.value, k.value), np.int32)
        lib.ref_graph_copy(h, eps, adj)
        lib.ref_graph_close(h)
        return eps, adj

    @staticmethod
    def encode(quant, metric, data):
        data = np.ascontiguousarray(data, dtype=np.float32)
        lib = _ref_lib()
        cs = lib.ref_code_size(quant.encode(), metric.encode(), data.shape[1])
        codes = np.zeros((data.shape[0], cs), np.uint8)
        params = np.zeros(2 * layout(quant, data.shape[1])[0] if quant == "SQ8" else 2, np.float32)
        lib.ref_encode(quant.encode(), metric.encode(), data, data.shape[0], data.shape[1], codes, params)
        return codes, params

    @staticmethod
    def query_distances(quant, metric, data, queries, ids):
        data = np.ascontiguousarray(data, dtype=np.float32)
        queries = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, data.shape[1])
        ids = np.ascontiguousarray(ids, dtype=np.int32).reshape(queries.shape[0], -1)
        out = np.zeros(ids.shape, np.float64)
        stride = 4 * (data.shape[1] + 128)
        qc = np.zeros((queries.shape[0], stride), np.uint8)
        _ref_lib().ref_query_distances(quant.encode(), metric.encode(), data, data.shape[0], data.shape[1], queries,
                                       queries.shape[0], ids, ids.shape[1], out, qc.ctypes.data, stride)
        return out, qc

    class Searcher:
        def __init__(self, graph_path, data, metric, quantizer, refine_quant=""):
            data = np.ascontiguousarray(data, dtype=np.float32)
            self.d = data.shape[1]
            self.h = _ref_lib().ref_searcher_create(graph_path.encode(), data, data.shape[0], data.shape[1],
                                                    metric.encode(), quantizer.encode(), refine_quant.encode())
            if not self.h:
                raise RuntimeError("reference create_searcher returned null")

        def set_ef(self, ef):
            _ref_lib().ref_searcher_set_ef(self.h, int(ef))

        def search(self, q, k):
            q = np.ascontiguousarray(q, dtype=np.float32).reshape(self.d)
            ids = np.zeros(k, np.int32)
            dis = np.zeros(k, np.float32)
            _ref_lib().ref_searcher_search(self.h, q, int(k), ids, dis)
            return ids, dis

        def batch_search(self, q, k):
            q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1, self.d)
            ids = np.zeros((q.shape[0], k), np.int32)
            dis = np.zeros((q.shape[0], k), np.float32)
            _ref_lib().ref_searcher_search_batch(self.h, q, q.shape[0], int(k), ids, dis)
            return ids, dis

        def get_last_search_dist_cmps(self):
            return _ref_lib().ref_searcher_dist_cmps(self.h)

        def __del__(self):
            if getattr(self, "h", None) and _ref is not None:
                _ref.ref_searcher_destroy(self.h)
                self.h = None
