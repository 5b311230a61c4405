"""Drop-in for the reference's ``glass`` module on the graph-search path.

Graph, Searcher, Index, build_graph and set_num_threads have the reference's signatures
(python/bindings.cc:231-269); searches and NSG/SSG graph builds run on the GPU through
libglass_gb300.so.  Importing fails loudly when the native
extension is missing: there is no CPU fallback.
"""

try:
    from pyglass_gb300._glass import (  # noqa: F401
        BatchGraph,
        Graph,
        Index,
        Searcher,
        Server,
        build_graph,
        device_count,
        knn_exact,
        set_num_threads,
        version,
    )
except ImportError as e:  # pragma: no cover - exercised only on a broken install
    raise ImportError(
        "pyglass_gb300's native extension is not built; run `python -m pyglass_gb300.build` "
        f"(nvcc for sm_103a is required): {e}"
    ) from e

__all__ = ["BatchGraph", "Graph", "Index", "Searcher", "Server", "build_graph", "knn_exact", "set_num_threads", "device_count",
           "version"]
