"""Drop-in for the reference's ``glass`` module on the graph-search path.

Graph, Searcher and set_num_threads have the reference's signatures (python/bindings.cc:239-269);
searches run on the GPU through libglass_gb300.so.  Importing fails loudly when the native
extension is missing: there is no CPU fallback.
"""

try:
    from pyglass_gb300._glass import Graph, Searcher, Server, device_count, knn_exact, set_num_threads, version  # noqa: F401
except ImportError as e:  # pragma: no cover - exercised only on a broken install
    raise ImportError(
        "pyglass_gb300's native extension is not built; run `python -m pyglass_gb300.build` "
        f"(nvcc for sm_103a is required): {e}"
    ) from e

__all__ = ["Graph", "Searcher", "Server", "knn_exact", "set_num_threads", "device_count", "version"]
