"""GB300-native graph search with the glass.Searcher / glass.Graph API of zilliztech/pyglass.

``from pyglass_gb300 import glass`` gives the drop-in module (Graph, Searcher, set_num_threads).
The compute path is libglass_gb300.so (hand-written sm_103a CUDA behind a C ABI, see
include/glass_gb300.h); there is no CPU fallback.
"""

__version__ = "0.1.0"
