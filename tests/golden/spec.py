"""What the golden fixtures contain; shared by the generator and the tests."""

import itertools

from pyglass_gb300 import datasets

N, D = 3000, 100          # d=100 exercises the padding of every quantizer (dalign 112 / 128)
NQ_DIST, NQ_SEARCH = 16, 60
GRAPHS = {"hnsw_d100": ("HNSW", 16, 40), "nsg_d100": ("NSG", 16, 40)}
QUANTS = [("SQ8U", "L2"), ("SQ8U", "IP"), ("SQ4U", "L2"), ("SQ4U", "IP"), ("E5M2", "L2"), ("E5M2", "IP"),
          ("FP32", "L2"), ("FP32", "IP"), ("FP16", "L2"), ("FP16", "IP"), ("BF16", "L2"), ("BF16", "IP"),
          ("SQ2U", "L2"), ("SQ2U", "IP"), ("SQ8", "L2"), ("SQ8", "IP"), ("SQ4UA", "L2"), ("SQ4UA", "IP"),
          ("SQ1", "L2"), ("SQ1", "IP")]
# (quant, metric, refine)
SEARCHERS = [("SQ8U", "L2", ""), ("SQ8U", "IP", ""), ("SQ4U", "L2", "FP32"), ("SQ4U", "IP", "FP32"),
             ("E5M2", "L2", ""), ("E5M2", "IP", ""), ("FP32", "L2", ""), ("FP32", "IP", ""), ("SQ8U", "L2", "FP32"),
             ("FP16", "L2", ""), ("FP16", "IP", ""), ("BF16", "L2", ""), ("BF16", "IP", ""),
             # make_refiner: an FP16 store; a known quantizer without a refiner; a name the map lacks (FP32)
             ("SQ4U", "L2", "FP16"), ("SQ8U", "IP", "FP16"), ("SQ4U", "L2", "BF16"), ("SQ4U", "IP", "FP64"),
             ("SQ2U", "L2", ""), ("SQ2U", "L2", "FP32"), ("SQ2U", "IP", "FP32"),
             ("SQ8", "L2", ""), ("SQ8", "IP", ""), ("SQ8", "L2", "FP32"),
             ("SQ4UA", "L2", ""), ("SQ4UA", "L2", "FP32"), ("SQ4UA", "IP", "FP32"), ("SQ1", "IP", ""),
             ("SQ1", "IP", "FP32")]  # SQ1 searchers exist for IP only (graph_searcher.hpp:362-369)
# (ef, k): includes k > ef, the case where search and batch_search differ (graph_searcher.hpp:134,152)
EFK = [(16, 10), (40, 10), (8, 20)]


def base():
    return datasets.gaussian(N, D, seed=11)


def queries():
    return datasets.gaussian(NQ_SEARCH, D, seed=11, stream=1)


# Float kernels whose rounding the reference's -Ofast build varies between its compiled copies (the
# batch loop, the single-query loop, the stand-alone computer differ by 1-2 ulp): their distances are
# checked to the floating-point tolerance (relative 1e-5); ids and distance counts stay exact.
FLOAT_TOLERANT = {("SQ8", "L2")}
# quantizer/metric pairs the reference has no searcher for (create_searcher returns null): their codes
# and distances are pinned at the quantizer level only
NO_SEARCHER = {("SQ1", "L2")}
SEARCHABLE = [qm for qm in QUANTS if qm not in NO_SEARCHER]
RTOL = 1e-5


def search_cases():
    for g, (q, m, r), (ef, k), mode in itertools.product(GRAPHS, SEARCHERS, EFK, ["batch", "single"]):
        if mode == "single" and ef != 8:
            continue
        yield (g, q, m, r, ef, k, mode)


def case_key(c):
    g, q, m, r, ef, k, mode = c
    return f"{g}/{q}/{m}/{r or '-'}/{ef}/{k}/{mode}"
