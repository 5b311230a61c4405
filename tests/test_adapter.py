"""The reference-side adapter (include/glass_gb300_adapter.hpp) compiles inside the reference's own
headers with the reference's flags, links against libglass_gb300.so, and drives it: a graph made
by the reference's Graph<int32_t> (HNSW levels included) goes through the C ABI, and without a GPU
the searcher's construction ends in the library's error, raised as std::runtime_error (runs where
the reference checkout exists)."""

import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MAIN = r"""
#include <cstdio>
#include <cstdlib>
#include <memory>
#include "glass_gb300_adapter.hpp"

int main() {
    glass::Graph<int32_t> g(6, 2);
    for (int i = 0; i < 6; ++i) { g.at(i, 0) = (i + 1) % 6; g.at(i, 1) = (i + 5) % 6; }
    g.eps = {0};
    // HNSW upper level: nodes 0 and 3 on level 1, linked to each other
    g.initializer = std::make_unique<glass::HNSWInitializer>(6, 1);
    g.initializer->ep = 0;
    for (int u : {0, 3}) {
        g.initializer->levels[u] = 1;
        g.initializer->lists[u] = (int *)std::malloc(sizeof(int));
        g.initializer->lists[u][0] = 3 - u;
    }
    try {
        glass::GpuGraphSearcher s(std::move(g), "L2", "SQ4U", "FP32");
        std::printf("constructed\n");
    } catch (const std::runtime_error &e) {
        std::printf("error: %s\n", e.what());
    }
    std::unique_ptr<glass::Builder> b = std::make_unique<glass::GpuNSG>(16, 0, false);
    std::printf("builder ok\n");
    return 0;
}
"""


@pytest.fixture(scope="module")
def reference_dir(oracle, glass):
    d = oracle.reference_dir()
    if d is None or not os.path.exists(os.path.join(d, "glass", "searcher", "searcher_base.hpp")):
        pytest.skip("reference checkout not available on this host")
    return d


def test_adapter_compiles_links_and_reports_errors(reference_dir, glass, tmp_path):
    src = tmp_path / "main.cc"
    src.write_text(MAIN)
    exe = str(tmp_path / "main")
    pkg = os.path.join(ROOT, "pyglass_gb300")
    cmd = ["g++", "-std=c++20", "-O1", "-march=native", "-fopenmp", "-I", reference_dir,
           "-I", os.path.join(reference_dir, "third_party", "helpa"), "-I", os.path.join(ROOT, "include"), str(src),
           "-o", exe, "-L", pkg, "-lglass_gb300", f"-Wl,-rpath,{pkg}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "builder ok" in out.stdout
    if glass.device_count() == 0:
        assert "error: " in out.stdout and "no CUDA device" in out.stdout
    else:
        assert "constructed" in out.stdout
