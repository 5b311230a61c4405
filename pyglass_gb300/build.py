"""Builds libglass_gb300.so (CUDA kernels + C ABI, sm_103a) and the _glass Python module in-tree.

    python -m pyglass_gb300.build        # or pyglass_gb300.build.build()

Translation units compile in parallel; outputs are skipped when newer than their sources.  The
Python module uses the pybind11 headers shipped inside the installed torch package, so no extra
dependency is needed on either host.
"""

from __future__ import annotations

import concurrent.futures as cf
import importlib.util
import os
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
INC = os.path.join(os.path.dirname(PKG), "include")
LIB = os.path.join(PKG, "libglass_gb300.so")
EXT = os.path.join(PKG, "_glass" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["search_kernel.cu", "search_fast.cu", "encode_kernel.cu", "order_kernel.cu", "calib_kernel.cu", "noalloc.cu", "knn_kernel.cu",
                "build_kernel.cu"]
HOST_SOURCES = ["gsx_api.cpp", "gsx_graph.cpp", "gsx_server.cpp", "gsx_capture.cpp"]
HEADERS = ["gsx_internal.h", "gsx_device.cuh", "gsx_host.h", "gsx_ranges.h", "search_core.cuh"]


def _newer(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _torch_include() -> str:
    spec = importlib.util.find_spec("torch")
    if spec is None or spec.origin is None:
        raise RuntimeError("torch is needed for its bundled pybind11 headers")
    return os.path.join(os.path.dirname(spec.origin), "include")


def build(verbose: bool = False) -> None:
    os.makedirs(OBJ, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INC, "glass_gb300.h")]
    jobs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        if not _newer(o, [s] + hdrs):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c", s, "-o", o])
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        if not _newer(o, [s] + hdrs):
            jobs.append([NVCC, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-x", "cu", "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 2))) as ex:
            list(ex.map(_run, jobs))
    objs = [os.path.join(OBJ, s + ".o") for s in CUDA_SOURCES + HOST_SOURCES]
    if not _newer(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lrt", "-lpthread", "-ldl"])
    bsrc = os.path.join(CSRC, "python", "bindings.cc")
    if not _newer(EXT, [bsrc, LIB, os.path.join(INC, "glass_gb300.h")]):
        py_inc = sysconfig.get_paths()["include"]
        _run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden", "-I", _torch_include(),
              "-I", py_inc, bsrc, "-o", EXT, "-L", PKG, "-lglass_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB, EXT)


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
