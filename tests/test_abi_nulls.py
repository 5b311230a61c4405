"""Every entry point of the C ABI, called with null handles, null pointers and zero sizes, returns
an error status (or, for destroy-style calls, does nothing) instead of crashing: a C caller that
passes a bad argument gets GSX_ERR_INVALID and a message, as the header promises.  The calls run in
a child process so that a crash is reported as a failure rather than ending the test run.  It runs
on hosts without a GPU, so that no call can reach a device."""

import json
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "glass_gb300.h")

# calls that accept a null handle by design (free-style calls) or take no handle
NO_HANDLE_OK = {"gsx_batch_graph_destroy"}
VOID_OR_INFO = {"gsx_last_error", "gsx_version", "gsx_device_count", "gsx_graph_destroy", "gsx_searcher_destroy",
                "gsx_server_destroy"}


def declarations():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = []
    for ret, name, params in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(gsx_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        ret = ret.strip().split("\n")[-1].strip()
        ps = [] if params.strip() == "void" else [" ".join(p.split()) for p in params.split(",")]
        out.append((ret, name, ps))
    return out


def ctype_of(param):
    if "*" in param:
        return "p"
    t = param.rsplit(" ", 1)[0].replace("const ", "")
    return {"int": "i32", "int32_t": "i32", "uint32_t": "u32", "int64_t": "i64", "uint64_t": "u64",
            "size_t": "u64", "double": "f64", "float": "f32"}[t]


CHILD = r"""
import ctypes as C, json, sys
lib = C.CDLL(sys.argv[1])
decls = json.loads(sys.argv[2])
T = {"p": C.c_void_p, "i32": C.c_int32, "u32": C.c_uint32, "i64": C.c_int64, "u64": C.c_uint64,
     "f64": C.c_double, "f32": C.c_float}
out = {}
for ret, name, kinds in decls:
    f = getattr(lib, name)
    f.argtypes = [T[k] for k in kinds]
    f.restype = C.c_char_p if ret.startswith("const char") else (None if ret == "void" else C.c_int)
    r = f(*[None if k == "p" else 0 for k in kinds])
    out[name] = r.decode() if isinstance(r, bytes) else r
    print(name, flush=True)
print("RESULT " + json.dumps(out), flush=True)
"""


def test_null_arguments_give_error_codes(glass):
    if glass.device_count() > 0:
        import pytest

        pytest.skip("runs on hosts without a GPU, where no call can reach a device")
    decls = [(ret, name, [ctype_of(p) for p in ps]) for ret, name, ps in declarations()]
    assert len(decls) >= 40
    lib = os.path.join(ROOT, "pyglass_gb300", "libglass_gb300.so")
    r = subprocess.run([sys.executable, "-c", CHILD, lib, json.dumps(decls)], capture_output=True, text=True,
                       timeout=300)
    last = r.stdout.strip().splitlines()[-1] if r.stdout.strip() else "(none)"
    assert r.returncode == 0, f"crashed after {last!r}: {r.stderr[-2000:]}"
    res = json.loads(last[len("RESULT "):])
    for ret, name, kinds in decls:
        if name in VOID_OR_INFO or ret != "int":
            continue
        if name in NO_HANDLE_OK:
            assert res[name] == 0, name
        else:
            assert res[name] == 1, f"{name} returned {res[name]} for null arguments, not GSX_ERR_INVALID"
