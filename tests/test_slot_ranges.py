"""The serving loop's slot allocator (pyglass_gb300/csrc/gsx_ranges.h) against a plain bitmap model:
random take/give sequences never hand out a slot twice, first-fit picks the lowest range that fits,
freed neighbours merge, and `largest` is the longest free run."""

import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include "gsx_ranges.h"
// reads commands from stdin: "i n" init, "t n" take, "g s n" give, "l" largest; prints results
int main() {
    gsx::Ranges r;
    char c;
    while (std::scanf(" %c", &c) == 1) {
        int a = 0, b = 0;
        if (c == 'i') { std::scanf("%d", &a); r.init(a); }
        else if (c == 't') { std::scanf("%d", &a); std::printf("%d\n", r.take(a)); }
        else if (c == 'g') { std::scanf("%d %d", &a, &b); r.give(a, b); }
        else if (c == 'l') { std::printf("%d\n", r.largest()); }
        else if (c == 'n') { std::printf("%d\n", (int)r.free_.size()); }
    }
    return 0;
}
"""


def model_take(free, n):
    run = 0
    for i, f in enumerate(free):
        run = run + 1 if f else 0
        if run == n:
            s = i - n + 1
            free[s : s + n] = False
            return s
    return -1


def model_runs(free):
    runs, run = [], 0
    for f in list(free) + [False]:
        if f:
            run += 1
        elif run:
            runs.append(run)
            run = 0
    return runs


def test_ranges_against_bitmap_model(tmp_path):
    src = tmp_path / "ranges.cc"
    src.write_text(DRIVER)
    exe = str(tmp_path / "ranges")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "pyglass_gb300", "csrc"), str(src), "-o", exe],
                   check=True)
    rng = np.random.default_rng(9)
    cap = 1000
    free = np.ones(cap, bool)
    held = []
    cmds, expect = [f"i {cap}"], []
    for _ in range(3000):
        if held and rng.random() < 0.45:
            s, n = held.pop(int(rng.integers(0, len(held))))
            free[s : s + n] = True
            cmds.append(f"g {s} {n}")
        else:
            n = int(rng.integers(1, 120))
            s = model_take(free, n)
            cmds.append(f"t {n}")
            expect.append(s)
            if s >= 0:
                held.append((s, n))
        runs = model_runs(free)
        cmds.append("l")
        expect.append(max(runs) if runs else 0)
        cmds.append("n")
        expect.append(len(runs))  # merged: one map entry per maximal free run
    out = subprocess.run([exe], input="\n".join(cmds) + "\n", capture_output=True, text=True, check=True)
    got = [int(v) for v in out.stdout.split()]
    assert got == expect
