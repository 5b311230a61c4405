"""Benchmark of the GB300 graph-search path on the 1M x 128 clustered workload.

Workload (synthetic stand-in, seeded; the reference's ann-benchmarks sets are not available):
1,000,000 x 128 base vectors from 1,024 Gaussian clusters (integers 0..255), 10,000 queries from
the same mixture, NSG graph R=32 L=50 built by the reference's CPU builder (data/clusters1m.glass,
made by oracle/build_graphs.py), searcher SQ4U + FP32 refine, k=10.  On a host without that file
both arms search the NSG R=32 L=50 graph that this package's GPU builder makes (deterministic;
the JSON line's config.graph says which graph was searched).

A step is one batched search of all 10,000 queries at the headline ef.  `value` is QPS with the
queries resident in HBM (CUDA events on the launching stream, L2 flushed by a 512 MB write
between steps); `e2e` is the same batch through the public API (Searcher.batch_search) with
host numpy buffers, copies included.  One JSON line is printed by rank 0.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--ef 128] [--impl reference]
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "QPS at recall@10>=0.95 (1M×128, SQ4U), batched/served vs plain; p50/p99 latency"
WORKLOAD = "clusters1m"
META = os.path.join(ROOT, "data", f"{WORKLOAD}.json")
SWEEP_EF = [16, 32, 64, 128]
K = 10


def args_():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--ef", type=int, default=128)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--cpu-sample", type=int, default=10000, help="queries per CPU-baseline step")
    p.add_argument("--gt-only", action="store_true", help="only the tensor-core ground truth (for ncu captures)")
    p.add_argument("--build-only", type=int, default=0, metavar="ROWS",
                   help="only the GPU NSG build of the first ROWS base rows (for ncu launch lists)")
    p.add_argument("--profile", action="store_true",
                   help="only the warm-up and timed device launches, for ncu captures (no autotuner run: the "
                        "tuning is --tuning's, else the default)")
    p.add_argument("--tuning", default=None, metavar="W,T,L,P,S",
                   help="with --profile: warps per block, table bits, lanes per row, prefetch bits, spill bits")
    p.add_argument("--case", default=None, choices=sorted(CASES),
                   help="one small case of other kernels (for ncu captures): " + "; ".join(
                       f"{k}: {v[0]}" for k, v in sorted(CASES.items())))
    return p.parse_args()


_BUILT = {}


def graph_file():
    """(path, format) of the searched graph: the reference-built file under data/, else (on a host
    without it) the same NSG R=32 L=50 built by this package's GPU builder with FP32 distances,
    saved once per process to a temporary glass file.  The GPU build is deterministic, so every
    process that falls back searches the same graph."""
    from pyglass_gb300 import datasets

    found = None if _BUILT.get("stale") else datasets.graph_file(WORKLOAD, ROOT)
    if found is not None:
        return found
    if "path" not in _BUILT:
        import tempfile

        from pyglass_gb300 import glass

        if glass.device_count() == 0:
            raise SystemExit(json.dumps({"error": f"data/{WORKLOAD}.glass missing and no GPU to build it: "
                                                  f"run python oracle/build_graphs.py {WORKLOAD}"}))
        base = datasets.WORKLOADS[WORKLOAD]["base"]()
        t = time.perf_counter()
        g = glass.Index("NSG", "L2", "FP32", 32, 50).build(base)
        _BUILT["seconds"] = time.perf_counter() - t
        path = os.path.join(tempfile.mkdtemp(), f"{WORKLOAD}_gpu_built.glass")
        g.save(path)
        _BUILT["path"] = path
    return _BUILT["path"], "glass"


def graph_source():
    """How the searched graph was made, for the JSON line."""
    if "path" in _BUILT:
        why = ("its base rows differ from this host's" if _BUILT.get("stale") else "it is absent on this host")
        return (f"NSG R=32 L=50 built by this package's GPU builder (FP32 distances, {_BUILT['seconds']:.1f} s): "
                f"the reference-built graph file was not used ({why})")
    return "NSG R=32 L=50 built by the reference's CPU builder (build quant SQ8U)"


def oracle_graph():
    """The searched graph read by the oracle's own loaders (glass or NSG format), so that the CPU
    legs never load this package's library."""
    from oracle import pyoracle

    path, fmt = graph_file()
    return pyoracle.Graph(path, fmt)


GT_FILE = os.path.join(ROOT, "data", f"{WORKLOAD}_gt.npy")


def file_ground_truth(base_checksum):
    """Exact top-100 ids of the workload's queries computed on the CPU by oracle/build_graphs.py,
    when present and made from these base rows (None otherwise)."""
    meta = json.load(open(META)) if os.path.exists(META) else {}
    if not os.path.exists(GT_FILE) or meta.get("gt_base_checksum") != base_checksum:
        return None
    return np.load(GT_FILE)


def load_workload():
    from pyglass_gb300 import datasets

    w = datasets.WORKLOADS[WORKLOAD]
    base, queries = w["base"](), w["queries"]()
    meta = json.load(open(META)) if os.path.exists(META) else {}
    if meta and datasets.checksum(base) != meta["base_checksum"]:
        # this host generates other base rows than the host that built data/'s graph: that graph
        # does not fit them, so search the GPU-built graph of these rows instead
        _BUILT["stale"] = True
        meta = {}
    return base, queries, meta


def workload_config(ef, nq):
    """The workload both arms run (the same dict on each, so their lines compare directly)."""
    return {"workload": "1,000,000 x 128 from 1,024 clusters (sigma 12, integers 0..255); NSG R=32 L=50; "
                        "10,000 queries; SQ4U + FP32 refine (reorder 15); k=10",
            "graph": graph_source(), "nq": nq, "k": K, "ef": ef, "metric": "L2", "quantizer": "SQ4U",
            "refine_quant": "FP32"}


def cpu_baseline(base, queries, ef, sample):
    """The oracle (C restatement of the reference searcher, bit-exact with it, OpenMP over all host
    cores) on the first `sample` queries, timed the way the reference's example harness times
    batch_search (examples/main.py:166-187: one warm-up, best of 5), plus its plain form (`search`,
    one query per call, one thread) on a few hundred queries.  Returns the summary, the searcher and
    the ids of the last batch."""
    import platform

    from oracle import pyoracle

    pyoracle.build(ref=False)
    s = pyoracle.Searcher(oracle_graph(), base, "L2", "SQ4U", "FP32")
    s.set_ef(ef)
    q = queries[:sample]
    s.batch_search(q, K)  # warm-up
    best = 1e30
    for _ in range(5):
        t = time.perf_counter()
        ids, _ = s.batch_search(q, K)
        best = min(best, time.perf_counter() - t)
    n_plain = min(200, sample)
    t = time.perf_counter()
    for i in range(n_plain):
        s.search(q[i], K)
    plain_qps = n_plain / (time.perf_counter() - t)
    cores = os.cpu_count() or 1
    return {"value": sample / best, "unit": "QPS", "cores": cores, "kind": "port", "host": platform.machine(),
            "sample": f"{sample} of the 10,000 queries at ef={ef}, one warm-up then best of 5, {cores} OpenMP threads",
            "plain_single_thread_qps": plain_qps,
            "port_vs_reference": "on x86 (8 cores, same workload, ef=128, interleaved runs) the port runs at "
                                 "0.58-0.75x the compiled reference's batch QPS (37-47k vs 62-64k); the reference "
                                 "sources are not on this host, so it cannot be compiled here",
            "plain_sample": f"search() on the first {n_plain} queries, one per call, one thread"}, s, ids


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region: the sampler
    starts before the region (the region begins once its first sample has arrived) and only the
    samples taken inside the region are summarised."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 20

    def __init__(self, dev):
        self.dev = dev
        self.p = None
        self.rows = []
        self.t0 = self.t1 = None

    def _read(self):
        for line in self.p.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                self.rows.append((time.perf_counter(), f))

    def __enter__(self):
        import threading

        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, bufsize=1)
        except OSError:
            self.p = None
        if self.p is not None:
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
            deadline = time.perf_counter() + 10
            while not self.rows and time.perf_counter() < deadline and self.p.poll() is None:
                time.sleep(0.005)
        self.t0 = time.perf_counter()
        return self

    def __exit__(self, *a):
        self.t1 = time.perf_counter()
        if self.p is None:
            return
        time.sleep(2 * self.PERIOD_MS / 1000)
        self.p.terminate()
        try:
            self.p.wait(timeout=10)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.th.join(timeout=5)

    def summary(self):
        inside = [f for t, f in self.rows if self.t0 is not None and self.t0 <= t <= self.t1 + self.PERIOD_MS / 1000]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        num = lambda x: x.replace(".", "", 1).isdigit()
        sm = [float(r[1]) for r in inside if num(r[1])]
        mx = [float(r[2]) for r in inside if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside), "region_s": round(self.t1 - self.t0, 3)}


def ground_truth(torch, glass, base_t, q_t, k):
    """Exact k nearest neighbours from the tensor-core kernel (gsx_knn_exact), spot-checked against
    a float64 CPU recompute on 20 queries."""
    ids = torch.empty((q_t.shape[0], k), dtype=torch.int32, device="cuda")
    dis = torch.empty((q_t.shape[0], k), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t = time.perf_counter()
    exact = glass.knn_exact(base_t.data_ptr(), base_t.shape[0], base_t.shape[1], q_t.data_ptr(), q_t.shape[0], k,
                            False, ids.data_ptr(), dis.data_ptr())
    secs = time.perf_counter() - t
    flops = 2.0 * q_t.shape[0] * base_t.shape[0] * 128 * (1 if exact else 3)
    gt, gd = ids.cpu().numpy(), dis.cpu().numpy()
    b = base_t.cpu().numpy().astype(np.float64)
    q = q_t[:20].cpu().numpy().astype(np.float64)
    ok = True
    for i in range(20):
        d = ((b - q[i]) ** 2).sum(1)
        kth = np.partition(d, k - 1)[k - 1]
        ok &= bool(np.allclose(np.sort(d[gt[i]]), np.sort(d)[:k]) and d[gt[i]].max() <= kth)
    return gt, {"kernel": "tcgen05 bf16 (single exact pass)" if exact else "tcgen05 bf16 hi/lo split",
                "cpu_recheck_20_queries": ok, "seconds_incl_setup_and_rescore": secs,
                "tensor_tflops_incl_setup": flops / secs / 1e12}


def recall(ids, gt):
    return float(np.mean([len(np.intersect1d(ids[i, :K], gt[i, :K])) for i in range(ids.shape[0])])) / K


def serving_leg(glass, s, queries):
    """Continuous batching under an open-loop Poisson stream: requests of 1..256 queries
    (log-uniform), k in {10, 100}, ef in {32, 64, 128, 256}; the saturation throughput is measured
    with a burst, then p50/p99 request latency at 10%, 50% and 90% of it."""
    srv = glass.Server(s, capacity=65536, kmax=100, efmax=256, streams=16)
    ks, efs = [10, 100], [32, 64, 128, 256]
    mean_size = 256 / np.log(257) - 0.5
    lat, sz, wall = srv.drive_poisson(queries, 2000, 1e7, 1, 256, ks, efs, 7)  # burst: saturation
    sat_qps = float(sz.sum() / wall)
    points = []
    for frac in (0.1, 0.5, 0.9):
        qps = frac * sat_qps
        rate = qps / mean_size
        n = int(min(30000, max(300, rate * 2.5)))
        lat, sz, wall = srv.drive_poisson(queries, n, rate, 1, 256, ks, efs, 11)
        points.append({"offered_qps": qps, "achieved_qps": float(sz.sum() / wall), "requests": n,
                       "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))})
    srv.close()
    return {"saturation_qps": sat_qps, "mix": "1..256 queries/request (log-uniform), k {10,100}, ef {32,64,128,256}",
            "points": points, "p50_ms": points[1]["p50_ms"], "p99_ms": points[1]["p99_ms"],
            "at": "50% of saturation"}


def graph_build_leg(glass, base, queries, gt, meta, ef, ref_recall):
    """NSG build of the workload's base set on the GPU (R 32, L 50, as the reference built the
    searched graph), then the same SQ4U + FP32 search on it at the headline ef."""
    idx = glass.Index("NSG", "L2", "FP32", 32, 50)
    t = time.perf_counter()
    g = idx.build(base)
    wall = time.perf_counter() - t
    s2 = glass.Searcher(g, base, "L2", "SQ4U", "FP32")
    s2.set_ef(ef)
    ids, _ = s2.batch_search(queries, K)
    out = {"index": "NSG R=32 L=50, FP32 distances, exact 64-NN graph", "seconds": wall, "stages": idx.stages(),
           "recall@10_at_ef": {"ef": ef, "gpu_built": recall(ids, gt), "searched_graph": ref_recall},
           "reference_cpu_seconds": meta.get("build_seconds"),
           "reference_cpu_note": "the reference's NSG builder (NN-Descent, SQ8U distances) on 8 x86 cores"}
    del s2, g
    return out


def graph_replay_leg(torch, s, dq, nq, steps, stream, flush, want_ids):
    """The headline batch captured once as a CUDA graph (Searcher.capture_batch_device) and
    replayed `steps` times on the bench stream: QPS from CUDA events (L2 flushed between replays)
    and whether the ids equal those of the direct launches."""
    try:
        ids = torch.empty((nq, K), dtype=torch.int32, device="cuda")
        dis = torch.empty((nq, K), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        g = s.capture_batch_device(dq.data_ptr(), nq, K, ids.data_ptr(), dis.data_ptr(), kmax=K)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            g.launch(stream.cuda_stream)
            e1.record(stream)
        torch.cuda.synchronize()
        ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in ev)
        out = {"qps": nq / (ms / 1000.0), "ms_per_replay": ms, "replays": steps,
               "overflowed_queries": g.overflow_count(),
               "same_ids_as_direct_launches": bool(np.array_equal(ids.cpu().numpy(), want_ids))}
        g.close()
        return out
    except Exception as e:  # reported, not fatal: the headline numbers above stand on their own
        return {"error": str(e)[:300]}


def replica_throughput(local_seconds, nq, steps, world, dist=None, device="cpu"):
    """Whole-job QPS of `world` replicas that each searched nq queries per step: the slowest
    rank's time bounds the job (max over ranks; no data is exchanged)."""
    total = float(local_seconds)
    if dist is not None and world > 1:
        import torch

        t = torch.tensor([total], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total = float(t.item())
    return world * nq * steps / total, total


def measured_peak():
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(mp["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(ef):
    """DRAM bytes (read + write) of one search launch from the committed ncu summary of this
    workload, or None when there is none for this ef."""
    import re

    path = os.path.join(ROOT, "profiles", f"search_sq4u_{WORKLOAD}_ef{ef}.md")
    if not os.path.exists(path):
        return None
    m = re.search(r"traffic per launch[^|]*\|\s*([0-9.]+) GB", open(path).read())
    return float(m.group(1)) * 1e9 if m else None


def run_reference(a):
    """The reference's CPU searcher on the same workload and config as the GPU arm: the oracle (the
    reference's search restated in C, bit-exact with it), all host cores, every step one
    batch_search of all 10,000 queries at the headline ef.  It loads only the oracle's libraries."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from pyglass_gb300 import datasets

    if datasets.graph_file(WORKLOAD, ROOT) is None:
        print(json.dumps({"impl": "reference", "unavailable": f"data/{WORKLOAD} graph absent: the reference-built "
                          f"graph is made by oracle/build_graphs.py on a host with the reference checkout"}))
        return
    base, queries, meta = load_workload()
    if _BUILT.get("stale"):
        print(json.dumps({"impl": "reference", "unavailable": "this host generates other base rows than the "
                          "host that built data/'s graph"}))
        return
    nq = queries.shape[0]
    cb, s, ids = cpu_baseline(base, queries, a.ef, nq)
    for _ in range(a.warmup):
        s.batch_search(queries, K)
    times = []
    for _ in range(a.steps):
        t = time.perf_counter()
        ids, _ = s.batch_search(queries, K)
        times.append(time.perf_counter() - t)
    ms = 1000 * statistics.mean(times)
    value = nq / (ms / 1000)
    best_of_5 = cb["value"]
    cb["value"] = value
    cb["sample"] = f"all {nq} queries per step at ef={a.ef}, {cb['cores']} OpenMP threads"
    cb["best_of_5_qps"] = best_of_5
    gt = file_ground_truth(meta.get("base_checksum"))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "QPS", "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u4+f32", "data": "synthetic", "config": workload_config(a.ef, nq),
        "recall@10": recall(ids, gt) if gt is not None else None,
        "ground_truth": "exact top-100 by brute force on the CPU (data/clusters1m_gt.npy)" if gt is not None
        else "absent on this host",
        "cpu_baseline": cb, "e2e": {"value": value, "unit": "QPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference searcher restated in C (oracle/glass_oracle.c), bit-exact with the compiled "
                "reference on x86 (ids, distances and distance counts); the reference sources are not on this "
                "host, so the reference itself cannot be compiled here"}
    print(json.dumps(line))


def run_gpu(a):
    import torch

    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from pyglass_gb300 import glass

    base, queries, meta = load_workload()
    nq, d = queries.shape
    if a.build_only:
        idx = glass.Index("NSG", "L2", "FP32", 32, 50)
        t = time.perf_counter()
        idx.build(base[: a.build_only])
        print(json.dumps({"build_only": a.build_only, "seconds": time.perf_counter() - t, "stages": idx.stages()}))
        return
    if a.gt_only:
        bt = torch.from_numpy(base).cuda()
        qt = torch.from_numpy(queries).cuda()
        for _ in range(2):
            gt, info = ground_truth(torch, glass, bt, qt, K)
        print(json.dumps({"gt_only": True, **info}))
        return
    # index load: the graph file into the device row layout's host form, then the searcher's SetData
    # (base rows up, calibration, encoding, refine store), each timed on its own
    gpath = graph_file()
    torch.cuda.synchronize()
    t = time.perf_counter()
    graph = glass.Graph(*gpath)
    t_graph = time.perf_counter() - t
    t = time.perf_counter()
    s = glass.Searcher(graph, base, "L2", "SQ4U", "FP32", device=local)
    torch.cuda.synchronize()
    index_load = {"graph_file": os.path.basename(gpath[0]), "graph_read_s": t_graph,
                  "set_data_s": time.perf_counter() - t,
                  "note": "graph file parsed into -1-padded rows on the host; SetData uploads the graph and the "
                          "fp32 rows and calibrates and encodes on the device"}
    s.set_ef(a.ef)
    s.batch_search(queries, K)  # sizes the visited table from this workload's visit counts
    if not a.profile:
        s.optimize()
    elif a.tuning:
        s.set_tuning(*[int(x) for x in a.tuning.split(",")])
    tuning = s.get_tuning()
    # a stream of our own: the legacy default stream has handle 0, which the C ABI reads as
    # "the searcher's stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dq = torch.from_numpy(queries).cuda()
    ids = torch.empty((nq, K), dtype=torch.int32, device="cuda")
    dis = torch.empty((nq, K), dtype=torch.float32, device="cuda")
    cmps = torch.empty(nq, dtype=torch.int32, device="cuda")
    exps = torch.empty(nq, dtype=torch.int32, device="cuda")
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 512 MB > L2

    def launch():
        s.batch_search_device(dq.data_ptr(), nq, K, ids.data_ptr(), dis.data_ptr(), cmps=cmps.data_ptr(),
                              expansions=exps.data_ptr(), kmax=K, stream=stream.cuda_stream)

    for _ in range(a.warmup):
        flush.zero_()
        launch()
    torch.cuda.synchronize()
    assert s.overflow_count() == 0
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            launch()
            e1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in ev]
    if a.profile:
        print(json.dumps({"profile": True, "ef": a.ef, "step_ms": step_ms, "tuning": tuning}))
        return
    value, total_s = replica_throughput(sum(step_ms) / 1000.0, nq, a.steps, world, dist, "cuda")
    # kernels of this package per step: the search launch, plus the two batch-order kernels
    # (order_keys, order_sort) unless the tuning turned the ordering off (prefetch bit 4); 10,000
    # queries exceed the resident warps of one launch, which is when the ordering runs
    launches_per_step = 1 + (0 if tuning["prefetch"] & 16 else 2)
    ms_per_step = 1000.0 * total_s / a.steps

    # algorithmic bytes of one launch: per query n_dist*csize + n_expand*4K + reorder_k rows of
    # the fp32 refine store + the query row + the k (id, dist) results
    c = cmps.cpu().numpy().astype(np.int64)
    x = exps.cpu().numpy().astype(np.int64)
    csize, Kdeg, reorder = 64, 32, 15
    alg_bytes = int((c * csize).sum() + (x * 4 * Kdeg).sum() + nq * (reorder * 4 * 128 + 4 * d + 8 * K))
    kern_s = statistics.mean(step_ms) / 1000.0
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / kern_s / 1e9
    traffic = profiled_traffic(a.ef)

    out_ids = ids.cpu().numpy()
    base_t = torch.from_numpy(base).cuda()
    gt, gt_info = ground_truth(torch, glass, base_t, dq, K)
    del base_t
    rec = recall(out_ids, gt)

    # ef sweep (one timed batch each)
    sweep = []
    for ef in SWEEP_EF:
        s.set_ef(ef)
        launch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.zero_()
        e0.record(stream)
        launch()
        e1.record(stream)
        torch.cuda.synchronize()
        sweep.append({"ef": ef, "qps": nq / (e0.elapsed_time(e1) / 1000), "recall@10": recall(ids.cpu().numpy(), gt),
                      "avg_dist_cmps": float(cmps.float().mean().item())})
    s.set_ef(a.ef)

    # the same search over 100,000 queries (the 10,000 repeated ten times) in one launch: about twenty
    # queries per resident warp, so the steady state shows apart from the 10,000-query batch's tail
    rep = 10
    dq_w = dq.repeat(rep, 1)
    nw = dq_w.shape[0]
    ids_w = torch.empty((nw, K), dtype=torch.int32, device="cuda")
    dis_w = torch.empty((nw, K), dtype=torch.float32, device="cuda")
    cm_w = torch.empty(nw, dtype=torch.int32, device="cuda")
    ex_w = torch.empty(nw, dtype=torch.int32, device="cuda")

    def launch_w():
        s.batch_search_device(dq_w.data_ptr(), nw, K, ids_w.data_ptr(), dis_w.data_ptr(), cmps=cm_w.data_ptr(),
                              expansions=ex_w.data_ptr(), kmax=K, stream=stream.cuda_stream)

    launch_w()
    w_ms = []
    for _ in range(3):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        launch_w()
        e1.record(stream)
        torch.cuda.synchronize()
        w_ms.append(e0.elapsed_time(e1))
    cw = cm_w.cpu().numpy().astype(np.int64)
    xw = ex_w.cpu().numpy().astype(np.int64)
    bytes_w = int((cw * csize).sum() + (xw * 4 * Kdeg).sum() + nw * (reorder * 4 * 128 + 4 * d + 8 * K))
    ach_w = bytes_w / (statistics.mean(w_ms) / 1000.0) / 1e9
    multiwave = {"nq": nw, "ms": statistics.mean(w_ms), "qps": nw / (statistics.mean(w_ms) / 1000.0),
                 "roofline_frac": ach_w / peak, "achieved_gbs": ach_w,
                 "same_ids_as_headline": bool(np.array_equal(ids_w.cpu().numpy()[:nq], out_ids)),
                 "overflowed_queries": s.overflow_count()}
    del dq_w, ids_w, dis_w, cm_w, ex_w

    # e2e: the public API with host buffers (copies in the timed region)
    for _ in range(2):
        s.batch_search(queries, K)
    e2e_t = []
    for _ in range(max(3, a.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        s.batch_search(queries, K)
        e2e_t.append(time.perf_counter() - t)
    e2e = {"value": nq / statistics.mean(e2e_t), "unit": "QPS", "h2d_bytes_per_step": nq * d * 4,
           "d2h_bytes_per_step": nq * K * 8 + nq * 4 + 4}

    # plain per-query GPU form: one search call per query
    lat = []
    for i in range(200):
        t = time.perf_counter()
        s.search(queries[i], K)
        lat.append(time.perf_counter() - t)
    lat_ms = np.array(lat[20:]) * 1000
    # the same queries' device time alone: one single-query launch each, CUDA events around it
    # (at k=10 and ef >= 15 the single-query pool and expansion limit equal the batch form's)
    dev_ms = []
    ids1 = torch.empty((1, K), dtype=torch.int32, device="cuda")
    dis1 = torch.empty((1, K), dtype=torch.float32, device="cuda")
    for i in range(200):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.batch_search_device(dq[i:i + 1].data_ptr(), 1, K, ids1.data_ptr(), dis1.data_ptr(), kmax=K,
                              stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        dev_ms.append(e0.elapsed_time(e1))
    dev_ms = np.array(dev_ms[20:])
    plain = {"qps": 1000.0 / float(lat_ms.mean()), "p50_ms": float(np.percentile(lat_ms, 50)),
             "p99_ms": float(np.percentile(lat_ms, 99)), "queries": int(lat_ms.size),
             "device_p50_ms": float(np.percentile(dev_ms, 50)), "device_p99_ms": float(np.percentile(dev_ms, 99)),
             "note": "qps and p50/p99 are per search() call from Python (host round trip included); device_* is "
                     "the single-query launch alone, timed with CUDA events"}

    serving = serving_leg(glass, s, queries)
    build = graph_build_leg(glass, base, queries, gt, meta, a.ef, rec) if rank == 0 else None
    replay = graph_replay_leg(torch, s, dq, nq, max(3, a.steps // 4), stream, flush, out_ids)

    if rank == 0:
        cb, _, cpu_ids = cpu_baseline(base, queries, a.ef, min(a.cpu_sample, nq))
        n_cmp = cpu_ids.shape[0]
        overlap = float(np.mean([len(np.intersect1d(out_ids[i], cpu_ids[i])) for i in range(n_cmp)])) / K
        parity = {"queries": n_cmp, "ef": a.ef, "reference_recall@10": recall(cpu_ids, gt[:n_cmp]),
                  "gpu_recall@10": recall(out_ids[:n_cmp], gt[:n_cmp]), "topk_id_overlap": overlap,
                  "ids_identical": bool(np.array_equal(out_ids[:n_cmp], cpu_ids)),
                  "reference": "the oracle (the reference searcher restated in C, bit-exact with it)"}
        line = {
            "metric": METRIC, "value": value, "unit": "QPS", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u4+f32", "data": "synthetic", "config": workload_config(a.ef, nq),
            "timing": "CUDA events on the launching stream; a 512 MB buffer written between timed steps (L2 flush)",
            "parallelism": f"replicas x{world}", "tuning": tuning,
            "recall@10": rec, "parity_vs_reference": parity,
            "recall_target_met": rec >= 0.95,
            "recall_target_note": None if rec >= 0.95 else
            ("recall@10 >= 0.95 is not reached on this NSG graph under the reference's search semantics "
             "(the reference's own searcher returns the same ids and recall, see parity_vs_reference); "
             "the semantics are kept, so QPS is reported at the reference's operating point"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "alg_bytes_per_launch": alg_bytes, "avg_dist_cmps": float(c.mean()),
                         "avg_expansions": float(x.mean())},
            "cpu_baseline": cb, "e2e": e2e, "gpu_launches": a.steps * launches_per_step, "clocks": clk.summary(),
            "plain_per_query": plain, "batched_over_plain": value / world / plain["qps"], "sweep": sweep,
            "multiwave_100k": multiwave, "index_load": index_load,
            "ground_truth": gt_info, "serving": serving, "graph_build": build, "cuda_graph_replay": replay,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def _case_search(workload, metric, quant, refine, ef, k, nq, launches):
    """Loads a workload's graph and rows, runs `launches` timed device batches of nq queries and
    returns the mean ms per launch (CUDA events on the launching stream)."""
    import torch

    from pyglass_gb300 import datasets, glass

    found = datasets.graph_file(workload, ROOT)
    if found is None:
        raise SystemExit(json.dumps({"error": f"data/{workload} graph absent (oracle/build_graphs.py {workload})"}))
    w = datasets.WORKLOADS[workload]
    base, queries = w["base"](), w["queries"]()[:nq]
    s = glass.Searcher(glass.Graph(*found), base, metric, quant, refine)
    s.set_ef(ef)
    s.batch_search(queries, k)
    stream = torch.cuda.Stream()
    dq = torch.from_numpy(queries).cuda()
    ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dis = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    ms = []
    for _ in range(launches):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.batch_search_device(dq.data_ptr(), nq, k, ids.data_ptr(), dis.data_ptr(), kmax=k, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return {"workload": workload, "quantizer": quant, "refine": refine, "metric": metric, "ef": ef, "k": k, "nq": nq,
            "ms_per_launch": ms, "tuning": s.get_tuning()}


def _case_setdata():
    """SetData of the 1M x 128 rows for every encoder family (calibration, encoding, padding), then
    one 10,000-query batch (batch-order kernels and the search)."""
    import torch

    from pyglass_gb300 import datasets, glass

    w = datasets.WORKLOADS[WORKLOAD]
    base, queries = w["base"](), w["queries"]()
    out = {}
    for quant, refine in (("SQ4U", "FP32"), ("SQ8U", ""), ("SQ8", ""), ("FP16", ""), ("E5M2", "")):
        g = glass.Graph(*graph_file())  # a searcher takes its graph (the reference moves it in)
        torch.cuda.synchronize()
        t = time.perf_counter()
        s = glass.Searcher(g, base, "L2", quant, refine)
        torch.cuda.synchronize()
        out[f"{quant}{'+' + refine if refine else ''}_setdata_s"] = time.perf_counter() - t
        if quant == "SQ4U":
            s.set_ef(128)
            s.batch_search(queries, K)
        del s
    return out


CASES = {
    "setdata": ("SetData of 1M x 128 rows for SQ4U+FP32, SQ8U, SQ8, FP16, E5M2 and one 10,000-query SQ4U batch",
                _case_setdata),
    "lowrank-e5m2": ("100,000 x 960 low-rank rows, HNSW R=32 L=200, E5M2, ef 128, 1,000 queries",
                     lambda: _case_search("lowrank100k", "L2", "E5M2", "", 128, 10, 1000, 5)),
    "lowrank-sq8u": ("100,000 x 960 low-rank rows, HNSW R=32 L=200, SQ8U, ef 128, 1,000 queries",
                     lambda: _case_search("lowrank100k", "L2", "SQ8U", "", 128, 10, 1000, 5)),
    "sphere-sq4u-ip": ("200,000 x 768 unit rows, NSG R=48 L=100, inner product, SQ4U + FP32 refine, ef 128, "
                       "2,000 queries", lambda: _case_search("sphere200k", "IP", "SQ4U", "FP32", 128, 10, 2000, 5)),
}


def run_case(a):
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    print(json.dumps({"case": a.case, "what": CASES[a.case][0], **CASES[a.case][1]()}))


def main():
    a = args_()
    if a.case:
        run_case(a)
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gpu(a)


if __name__ == "__main__":
    main()
