"""The multi-GPU form is replicas only (queries are independent; each GPU holds the whole index and
searches its own query stream).  These CPU tests run the bench's rank logic as two gloo processes:
throughput aggregation over ranks, and the reference arm running on rank 0 alone."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = [2.0, 3.0][rank]  # seconds this replica took for its queries
    value, total = bench.replica_throughput(local, nq=1000, steps=4, world=world, dist=dist)
    dist.barrier()
    q.put((rank, value, total))
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, total in got:
        assert total == 3.0                       # max over ranks
        assert value == pytest.approx(2 * 1000 * 4 / 3.0)


def test_single_process_needs_no_process_group():
    import bench

    value, total = bench.replica_throughput(2.0, nq=500, steps=2, world=1)
    assert (value, total) == (500.0, 2.0)


def _ref_worker(rank, world, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    ran = []
    bench.load_workload = lambda: ran.append(rank) or (_ for _ in ()).throw(SystemExit(0))
    try:
        bench.run_reference(type("A", (), {"cpu_sample": 10, "ef": 16, "warmup": 1, "steps": 1, "gpus": world})())
    except SystemExit:
        pass
    q.put((rank, ran))


def test_reference_arm_runs_on_rank0_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_ref_worker, args=(r, 2, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=60) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert got[0] == [0] and got[1] == []
