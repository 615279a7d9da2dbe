"""Replica runs of the benchmark (one process per GPU, no data-path
collective): the timing reduction and barrier that bench.py uses across ranks,
run as two gloo ranks on the CPU.  A fit does not shard across GPUs in this
build; N GPUs run N independent replicas of the same fit and the reported
time is the maximum over ranks."""
import json
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank's "fit time" differs; every rank must see the slowest
        t = bench.max_over_ranks(10.0 + 3.0 * rank, world)
        bench.barrier(world)
        # reference arm: rank 0 alone runs it; the others return at once
        args = bench.parse(["--impl", "reference"])
        silent = bench.run_reference(args, world, rank) is None if rank != 0 else True
        out_q.put((rank, t, silent))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_silent_reference_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in res] == [0, 1]
    assert all(t == 13.0 for _, t, _ in res)
    assert all(s for _, _, s in res)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(4.5, 1) == 4.5
    bench.barrier(1)
    json.dumps({"ok": True})
