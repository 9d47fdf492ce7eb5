"""The N > 1 path of bench.py on CPU: two gloo ranks.

Each rank runs its own copy of the workload with its own seed (weak scaling, no collective on
the data path); at the end the job's time is the slowest rank's and the job's flips are the sum
over ranks.  The ranks here are CPU processes: only the host-side sharding and reduction run."""
import os
import socket
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    import rewl_simulator_gb300 as rg
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        seeds = [ins.seed for ins in bench.make_batch(rg, bench.rank_seed(r), device=local).instances]
        # rank-dependent per-rank figures: times 10 + r ms and 3 + r s; flips 100 (r + 1) and 7
        times, counts = bench.reduce_over_ranks([10.0 + r, 3.0 + r], [100.0 * (r + 1), 7.0])
        q.put((r, w, seeds, times, counts))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_reduce():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    seeds = [o[2] for o in out]
    assert seeds[0] != seeds[1], "each rank must run independent instances"
    for r, w, _, times, counts in out:
        assert w == world
        assert times == [10.0 + (world - 1), 3.0 + (world - 1)]          # the slowest rank
        assert counts == [sum(100.0 * (k + 1) for k in range(world)), 7.0 * world]
