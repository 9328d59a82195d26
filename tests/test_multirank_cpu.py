"""The multi-rank host logic of bench.py on CPU with the gloo backend,
world size 2: each rank's plan holds its own spots, with no overlap
(replicas by spot, no data-path collective), and timings reduce to the
slowest rank."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        plan = bench.plan_spots("plan512", rank, 8)
        seeds = torch.tensor([b["seed"] for b in plan], dtype=torch.int64)
        assert [b["seed"] for b in plan] == bench.spot_seeds(rank, 8)
        gathered = [torch.zeros_like(seeds) for _ in range(world)]
        dist.all_gather(gathered, seeds)
        slowest = bench.max_over_ranks(10.0 * (rank + 1), dist, "cpu")
        q.put((rank, [g.tolist() for g in gathered], slowest))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_spots_and_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    seeds0, seeds1 = out[0][1]
    assert not set(seeds0) & set(seeds1)            # no spot on two ranks
    assert out[0][1] == out[1][1]                  # both ranks see the same sharding
    assert out[0][2] == out[1][2] == 20.0          # the slowest rank's time
    assert len(set(seeds0)) == 8


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.spot_seeds(0, 3) == [bench.BEAM["seed"] + i for i in range(3)]
    # the plan is reproducible and spans the batching form's ranges
    p1, p2 = bench.plan_spots("plan512", 0, 512), bench.plan_spots("plan512", 0, 512)
    assert p1 == p2
    E = [b["E0"] for b in p1]
    assert min(E) >= 70.0 and max(E) <= 230.0 and all((e - 70.0) % 2.0 == 0.0 for e in E)
    assert all(3.0 <= b["sigma_x"] <= 6.0 and -50.0 <= b["x0"] <= 50.0 for b in p1)
