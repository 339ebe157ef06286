"""Replicas across ranks (host logic, CPU): sharding of independent requests,
max-over-ranks timing and the aggregate rate, with two gloo ranks."""
import os
import socket

import pytest


def test_shard_covers_each_item_once_and_balances(kh):
    from khronos_gb300 import configs
    from khronos_gb300.replicas import shard

    stream = configs.serving_stream(64, seed=2024)
    work = [r.work for r in stream]
    for world in (1, 2, 3, 8):
        parts = [shard(work, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(work)))
        loads = [sum(work[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(work)  # greedy bound
        assert parts == [shard(work, world, r) for r in range(world)]  # deterministic
    with pytest.raises(ValueError):
        shard(work, 2, 2)


def test_aggregate_rate(kh):
    from khronos_gb300.replicas import aggregate_rate

    assert aggregate_rate(1e9, 2.0, 4) == pytest.approx(2e9)
    with pytest.raises(ValueError):
        aggregate_rate(1.0, 0.0, 1)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    import __graft_entry__

    __graft_entry__.package()
    import torch.distributed as dist
    from khronos_gb300 import configs
    from khronos_gb300.replicas import aggregate_rate, max_over_ranks, shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        work = [r.work for r in configs.serving_stream(32, seed=7)]
        mine = shard(work, world, rank)
        dist.barrier()
        fake_seconds = 1.0 + rank  # rank r "took" 1 + r seconds
        t = max_over_ranks(fake_seconds, dist, device="cpu")
        units = sum(work[i] for i in mine)
        import torch

        u = torch.tensor([float(units)], dtype=torch.float64)
        dist.all_reduce(u)
        out.put((rank, mine, t, float(u.item()), aggregate_rate(1e6, t, world)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(kh):
    import torch.multiprocessing as mp

    world = 2
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from khronos_gb300 import configs

    work = [r.work for r in configs.serving_stream(32, seed=7)]
    owned = sorted(res[0][1] + res[1][1])
    assert owned == list(range(32)) and not set(res[0][1]) & set(res[1][1])
    assert res[0][2] == res[1][2] == 2.0  # max over ranks
    assert res[0][3] == pytest.approx(sum(work))
    assert res[0][4] == pytest.approx(2 * 1e6 / 2.0)
