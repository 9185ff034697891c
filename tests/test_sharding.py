"""World-level sharding across ranks (CPU): the assignment, and the two-rank host
path of bench.py (shards, barrier, max over ranks, result gathering) over gloo."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from falling_sand_engine_gb300.sharding import shard_loads, shard_worlds  # noqa: E402


@pytest.mark.parametrize("world_size", [1, 2, 3, 4, 8])
def test_shards_partition_and_balance(world_size):
    rng = np.random.default_rng(world_size)
    sides = np.arange(128, 2049, 64)
    fp = [int(rng.choice(sides)) * int(rng.choice(sides)) for _ in range(256)]
    shards = shard_worlds(fp, world_size)
    assert len(shards) == world_size
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(fp)))
    loads = shard_loads(fp, shards)
    # greedy largest-first: no rank exceeds another by more than one world
    assert max(loads) - min(loads) <= max(fp)
    # deterministic: every rank derives the same split
    assert shards == shard_worlds(list(fp), world_size)


def test_more_ranks_than_worlds():
    shards = shard_worlds([5, 3], 4)
    assert sorted(i for s in shards for i in s) == [0, 1]
    assert sum(1 for s in shards if not s) == 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world_size, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world_size)
    sizes = bench.config2_sizes(256, 1234)
    mine = shard_worlds([w * h for w, h in sizes], world_size)[rank]
    shards = bench.gather_objects(mine, world_size)
    bench.barrier(world_size)
    mx = bench.max_over_ranks(1.5 + rank, world_size)
    cells = sum(sizes[i][0] * sizes[i][1] for i in mine)
    total = sum(bench.gather_objects(cells, world_size))
    with open(os.path.join(out_dir, "rank%d.txt" % rank), "w") as f:
        f.write(repr((shards, mx, total)))
    dist.destroy_process_group()


def test_two_rank_gloo_host_path(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    import ast

    res = [ast.literal_eval(open(tmp_path / ("rank%d.txt" % r)).read()) for r in range(2)]
    sizes = __import__("bench").config2_sizes(256, 1234)
    for shards, mx, total in res:
        assert mx == 2.5
        assert sorted(shards[0] + shards[1]) == list(range(256))
        assert not set(shards[0]) & set(shards[1])
        assert total == sum(w * h for w, h in sizes)
    assert res[0] == res[1]
