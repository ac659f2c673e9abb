"""The bench's N-GPU path on CPU: two `gloo` ranks split the tree population round-robin
(replicas only: no data exchange) and combine their figures, slowest-rank time and summed
work, the way `bench.py --gpus N` does under torchrun."""
import os
import socket

import pytest
import torch.multiprocessing as tmp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
COUNT, SEED = 64, 3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                            rank=rank, world_size=world)
    try:
        mine = bench.shard(bench.tree_population(COUNT, SEED), rank, world)
        n_elem = sum(size for _, size in mine)
        # rank-dependent timings: the job's time is the slowest rank's
        ms, e2e_s, n_all, alg_all = bench.combine_ranks(
            dist, "cpu", 10.0 * (rank + 1), 1.0 + rank, n_elem, 2.0 * n_elem)
        out.put((rank, [s for s, _ in mine], n_elem, ms, e2e_s, n_all, alg_all))
    finally:
        dist.destroy_process_group()


def test_two_rank_shards_and_reduction():
    world = 2
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import sys
    sys.path.insert(0, ROOT)
    import bench
    pop = bench.tree_population(COUNT, SEED)
    seeds = [s for r in res for s in r[1]]
    # disjoint shards covering the whole population, balanced to within one tree
    assert sorted(seeds) == sorted(s for s, _ in pop)
    assert abs(len(res[0][1]) - len(res[1][1])) <= 1
    total = sum(size for _, size in pop)
    for rank, _, n_elem, ms, e2e_s, n_all, alg_all in res:
        assert ms == 20.0 and e2e_s == 2.0
        assert n_all == float(total) and alg_all == 2.0 * total
    assert res[0][2] + res[1][2] == total


def test_single_process_passthrough():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.combine_ranks(None, "cpu", 5.0, 2.0, 7, 9.0) == (5.0, 2.0, 7.0, 9.0)
    assert bench.shard(list(range(5)), 0, 1) == list(range(5))
    assert bench.shard(list(range(5)), 1, 2) == [1, 3]
