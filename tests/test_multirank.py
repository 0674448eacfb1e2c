"""The host logic of multi-process runs on CPU with the gloo backend
(world size 2): partitioning of batched systems across ranks by predicted
pair bytes, and the max-over-ranks timing reduction the benchmark uses."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

import configs as cf


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, costs, out):
    import torch
    import torch.distributed as dist

    import __graft_entry__ as graft

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sh = graft.load_package_module("sharding")
        mine = sh.rank_systems(costs, rank, world)
        # every rank's list, gathered: disjoint and complete
        lists = [None] * world
        dist.all_gather_object(lists, mine)
        t = sh.max_over_ranks(1.0 + rank)
        load = float(sum(costs[k] for k in mine))
        loads = [None] * world
        dist.all_gather_object(loads, load)
        if rank == 0:
            out.put((lists, t, loads))
    finally:
        dist.destroy_process_group()


def test_partition_two_ranks_gloo():
    rng = np.random.default_rng(0)
    nat = np.exp(rng.uniform(np.log(8), np.log(4096), 400)).astype(int)
    costs = [float(n) ** 1.0 * rng.uniform(0.5, 1.5) for n in nat]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    lists, t, loads = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    flat = sorted(lists[0] + lists[1])
    assert flat == list(range(len(costs)))
    assert not set(lists[0]) & set(lists[1])
    assert t == 2.0  # max over ranks
    assert max(loads) / min(loads) < 1.02  # balanced


def test_predicted_pairs_matches_uniform_density():
    import __graft_entry__ as graft

    sh = graft.load_package_module("sharding")
    X, C, L = cf.rand_config(10000, seed=0)
    # 4/3 pi rc^3 rho N = 26,180 * 10 for rc = 5, rho = 0.05
    assert abs(sh.predicted_pairs(10000, C, 5.0) - 261799) < 1
    parts = sh.partition([5.0, 4.0, 3.0, 3.0, 2.0, 2.0, 1.0], 3)
    assert sorted(sum(parts, [])) == list(range(7))
