"""Multi-rank host logic on CPU: two gloo ranks (one process each) shard a
swap-test batch, evaluate their units (here the FP64 closed form stands in
for the GPU engine, which needs a device), gather the results to rank 0 and
take the step time as the maximum over ranks -- the same calls bench.py
makes with --gpus N under torchrun."""
import os
import socket

import numpy as np
import pytest

from quantumlab_gb300 import sharding
from quantumlab_gb300 import workloads as W

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, result_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ds, comps, vecs, cents = W.gaussian_mixture_vectors(count=256, seed=5)
        pool, offsets, dims, ia, ib = W.swap_test_pool(vecs, cents)
        items = list(vecs) + [m for d in range(4, 11) for m in cents[d]]
        mine = sharding.shard_units(sharding.swap_test_cost(dims[ia]), world, rank)
        vals = np.array([(1 + np.dot(items[ia[k]], items[ib[k]]) ** 2) / 2 for k in mine])
        full = sharding.gather_to_rank0(mine, vals, len(ia), world)
        t = sharding.max_over_ranks(float(rank + 1), world)
        load = float(np.sum(sharding.swap_test_cost(dims[ia[mine]])))
        loads = [None] * world
        dist.all_gather_object(loads, load)
        if rank == 0:
            np.savez(result_path, full=full, t=t, loads=np.array(loads),
                     want=np.array([(1 + np.dot(items[a], items[b]) ** 2) / 2 for a, b in zip(ia, ib)]),
                     maxcost=float(np.max(sharding.swap_test_cost(dims[ia]))))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_gather_and_time(tmp_path):
    path = str(tmp_path / "r.npz")
    mp.spawn(_rank_main, args=(2, _free_port(), path), nprocs=2, join=True)
    r = np.load(path)
    assert not np.any(np.isnan(r["full"]))              # every unit done exactly by one rank
    assert np.max(np.abs(r["full"] - r["want"])) < 1e-15
    assert r["t"] == 2.0                                 # max over ranks
    loads = r["loads"]
    assert abs(loads[0] - loads[1]) <= r["maxcost"]      # balanced to within one unit


def test_shards_partition_the_units():
    costs = np.random.default_rng(1).integers(1, 1000, size=777).astype(float)
    for world in (1, 2, 3, 8):
        parts = [sharding.shard_units(costs, world, r) for r in range(world)]
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(len(costs)))
        loads = [costs[p].sum() for p in parts]
        assert max(loads) - min(loads) <= costs.max()


@pytest.mark.parametrize("world", [2, 4])
def test_trotter_instances_shard_by_cost(world):
    """The 64 Fermi-Hubbard instances of configuration 4 are dealt to ranks by
    cost (a rank then runs its share as one Trotter batch, whatever the
    orders and step counts); the loads differ by at most one instance."""
    from quantumlab_gb300 import workloads as W
    from quantumlab_gb300.sharding import shard_units, trotter_instance_cost

    inst = W.hubbard_instances(64)
    steps = [int(round(1.0 / dt)) for _, dt, _ in inst]
    order = [o for _, _, o in inst]
    cost = trotter_instance_cost(steps, order)
    seen, loads = [], []
    for rank in range(world):
        mine = shard_units(cost, world, rank)
        loads.append(cost[mine].sum())
        seen += list(mine)
    assert sorted(seen) == list(range(64))
    assert max(loads) - min(loads) <= cost.max()


def test_trotter_cost_counts_the_exponentials():
    """Exponentials per step: 1 at order 1, 2 at order 2, 10 at order 4
    (five second-order products), 50 at order 6."""
    from quantumlab_gb300.sharding import trotter_instance_cost
    assert list(trotter_instance_cost([10, 10, 10, 10], [1, 2, 4, 6])) == [10.0, 20.0, 100.0, 500.0]
    costs = trotter_instance_cost([3, 3, 3, 3], [4, 1, 1, 1])
    parts = [sharding.shard_units(costs, 2, r) for r in range(2)]
    assert sorted(len(p) for p in parts) == [1, 3]          # the order-4 instance alone on one rank
