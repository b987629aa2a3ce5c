"""Sharding a batch over ranks (one process per GPU) on the CPU: the partition, and a
world-size-2 gloo run of the oracle's batch whose gathered results equal one process
running every instance."""
import json
import os
import socket

import numpy as np
import pytest

from neofiz_gb300 import scenes
from neofiz_gb300.shard import instance_cost, partition, shard


def _rods():
    rods = scenes.taylor_sweep(6, seed=31)
    for r, (nr, nz) in zip(rods, [(4, 20), (6, 30), (3, 15), (5, 25), (4, 24), (3, 18)]):
        r["nr"], r["nz"], r["t_end"] = nr, nz, 3.0e-6
    return rods


def test_partition_covers_every_instance_once_and_balances():
    costs = [7.0, 3.0, 5.0, 5.0, 1.0, 9.0, 2.0]
    parts = partition(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert partition(costs, 3) == parts                     # deterministic
    assert partition(costs, 1) == [list(range(len(costs)))]
    with pytest.raises(ValueError):
        partition(costs, 0)


def test_cost_follows_elements_and_steps():
    inst = scenes.sweep_instances(_rods())
    c = [instance_cost(x, 0.6) for x in inst]
    assert all(v > 0 for v in c)
    assert c[1] > c[2]                                       # 6x30 against 3x15


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from neofiz_gb300.shard import gather
    from oracle.oracle import OracleBatch
    rods = _rods()
    inst = scenes.sweep_instances(rods)
    mine = shard(inst, world, rank, 0.6)
    b = OracleBatch([inst[i] for i in mine], scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.run()
    steps = b.state()["steps"]
    lengths = [m.length for m in b.measure()]
    local = {i: (int(steps[j]), float(lengths[j])) for j, i in enumerate(mine)}
    full = gather(local, world)
    if rank == 0:
        with open(out, "w") as f:
            json.dump({str(k): v for k, v in full.items()}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_the_single_process_results(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from oracle.oracle import OracleBatch
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "gathered.json")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    got = json.load(open(out))
    inst = scenes.sweep_instances(_rods())
    b = OracleBatch(inst, scenes.Formulation.AXISYMMETRIC, cfl=0.6)
    b.run()
    steps = b.state()["steps"]
    lengths = [m.length for m in b.measure()]
    assert sorted(int(k) for k in got) == list(range(len(inst)))
    for k in range(len(inst)):
        assert got[str(k)] == [int(steps[k]), float(lengths[k])]
