"""Multi-process ensemble sharding on CPU (gloo, world_size 2).

- Every system is owned by exactly one rank, and the ranks' body totals stay
  within the largest system of each other.
- Each rank steps its own shard of a small ensemble (the oracle's CPU
  restatement of the reference's step, BarnesHutParticleSystem.cpp:301-347,
  on each system) and the per-system FP64 energy and momentum are gathered
  once at the end: they equal a single-rank run system by system (states bit
  for bit; FP64 sums to 1e-12, since the oracle's OpenMP reductions may add in
  another order)."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from stellarsolver_gb300 import models, sharding


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = sharding.shard_of(sizes, world, rank)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    load = sum(int(sizes[i]) for i in mine)
    loads = [None] * world
    dist.all_gather_object(loads, load)
    if rank == 0:
        q.put((gathered, loads))
    dist.destroy_process_group()


def test_two_ranks_partition_the_ensemble():
    sizes = models.ensemble_sizes(256)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, list(map(int, sizes)), q), nprocs=2, join=True,
                       start_method="spawn")
    gathered, loads = q.get(timeout=60)
    allsys = sorted(i for part in gathered for i in part)
    assert allsys == list(range(len(sizes)))
    assert abs(loads[0] - loads[1]) <= int(np.max(sizes))


SMALL = dict(count=8, lo=1 << 8, hi=1 << 11)
STEPS = 3
EPS2, DT = 1e-4, 1e-4


def _oracle_backend():
    """load / step / diagnostics over the oracle's CPU step, one system at a time."""
    import pyoracle as po

    sizes = models.ensemble_sizes(**SMALL)

    def load(indices):
        systems = models.ensemble(sizes, indices=indices)
        return {"idx": list(indices), "st": [list(sy[:4]) + [sy[4]] for sy in systems]}

    def step(h, steps):
        for st in h["st"]:
            for _ in range(steps):
                st[:4] = po.step_ref(*st[:4], st[4], 0.5, EPS2, DT, 1.0)[:4]

    def diagnostics(h):
        rows = []
        for x, y, vx, vy, m in h["st"]:
            rows.append(list(po.energy_f64(x, y, vx, vy, m, EPS2)) +
                        [float(np.sum(x.astype(np.float64))), float(np.sum(y.astype(np.float64)))])
        return rows

    return sizes, load, step, diagnostics


def _stepping_worker(rank, world, port, q):
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sizes, load, step, diag = _oracle_backend()
    rows = sharding.run_sharded(sizes, world, rank, load, step, diag, STEPS,
                                all_gather_object=dist.all_gather_object)
    q.put((rank, sharding.shard_of(sizes, world, rank), rows))
    dist.destroy_process_group()


def test_two_ranks_step_their_shards_and_gather(oracle):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    mp.start_processes(_stepping_worker, args=(2, port, q), nprocs=2, join=True,
                       start_method="spawn")
    got = {}
    for _ in range(2):
        rank, mine, rows = q.get(timeout=120)
        got[rank] = (mine, rows)
    sizes, load, step, diag = _oracle_backend()
    single = sharding.run_sharded(sizes, 1, 0, load, step, diag, STEPS)
    assert got[0][0] and got[1][0]  # both ranks own systems
    for r in (0, 1):
        rows = got[r][1]
        assert rows.shape == single.shape == (len(sizes), 6)
        # positions (sums of the stepped float arrays) bit for bit, FP64 sums to 1e-12
        assert np.array_equal(rows[:, 4:], single[:, 4:])
        scale = np.abs(single[:, :2]).max(axis=1, keepdims=True)  # |KE|, |PE| per system
        assert np.all(np.abs(rows[:, :4] - single[:, :4]) <= 1e-12 * scale)


def test_single_rank_owns_everything():
    sizes = [5, 1, 7]
    assert sharding.shard_systems(sizes, 1) == [[0, 1, 2]]
