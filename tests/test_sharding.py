"""Multi-process ensemble sharding on CPU (gloo, world_size 2): every system
is owned by exactly one rank, and the ranks' body totals stay within the
largest system of each other."""
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


def test_single_rank_owns_everything():
    sizes = [5, 1, 7]
    assert sharding.shard_systems(sizes, 1) == [[0, 1, 2]]
