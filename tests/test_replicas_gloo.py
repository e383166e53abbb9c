"""Multi-process host logic of the replica split (CPU, gloo, world size 2):
ranks own disjoint members and the timing reduction takes the max."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from aeolus_gb300 import workloads as W
from aeolus_gb300.replicas import max_over_ranks, member_seed_base


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        B = 3
        states, _ = W.member_states(5, B, seed=member_seed_base(rank, B))
        mine = torch.as_tensor(states.reshape(B, -1).real.copy())
        gathered = [torch.zeros_like(mine) for _ in range(world)]
        dist.all_gather(gathered, mine)
        t = max_over_ranks(10.0 + rank)
        if rank == 0:
            rows = torch.cat(gathered).numpy()
            out.put((t, len({r.tobytes() for r in rows}), rows.shape[0]))
    finally:
        dist.destroy_process_group()


def test_replica_members_disjoint_and_max_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    t, distinct, total = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert t == 11.0
    assert distinct == total == 6


def test_single_process_max_is_identity():
    assert max_over_ranks(3.5) == 3.5
    assert member_seed_base(0, 64) == 0 and member_seed_base(2, 64) == 128000
