"""Multi-process paths on CPU with gloo (world size 2): the ensemble's member
sharding and the benchmark's max-over-ranks timing. No GPU involved; the
data path has no collective (members are independent), so these check the
host logic a multi-GPU run relies on."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from pyphasefield_gb300.ensemble import partition_members
    rng = torch.Generator().manual_seed(0)
    sides = (torch.rand(64, generator=rng) * 896 + 128).int().tolist()
    cells = [s * s for s in sides]
    mine = partition_members(cells, world)[rank]
    # every rank computes the same split; gather to check it is a partition
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    # max-over-ranks of per-rank elapsed time (as bench.py does)
    t = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    load = torch.tensor([float(sum(cells[i] for i in mine))], dtype=torch.float64)
    loads = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(loads, load)
    if rank == 0:
        q.put((gathered, t.item(), [x.item() for x in loads], sum(cells)))
    dist.barrier()
    dist.destroy_process_group()


def test_ensemble_sharding_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered, tmax, loads, total = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    flat = sorted(i for part in gathered for i in part)
    assert flat == list(range(64))
    assert tmax == 2.0
    assert sum(loads) == total and max(loads) / min(loads) < 1.05
