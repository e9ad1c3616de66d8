"""Multi-process (gloo, world size 2, CPU) test of the batched-solve sharding: every rank computes
its share from the sizes alone; together the shares cover each subproblem exactly once and the
estimated work is balanced."""

import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _worker(rank, world, port, sizes, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from warp_gb300 import batched

        mine = batched.shard(sizes, rank, world)
        n = torch.tensor([len(mine)], dtype=torch.int64)
        counts = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(counts, n)
        m = int(max(c.item() for c in counts))
        buf = torch.full((m,), -1, dtype=torch.int64)
        buf[: len(mine)] = torch.from_numpy(mine)
        bufs = [torch.zeros(m, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(bufs, buf)
        if rank == 0:
            out.put([b[b >= 0].tolist() for b in bufs])
    finally:
        dist.destroy_process_group()


def test_shard_covers_batch_once_and_balances():
    rng = np.random.default_rng(0)
    sizes = (rng.integers(16, 129, size=4096) + 1) ** 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + int(os.getpid()) % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    parts = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    allidx = sorted(parts[0] + parts[1])
    assert allidx == list(range(len(sizes)))
    work = [float(np.sum(sizes[np.array(p)].astype(np.float64) ** 1.5)) for p in parts]
    assert abs(work[0] - work[1]) <= 0.01 * max(work)


def test_shard_single_rank_is_everything():
    from warp_gb300 import batched

    assert list(batched.shard([3, 1, 2], 0, 1)) == [0, 1, 2]
    with pytest.raises(ValueError):
        batched.shard([3, 1, 2], 2, 2)
