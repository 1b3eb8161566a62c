"""Sharding of batched cases over GPUs (greedy size balancing, no data
exchange): the partition itself, and a two-rank gloo run on CPU in which
each rank derives its share independently and the shares cover every case
exactly once with balanced loads."""
import os
import socket

import numpy as np
import pytest


def test_partition_is_balanced_and_complete():
    from mstcfd.batch import partition_cases
    rng = np.random.default_rng(3)
    sizes = rng.integers(20000, 400000, 256)
    for n in (1, 2, 4, 8):
        parts = partition_cases(sizes, n)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = [int(sizes[p].sum()) for p in parts]
        # greedy LPT: within the largest case of the ideal share
        assert max(loads) - min(loads) <= sizes.max()
    assert partition_cases([5, 5, 5], 4)[3] == []


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, sizes, out):
    import torch
    import torch.distributed as dist
    from mstcfd.batch import partition_cases
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    mine = partition_cases(sizes, ws)[rank]
    mask = torch.zeros(len(sizes), dtype=torch.int64)
    mask[mine] = 1
    cells = torch.tensor([int(np.asarray(sizes)[mine].sum())], dtype=torch.int64)
    dist.all_reduce(mask)
    dist.all_reduce(cells)
    out[rank] = (mask.tolist(), int(cells.item()))
    dist.destroy_process_group()


def test_two_rank_gloo_shards_cover_all_cases():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sizes = [int(x) for x in np.random.default_rng(5).integers(1000, 9000, 37)]
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(2, _free_port(), sizes, out), nprocs=2,
                       start_method="spawn", join=True)
    for r in range(2):
        mask, cells = out[r]
        assert mask == [1] * len(sizes)
        assert cells == sum(sizes)
