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


_SOLVE_SPECS = [(900, 8.0, 2.0, 1), (1400, 11.0, 2.6, 2), (700, 6.0, 1.9, 3), (1100, 9.5, 2.3, 4)]
_SOLVE_ITERS = 60


def _solve_case(k):
    """One ramp of _SOLVE_SPECS by the oracle's LU-SGS (inviscid, FP64)."""
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    cells, angle, mach, seed = _SOLVE_SPECS[k]
    m = mg.wedge(cells, angle, seed=seed)
    om = po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                             m["n_cells"])
    prm = po.params_ext(1, 2, limiter=1, quirks=0, inlet_q=mg.freestream(mach))
    col, _ = po.greedy_colors(om)
    q, hist = po.lusgs_iterate(om, prm, mg.freestream(mach, om.n_cells), col, _SOLVE_ITERS,
                               cfl0=50.0, cfl_max=100.0, omega=1.2, freeze_tol=0.1)
    return q, hist


def _solve_rank_main(rank, ws, port, out):
    import torch.distributed as dist
    from mstcfd.batch import partition_cases
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sizes = [s[0] for s in _SOLVE_SPECS]
    mine = partition_cases(sizes, ws)[rank]
    local = {k: _solve_case(k) for k in mine}
    gathered = [None] * ws
    # the only exchange: the final per-case results, gathered once at the end
    dist.all_gather_object(gathered, local)
    if rank == 0:
        out["all"] = {k: v for part in gathered for k, v in part.items()}
    dist.destroy_process_group()


def test_two_rank_gloo_ranks_solve_their_shares():
    """Each of two CPU ranks solves its share of a batch (the oracle's
    implicit iterations standing in for the GPU batch); the gathered
    results equal the single-rank solves bit for bit, because cases never
    interact."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_solve_rank_main, args=(2, _free_port(), out), nprocs=2,
                       start_method="spawn", join=True)
    got = out["all"]
    assert sorted(got) == list(range(len(_SOLVE_SPECS)))
    for k in range(len(_SOLVE_SPECS)):
        q, hist = _solve_case(k)
        assert np.array_equal(got[k][0], q), k
        assert np.array_equal(got[k][1], hist), k
        assert hist[-1] < hist[0]
