"""Multi-rank host logic on CPU (gloo, world_size 2): the ensemble split by
systems and the whole-job timing (maximum over ranks).

Each rank builds its own slice of the seeded ensemble; the slices must be
disjoint, cover systems [0, 2n) in order, and equal the single-process
ensemble's systems bit for bit.  max_over_ranks must return the largest
rank's value on every rank.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_per_rank, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__
    rg = __graft_entry__.load_package()
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        first, count = rg.shard.ensemble_range(n_per_rank, rank, world)
        systems = rg.ic.config4(n_systems=count, n_min=16, n_max=64, first=first)
        rg.shard.barrier()
        m = rg.shard.max_over_ranks(10.0 + rank)
        sizes = torch.tensor([s.n for s in systems], dtype=torch.int64)
        gathered = [torch.zeros_like(sizes) for _ in range(world)]
        dist.all_gather(gathered, sizes)
        x0 = torch.tensor([float(s.r["x"][1]) for s in systems], dtype=torch.float64)
        gx = [torch.zeros_like(x0) for _ in range(world)]
        dist.all_gather(gx, x0)
        np.savez(os.path.join(out_dir, "rank%d.npz" % rank), first=first, count=count, m=m,
                 sizes=torch.cat(gathered).numpy(), x=torch.cat(gx).numpy())
    finally:
        dist.destroy_process_group()


def test_ensemble_split_and_max_over_ranks(tmp_path, rg):
    world, n = 2, 3
    mp.start_processes(_worker, args=(world, _free_port(), n, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    whole = rg.ic.config4(n_systems=world * n, n_min=16, n_max=64)
    for rank in range(world):
        d = np.load(tmp_path / ("rank%d.npz" % rank))
        assert int(d["first"]) == rank * n and int(d["count"]) == n
        assert float(d["m"]) == 10.0 + world - 1          # the largest rank's value on every rank
        assert list(d["sizes"]) == [s.n for s in whole]   # slices in order, disjoint, complete
        assert np.array_equal(d["x"], np.array([s.r["x"][1] for s in whole]))


def test_ensemble_range_rejects_bad_rank(rg):
    with pytest.raises(ValueError):
        rg.shard.ensemble_range(4, 2, 2)
    assert rg.shard.max_over_ranks(3.5) == 3.5   # no process group: the value itself
