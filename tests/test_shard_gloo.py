"""Multi-process (world_size 2, gloo, CPU) test of the sharded batch layout:
each rank solves its contiguous share of the systems; gathering the shares
reproduces the single-process solve exactly.  The per-rank solve here is the
oracle (CPU); on GPUs the same shard ranges feed pcrp_solve_f64."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from pcrp.shard import local_view, shard_range


def test_shard_ranges_partition_the_batch():
    for m in (0, 1, 2, 7, 256, 1001):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(m, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == m
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _worker(rank, world, port, m, n, out_path):
    import torch
    import oracle as O
    import pcrp
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    arrs = pcrp.generate(pcrp.GEN_DOMINANT, 5, m, n)
    local, ml = local_view(arrs, m, n, world, rank)
    x_local = O.pcr(*local, ml, n) if ml else np.zeros(0)
    # gather the variable-size shares on rank 0
    counts = [shard_range(m, world, r)[1] - shard_range(m, world, r)[0] for r in range(world)]
    mx = max(counts) * n
    buf = torch.zeros(mx, dtype=torch.float64)
    buf[: x_local.size] = torch.from_numpy(x_local)
    bufs = [torch.zeros(mx, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(bufs, buf)
    if rank == 0:
        x = np.concatenate([bufs[r][: counts[r] * n].numpy() for r in range(world)])
        np.save(out_path, x)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_solve_matches_single_process(tmp_path):
    import socket
    import oracle as O
    import pcrp
    m, n = 7, 300
    s = socket.socket(); s.bind(("127.0.0.1", 0)); port = s.getsockname()[1]; s.close()
    out = str(tmp_path / "x.npy")
    mp.spawn(_worker, args=(2, port, m, n, out), nprocs=2, join=True)
    x = np.load(out)
    arrs = pcrp.generate(pcrp.GEN_DOMINANT, 5, m, n)
    assert np.array_equal(x, O.pcr(*arrs, m, n))
