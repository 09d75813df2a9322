"""Multi-rank path on CPU: two gloo ranks split a polymul batch by pairs and
all-gather the parts; the result equals the single-process result.  The
oracle stands in for each rank's GPU compute."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from yell_gb300.shard import shard_range, sharded_polymul


def test_shard_range_partitions():
    for n in (0, 1, 5, 16, 17):
        for world in (1, 2, 3, 4):
            ranges = [shard_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, a, b, log_n, out_path):
    import torch

    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    orc = oracle.Oracle("port")

    def compute(pa, pb):
        return np.stack([orc.polymul(pa[i], pb[i], log_n, 0) for i in range(pa.shape[0])]) \
            if pa.shape[0] else np.zeros((0,) + pa.shape[1:], np.uint64)

    def gather(part):
        t = torch.from_numpy(part.view(np.int64).reshape(-1))
        sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(sizes, torch.tensor([t.numel()]))
        mx = int(max(s.item() for s in sizes))
        padded = torch.zeros(mx, dtype=torch.int64)
        padded[: t.numel()] = t
        bufs = [torch.zeros(mx, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(bufs, padded)
        shape = part.shape[1:]
        return [bufs[r][: int(sizes[r].item())].numpy().view(np.uint64).reshape((-1,) + shape)
                for r in range(world)]

    full, _ = sharded_polymul(a, b, compute, rank, world, gather=gather)
    if rank == 0:
        np.save(out_path, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_polymul_matches_single(tmp_path, orc):
    from yell_gb300.inputs import uniform_polys

    log_n, pairs, L = 8, 5, 2
    ps = np.array([orc.prime(i) for i in range(L)], dtype=np.uint64)
    a = uniform_polys(21, pairs, L, log_n, ps)
    b = uniform_polys(22, pairs, L, log_n, ps)
    out = str(tmp_path / "full.npy")
    mp.start_processes(_worker, args=(2, _free_port(), a, b, log_n, out), nprocs=2,
                       start_method="spawn")
    full = np.load(out)
    want = np.stack([orc.polymul(a[i], b[i], log_n, 0) for i in range(pairs)])
    assert np.array_equal(full, want)
