"""Ray sharding and the benchmark's cross-rank timing reduction, on CPU with
two gloo ranks (no GPU)."""
import os
import socket

import numpy as np
import pytest

from igx_raytracing_gb300.dist import shard_range


def test_shard_range_partitions_exactly():
    for n in (0, 1, 7, 64, 1000003):
        for world in (1, 2, 3, 8):
            parts = [shard_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            for (a, b), (c, d) in zip(parts, parts[1:]):
                assert b == c
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from igx_raytracing_gb300 import scenes
    from igx_raytracing_gb300.dist import max_over_ranks, shard_range, sum_over_ranks
    from oracle import pyoracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tris, rays = scenes.workload_small()
        b, e = shard_range(len(rays), rank, world)
        hits, _ = pyoracle.trace_geometry(tris, rays[b:e])  # this rank's slice only
        np.save(os.path.join(out_dir, f"hits{rank}.npy"), hits)
        slowest = max_over_ranks(1.0 + rank)
        total = sum_over_ranks(e - b)
        np.save(os.path.join(out_dir, f"red{rank}.npy"), np.array([slowest, total]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_rays_and_reduce(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    from igx_raytracing_gb300 import scenes
    from oracle import pyoracle

    tris, rays = scenes.workload_small()
    whole, _ = pyoracle.trace_geometry(tris, rays)
    parts = np.concatenate([np.load(os.path.join(tmp_path, f"hits{r}.npy")) for r in range(world)])
    assert parts.tobytes() == whole.tobytes()  # disjoint slices, no exchange needed
    for r in range(world):
        slowest, total = np.load(os.path.join(tmp_path, f"red{r}.npy"))
        assert slowest == 2.0 and total == len(rays)
