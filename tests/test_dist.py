"""Ray sharding (dist.trace_sharded: each rank traces a contiguous slice of
the rays, the slices are gathered once) and the benchmark's cross-rank timing
reduction, with two gloo ranks: on CPU with the oracle as each rank's tracer,
and (marked gpu) with the engine in both ranks."""
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


def _sharded_worker(rank, world, port, out_dir, on_gpu):
    import torch.distributed as dist

    from igx_raytracing_gb300 import scenes
    from igx_raytracing_gb300.dist import trace_sharded

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tris = scenes.random_triangles(20000, 4242)
        rays = scenes.incoherent_rays(30001, 4243)
        prev = np.arange(len(rays), dtype=np.uint32) % 20000
        if on_gpu:
            # every rank holds a replica of the scene and traces its slice on
            # the GPU (one device here: the ranks' kernels wait on nothing)
            import igx_raytracing_gb300 as igx

            with igx.Context(0) as ctx:
                scene = ctx.create_scene(tris)
                hits, b, e = trace_sharded(scene.trace_geometry, rays, prev)
                occ, _, _ = trace_sharded(scene.trace_occlusion, rays, prev)
                scene.close()
        else:
            from oracle import pyoracle

            nodes, prims = pyoracle.bvh_build(tris)
            hits, b, e = trace_sharded(lambda r, p: pyoracle.bvh_trace(0, nodes, prims, r, p), rays, prev)
            occ, _, _ = trace_sharded(lambda r, p: pyoracle.bvh_trace(0, nodes, prims, r, p, mode=1), rays, prev)
        assert (b, e) == (0, len(rays))
        np.save(os.path.join(out_dir, f"hits{rank}.npy"), hits)
        np.save(os.path.join(out_dir, f"occ{rank}.npy"), occ)
    finally:
        dist.destroy_process_group()


def _check_sharded(out_dir, world):
    from igx_raytracing_gb300 import scenes
    from oracle import pyoracle

    tris = scenes.random_triangles(20000, 4242)
    rays = scenes.incoherent_rays(30001, 4243)
    prev = np.arange(len(rays), dtype=np.uint32) % 20000
    hits, flags = pyoracle.trace_geometry(tris, rays, prev)
    occ, _ = pyoracle.trace_occlusion(tris, rays, prev)
    ok = (flags & pyoracle.EVENT_NAN_T) == 0
    for r in range(world):
        got = np.load(os.path.join(out_dir, f"hits{r}.npy"))
        assert got[ok].tobytes() == hits[ok].tobytes()  # every rank holds the whole batch
        assert np.array_equal(np.load(os.path.join(out_dir, f"occ{r}.npy"))[ok], occ[ok])


def test_two_gloo_ranks_trace_sharded_and_gather(tmp_path):
    """trace_sharded's slicing and gather on two gloo ranks, each tracing its
    slice with the oracle's CPU traversal, against the brute-force oracle."""
    import torch.multiprocessing as mp

    mp.start_processes(_sharded_worker, args=(2, _free_port(), str(tmp_path), False), nprocs=2,
                       start_method="spawn", join=True)
    _check_sharded(str(tmp_path), 2)


@pytest.mark.gpu
def test_two_ranks_trace_sharded_through_the_engine(tmp_path):
    """The same with the engine: two processes, each with its own context
    and replica of the scene on the GPU, trace their slices through the C
    ABI and gather over gloo."""
    import torch.multiprocessing as mp

    mp.start_processes(_sharded_worker, args=(2, _free_port(), str(tmp_path), True), nprocs=2,
                       start_method="spawn", join=True)
    _check_sharded(str(tmp_path), 2)
