"""The benchmark's host-side helpers (CPU): the device-overlap count of the
serving run, the algorithmic bytes of a launch, and the DRAM-traffic lookup
that fills each bench line's roofline.traffic from profiles/dram_traffic.txt
(every workload, batch and layout key the bench asks for must be there)."""
import numpy as np

import bench


def _iv(start_us, end_us, stream):
    return {"start_ns": start_us * 1000, "end_ns": end_us * 1000, "stream": stream}


def test_device_overlap_counts_pairs_across_streams():
    times = [_iv(0, 100, 0), _iv(50, 150, 1), _iv(120, 130, 0), _iv(200, 300, 1), _iv(250, 260, 1)]
    d = bench._device_overlap(times)
    # (0-100, 50-150) and (50-150, 120-130) overlap on different streams;
    # (200-300, 250-260) overlap on the same stream and do not count
    assert d["overlapping_pairs"] == 2
    assert d["batches"] == 5
    # busy: 0..150 and 200..300 us; two or more: 50..100, 120..130, 250..260 us
    assert d["busy_ms"] == 0.25
    assert d["two_or_more_kernels_ms"] == 0.07


def test_device_overlap_of_nothing():
    d = bench._device_overlap([])
    assert d["overlapping_pairs"] == 0 and d["busy_ms"] == 0


def test_algorithmic_bytes_per_layout():
    nf = np.array([10, 20], np.uint32)
    pf = np.array([3, 1], np.uint32)
    # closest hit with prev_hit: ray + hit + prev per ray, nodes and records
    b = bench.algorithmic_bytes(nf, pf, 0, True, 0)
    assert b == 2 * (32 + 16 + 4) + 64 * 30 + 48 * 4
    # any hit, BVH4 nodes
    assert bench.algorithmic_bytes(nf, pf, 1, False, 1) == 2 * (32 + 4) + 128 * 30 + 48 * 4


def test_traffic_lookup_has_every_key_the_bench_uses():
    keys = [("sphere_1m_1080p_primary_bounce_shadow", b, 0) for b in ("primary", "bounce", "shadow")]
    keys += [("random_1m_tris_4m_incoherent_rays", "incoherent", 0),
             ("random_2m_tris_4m_incoherent_rays", "incoherent", 0),
             ("gbuffer_sphere_1m_1080p", "gbuffer", 0),
             ("shadowmask_sphere_1m_1080p_1_sample", "pass", 0),
             ("mixed_1m_tris_64k_spheres_64k_cubes_4_planes_4m_incoherent", "mixed", 0),
             ("dynamic_sphere_1m_refit_1080p_primary", "frame", 0),
             ("batch_64_scenes_1k_512k_tris_4k_2m_rays", "batch", 0)]
    for w, b, layout in keys:
        t = bench.traffic_from_profiles(w, b, layout)
        assert isinstance(t, int) and t > 0, (w, b)
    # a layout without a capture has no traffic figure (null in the line)
    assert bench.traffic_from_profiles("gbuffer_sphere_1m_1080p", "gbuffer", 2) is None
