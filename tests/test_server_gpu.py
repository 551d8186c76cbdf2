"""Serving loop (GPU): admission under a memory cap, continuous batching,
request slicing, paced replay, and results that equal the oracle's for a
request alone and in a mix."""
import math
import threading
import time

import numpy as np
import pytest

from conftest import bits
from igx_raytracing_gb300 import IgxrtError, Server, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _scenes(ctx, n=4, seed=0, with_tris=False):
    out, tris_of = [], []
    for s in range(n):
        tris = scenes.random_triangles(5000 + 7000 * s, 8100 + 10 * seed + s, mu=math.log(0.02))
        out.append(ctx.create_scene(tris))
        tris_of.append(tris)
    return (out, tris_of) if with_tris else out


def _oracle_check(tris, rays, prev, mode, got):
    """The served result against the brute-force oracle (the reference's
    linear loop, trace.glsl:9-98), rays with a NaN-t event left out."""
    if mode == 0:
        e, flags = pyoracle.trace_geometry(tris, rays, prev)
        ok = (flags & pyoracle.EVENT_NAN_T) == 0
        assert np.array_equal(got["prim"][ok], e["prim"][ok])
        for f in ("t", "u", "v"):
            assert np.array_equal(bits(got[f])[ok], bits(e[f])[ok])
    else:
        e, flags = pyoracle.trace_occlusion(tris, rays, prev)
        ok = (flags & pyoracle.EVENT_NAN_T) == 0
        assert np.array_equal(got[ok], e[ok])


def _requests(nscenes, nreq, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(nreq):
        sid = int(rng.integers(0, nscenes))
        n = int(np.exp(rng.uniform(math.log(1), math.log(40000))))
        rays = scenes.batch_rays(k, n)
        mode = int(rng.integers(0, 2))
        if mode == 1:
            rays["tmax"] = rng.uniform(0.01, 0.6, n).astype(np.float32)
        prev = rng.integers(0, 5000, n).astype(np.uint32) if k % 3 == 0 else None
        reqs.append((sid, rays, prev, mode))
    return reqs


def _same(a, b, mode):
    if mode == 0:
        assert np.array_equal(a["prim"], b["prim"])
        for f in ("t", "u", "v"):
            assert np.array_equal(bits(a[f]), bits(b[f]))
    else:
        assert np.array_equal(a, b)


def test_results_alone_equal_results_in_the_mix(ctx):
    sc, tris_of = _scenes(ctx, with_tris=True)
    reqs = _requests(len(sc), 60, seed=1)
    srv = Server(ctx, streams=3, max_batch_rays=200000, slice_rays=4096)
    ids = [srv.add_scene(s) for s in sc]
    alone = []
    for sid, rays, prev, mode in reqs:  # one at a time: each request in batches of its own
        t = srv.submit(ids[sid], rays, prev, mode)
        alone.append(srv.wait(t)["out"].copy())
    batches_alone = srv.stats()["batches"]
    tickets = [srv.submit(ids[sid], rays, prev, mode) for sid, rays, prev, mode in reqs]
    mixed = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == 2 * len(reqs) and st["rejected"] == 0
    assert st["batches"] - batches_alone < batches_alone  # the mixed pass was coalesced
    for (sid, rays, prev, mode), a, m in zip(reqs, alone, mixed):
        _same(a, m["out"], mode)
        _oracle_check(tris_of[sid], rays, prev, mode, a)
    assert st["p50_ms"] > 0 and st["p99_ms"] >= st["p50_ms"]


def test_admission_waits_for_memory_and_refuses_oversize(ctx):
    sc = _scenes(ctx, n=2, seed=2)
    cap = 4 << 20  # 4 MiB: room for about 80K closest-hit rays at a time
    srv = Server(ctx, memory_cap_bytes=cap, streams=2, max_batch_rays=50000)
    ids = [srv.add_scene(s) for s in sc]
    rays = scenes.incoherent_rays(30000, 77)  # 1.44 MiB of buffers per request
    tickets = [srv.submit(ids[k % 2], rays) for k in range(24)]
    outs = [srv.wait(t, timeout=60.0)["out"] for t in tickets]
    for k, o in enumerate(outs):
        _same(o, sc[k % 2].trace_geometry(rays), 0)
    st = srv.stats()
    assert st["peak_memory_bytes"] <= cap
    assert st["peak_pending"] >= 1  # requests waited for admission
    big = scenes.incoherent_rays(100000, 78)  # 4.8 MiB: can never fit
    with pytest.raises(IgxrtError):
        srv.submit(ids[0], big)
    assert srv.stats()["rejected"] == 1
    t = srv.submit(ids[0], rays[:0])  # an empty request completes at once
    assert srv.wait(t, timeout=1.0)["out"].size == 0
    srv.close()


def _overlapping_pairs(times):
    """Pairs of batches on different streams whose device intervals
    (first CTA start to last warp exit, %globaltimer) intersect."""
    pairs = 0
    t = sorted(times.tolist(), key=lambda x: x[0])
    for i in range(len(t)):
        for j in range(i + 1, len(t)):
            if t[j][0] >= t[i][1]:
                break
            if t[j][3] != t[i][3]:
                pairs += 1
    return pairs


def test_concurrent_clients_overlap_on_the_device(ctx):
    sc = _scenes(ctx, n=3, seed=3)
    srv = Server(ctx, streams=3, max_batch_rays=60000)
    ids = [srv.add_scene(s) for s in sc]
    reqs = _requests(len(sc), 90, seed=4)
    results = [None] * len(reqs)

    def client(part):
        for k in range(part, len(reqs), 3):
            sid, rays, prev, mode = reqs[k]
            t = srv.submit(ids[sid], rays, prev, mode)
            results[k] = (t, mode)

    threads = [threading.Thread(target=client, args=(p,)) for p in range(3)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for k, (t, mode) in enumerate(results):
        sid, rays, prev, _ = reqs[k]
        out = srv.wait(t, timeout=60.0)["out"]
        plain = sc[sid].trace_geometry(rays, prev) if mode == 0 else sc[sid].trace_occlusion(rays, prev)
        _same(out, plain, mode)
    st = srv.stats()
    times = srv.batch_times()
    srv.close()
    assert st["completed"] == len(reqs)
    assert len(times) == st["batches"]
    assert (times["end_ns"] >= times["start_ns"]).all()


def test_batches_on_different_streams_overlap_on_the_device(ctx):
    """Twelve 150K-ray requests at once on three streams: every batch kernel
    leaves room on the GPU, and the next stream's kernel starts before the
    last warp of the previous one has left (their own %globaltimer stamps),
    not only queued together.  The rays and results are in pinned memory, so
    the server's copies are asynchronous (a copy to or from pageable memory
    holds the scheduler thread until it is done)."""
    import torch

    from igx_raytracing_gb300 import HIT_DTYPE, RAY_DTYPE

    sc = _scenes(ctx, n=3, seed=7)
    srv = Server(ctx, streams=3, slice_rays=150000, max_batch_rays=150000)
    ids = [srv.add_scene(s) for s in sc]

    def pinned(a, dtype):
        p = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory().numpy().view(dtype)
        p[:] = a
        return p

    rays = [pinned(scenes.incoherent_rays(150000, 700 + k), RAY_DTYPE) for k in range(12)]
    outs = [pinned(np.zeros(150000, HIT_DTYPE), HIT_DTYPE) for _ in range(12)]
    tickets = [srv.submit(ids[k % 3], r, out=o) for k, (r, o) in enumerate(zip(rays, outs))]
    for t in tickets:
        srv.wait(t, timeout=60.0)
    times = srv.batch_times()
    srv.close()
    for k, o in enumerate(outs):
        _same(o, sc[k % 3].trace_geometry(rays[k]), 0)
    assert len(times) == 12 and set(times["stream"].tolist()) == {0, 1, 2}
    assert _overlapping_pairs(times) >= 1


def test_large_requests_are_sliced_and_equal_the_oracle(ctx):
    sc, tris_of = _scenes(ctx, n=2, seed=5, with_tris=True)
    srv = Server(ctx, streams=2, slice_rays=8192, max_batch_rays=20000)
    ids = [srv.add_scene(s) for s in sc]
    big = scenes.batch_rays(3, 70001)
    small = [scenes.incoherent_rays(300 + 7 * k, 500 + k) for k in range(12)]
    t_big = srv.submit(ids[1], big)
    t_small = [srv.submit(ids[k % 2], r) for k, r in enumerate(small)]
    w_big = srv.wait(t_big, timeout=60.0)
    w_small = [srv.wait(t, timeout=60.0) for t in t_small]
    st = srv.stats()
    srv.close()
    assert st["batches"] >= 70001 // 8192 + 1  # the large request spans several launches
    _oracle_check(tris_of[1], big, None, 0, w_big["out"])
    for k, (r, w) in enumerate(zip(small, w_small)):
        _oracle_check(tris_of[k % 2], r, None, 0, w["out"])
    # small requests queued behind the large one were not held back until it finished
    assert min(w["completed"] for w in w_small) < w_big["completed"]


def test_replay_paces_requests_and_times_them_from_arrival(ctx):
    sc, tris_of = _scenes(ctx, n=2, seed=6, with_tris=True)
    srv = Server(ctx, streams=2)
    ids = [srv.add_scene(s) for s in sc]
    reqs, arrivals = [], []
    for k in range(40):
        rays = scenes.incoherent_rays(500 + 97 * k, 600 + k)
        reqs.append((ids[k % 2], rays, None, k % 2, None))
        arrivals.append(0.002 * k)
    tickets = srv.replay(reqs, arrivals)
    assert all(tickets)
    stats = [srv.wait(t, timeout=60.0) for t in tickets]
    st = srv.stats()
    srv.close()
    a0 = stats[0]["arrival"]
    for k, (w, (sid, rays, _, mode, _)) in enumerate(zip(stats, reqs)):
        # submitted at (never before) its scheduled arrival, 2 ms apart
        assert abs((w["arrival"] - a0) - arrivals[k]) < 1e-6
        assert w["submitted"] >= w["arrival"] - 1e-9
        assert w["completed"] >= w["submitted"]
        _oracle_check(tris_of[k % 2], rays, None, mode, w["out"])
    lat = sorted(1e3 * (w["completed"] - w["arrival"]) for w in stats)
    assert abs(st["p50_ms"] - lat[int(0.5 * (len(lat) - 1) + 0.5)]) < 1e-6
