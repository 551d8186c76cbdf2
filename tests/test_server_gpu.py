"""Serving loop (GPU): admission under a memory cap, continuous batching, and
results that are the same for a request alone and in a mix."""
import math
import threading
import time

import numpy as np
import pytest

from conftest import bits
from igx_raytracing_gb300 import IgxrtError, Server, scenes

pytestmark = pytest.mark.gpu


def _scenes(ctx, n=4, seed=0):
    out = []
    for s in range(n):
        tris = scenes.random_triangles(5000 + 7000 * s, 8100 + 10 * seed + s, mu=math.log(0.02))
        out.append(ctx.create_scene(tris))
    return out


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
    sc = _scenes(ctx)
    reqs = _requests(len(sc), 60, seed=1)
    srv = Server(ctx, streams=3, max_batch_rays=200000)
    ids = [srv.add_scene(s) for s in sc]
    alone = []
    for sid, rays, prev, mode in reqs:  # one at a time: each request in a batch of its own
        t = srv.submit(ids[sid], rays, prev, mode)
        alone.append(srv.wait(t)["out"].copy())
    tickets = [srv.submit(ids[sid], rays, prev, mode) for sid, rays, prev, mode in reqs]
    mixed = [srv.wait(t) for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == 2 * len(reqs) and st["rejected"] == 0
    assert st["batches"] < 2 * len(reqs)  # the mixed pass was coalesced
    for (sid, rays, prev, mode), a, m in zip(reqs, alone, mixed):
        _same(a, m["out"], mode)
        plain = (sc[sid].trace_geometry(rays, prev) if mode == 0
                 else sc[sid].trace_occlusion(rays, prev))
        _same(a, plain, mode)
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
    srv.close()
    assert st["completed"] == len(reqs)
    assert st["peak_in_flight_batches"] >= 2
