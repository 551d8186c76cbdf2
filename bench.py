"""Benchmark of the GB300 ray-query engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl engine|reference]

Workloads (seeded synthetic inputs, no dataset):
  sphere        (default) 1,048,576-triangle displaced sphere; per step the
                1920x1080 primaries (closest hit), one cosine bounce per hit
                (closest hit, prev_hit = hit) and one shadow ray per hit toward
                (3,3,3) (any hit, tmax = light distance).
  small         4,096-triangle heightfield, 256x256 primaries.
  incoherent    2,097,152 random triangles, 4,194,304 incoherent rays.
  incoherent1m  1,048,576 random triangles, 4,194,304 incoherent rays.
  batch         64 random-triangle scenes (1K-512K triangles, 4K-2M rays each):
                one autotuned, graph-captured persistent launch vs 64
                sequential plain launches.
  serve         32 resident scenes, Poisson requests (--rate, --duration)
                through the serving loop vs one request per launch.
  gbuffer       the sphere's 1080p raygen pass as one kernel (rays, hits,
                dirObject / uvNormal encodings) vs camera rays + plain trace.
  shadowmask    the sphere's shadow pass packed into ballot words vs plain
                any-hit on the same rays.
  mixed         1M triangles + 64K spheres + 64K cubes + 4 planes, 4M
                incoherent rays.
  dynamic       the sphere deforming every frame: refit + 1080p primaries
                per step, beside a GPU rebuild per frame.

value: Mrays/s over all rays of a step, inputs resident in device memory,
CUDA-event time per step (L2 flushed between steps), plain kernels with the
launch shape the engine's autotuner picks for the step; in the sphere step
the shadow launch is queued IGXRT_TRACE_INDEPENDENT of the bounce launch
before it (both read only the primary hits), so it may start while the
bounce launch drains.  batched: the same step as one graph-captured
persistent launch.  e2e: the same rays through the C ABI with pinned host
buffers, all host-device traffic inside the timed region.  The headline
route passes the pinned arrays to the stream-ordered calls: the kernels read
the rays and write the results in host memory over NVLink-C2C, with one
synchronization per step.  Beside it: host-memory calls on the same memory
(each returns with its results in host memory), and those calls staged
(copy up, trace, copy down).

The default (sphere) line also carries, measured in the same run with their
own clock records: `incoherent1m` (the roofline target's workload),
`incoherent` (2M triangles), `batch` (64 scenes: one batched launch against
64 plain launches) and `serve` (--serve-seconds of Poisson arrivals at
--rate, latency from each request's scheduled arrival).  --no-extras leaves
them out.

--impl reference times the reference's traversal restated on the CPU (the
oracle's BVH traversal, on a BVH the oracle builds itself) on all host cores,
every ray of the same workload each step; the engine library is not loaded.
--gpus N starts N ranks (one per GPU) when not already under torchrun; each
rank traces the whole step on its own GPU (weak scaling).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "Mrays/s closest-hit, batched/served vs plain kernel; serving p50/p99 ms"
UNIT = "Mrays/s"
RAY_BYTES = 32
HIT_BYTES = 16
OCC_BYTES = 4
PREV_BYTES = 4
NODE_BYTES = {0: 64, 1: 128, 2: 96}
LAYOUT_NAMES = {0: "bvh2", 1: "bvh4", 2: "bvh8"}
LAYOUT_IDS = {v: k for k, v in LAYOUT_NAMES.items()}
PRIM_BYTES = 48


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------
# Workloads: a list of batches (rays, prev, mode) over one triangle set
# --------------------------------------------------------------------------

L2_NOTE = "GPU arm: a 256 MiB buffer is written between timed steps; inputs stay resident"


def workload_config(name: str, tris, batches) -> dict:
    """The workload's description, identical in the engine and reference
    arms: its name, sizes and a digest of every ray, prev_hit and query mode
    of a step (both arms trace the same bytes)."""
    h = hashlib.sha1()
    for _, rays, prev, mode in batches:
        h.update(np.ascontiguousarray(rays).tobytes())
        if prev is not None:
            h.update(np.ascontiguousarray(prev).tobytes())
        h.update(bytes([mode]))
    return {"workload": name, "triangles": int(len(tris)),
            "rays_per_step": int(sum(len(b[1]) for b in batches)), "rays_sha1": h.hexdigest()[:16],
            "l2": L2_NOTE}


WORKLOAD_NAMES = {"small": "heightfield_4k_256x256_primary",
                  "incoherent": "random_2m_tris_4m_incoherent_rays",
                  "incoherent1m": "random_1m_tris_4m_incoherent_rays",
                  "sphere": "sphere_1m_1080p_primary_bounce_shadow"}


def make_workload(name: str, primary_hits=None):
    """(triangles, batches, config) of a workload.  The sphere's bounce and
    shadow rays start at the primary hits: `primary_hits(tris, rays)` gives
    them (the engine in the engine arm, the oracle in the reference arm; the
    two are equal bit for bit, which the CPU-baseline leg checks)."""
    from igx_raytracing_gb300 import scenes

    if name == "small":
        tris, rays = scenes.workload_small()
        batches = [("primary", rays, None, 0)]
    elif name in ("incoherent", "incoherent1m"):
        nt = 2_097_152 if name == "incoherent" else 1_048_576
        tris, rays = scenes.workload_incoherent(nt, 4_194_304, variant=0 if name == "incoherent" else 1)
        batches = [("incoherent", rays, None, 0)]
    elif name == "sphere":
        tris, prim = scenes.workload_sphere_primary()
        hits = primary_hits(tris, prim)
        bounce, shadow, prev = scenes.secondary_rays(tris, prim, hits, scenes.SPHERE_LIGHT,
                                                     scenes.seed_for(2, 50))
        batches = [("primary", prim, None, 0), ("bounce", bounce, prev, 0), ("shadow", shadow, prev, 1)]
    else:
        raise SystemExit(f"unknown workload {name}")
    return tris, batches, workload_config(WORKLOAD_NAMES[name], tris, batches)


def algorithmic_bytes(nf: np.ndarray, pf: np.ndarray, mode: int, has_prev: bool, layout: int) -> int:
    per_ray = RAY_BYTES + (HIT_BYTES if mode == 0 else OCC_BYTES) + (PREV_BYTES if has_prev else 0)
    return int(per_ray * len(nf) + NODE_BYTES[layout] * int(nf.sum(dtype=np.int64))
               + PRIM_BYTES * int(pf.sum(dtype=np.int64)))


def measured_peaks() -> dict:
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def traffic_from_profiles(workload: str, batch: str, layout: int):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    from the committed ncu summary profiles/dram_traffic.txt: lines of
    `<workload> <batch> <layout> <bytes>`, '#' starts a comment."""
    p = os.path.join(REPO, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split("#", 1)[0].split()
            if len(parts) == 4 and parts[0] == workload and parts[1] == batch and parts[2] == LAYOUT_NAMES[layout]:
                return int(parts[3])
    return None


TIMED_REGION = "igxrt_timed_region"


def timed_region_start():
    """NVTX start/end range around the timed steps, so a profiler can list the
    launches of the timed region alone (ncu --nvtx --nvtx-include
    igxrt_timed_region)."""
    try:
        import torch

        return torch.cuda.nvtx.range_start(TIMED_REGION)
    except Exception:
        return None


def timed_region_end(handle) -> None:
    if handle is None:
        return
    try:
        import torch

        torch.cuda.nvtx.range_end(handle)
    except Exception:
        pass


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, interval_ms: int = 20, tag: str = ""):
        """interval_ms: 20 covers timed regions of a few ms; a long serving
        run samples every 250 ms, since each nvidia-smi query briefly holds
        driver locks that the serving thread's CUDA calls then wait on."""
        self.device = device
        self.interval_ms = interval_ms
        self.proc = None
        # the raw samples: IGXRT_CLOCKS_DIR if set, else the temp directory
        import tempfile
        self.path = os.path.join(os.environ.get("IGXRT_CLOCKS_DIR") or tempfile.gettempdir(),
                                 f"igxrt_clocks_dev{device}{tag}.csv")

    def start(self):
        """Starts sampling and returns once the first sample is in, so even a
        short timed region that follows is covered."""
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU baseline: the oracle's BVH traversal (transcription of the reference's
# triangle test) on all host cores, over a bounded strided sample
# --------------------------------------------------------------------------

def cpu_baseline(bvh, batches, budget_s: float = 12.0, layout: int = 0, engine_primary_hits=None) -> dict:
    from oracle import pyoracle

    nodes, prims = bvh.arrays(layout)
    threads = pyoracle.hardware_threads()
    total = sum(len(b[1]) for b in batches)

    def run(stride: int):
        n = 0
        t0 = time.perf_counter()
        for _, rays, prev, mode in batches:
            r = rays[::stride]
            p = None if prev is None else prev[::stride]
            pyoracle.bvh_trace(layout, nodes, prims, r, p, mode=mode, threads=threads)
            n += len(r)
        return n, time.perf_counter() - t0

    # estimate on a small strided sample, then either repeat whole passes
    # until the budget is spent or trace one strided pass of about that length
    probe = max(1, total // 20000)
    n0, dt0 = run(probe)
    full_pass_s = dt0 * total / max(n0, 1)
    stride = 1 if full_pass_s <= budget_s else int(math.ceil(full_pass_s / budget_s))
    n = 0
    dt = 0.0
    passes = 0
    while dt < budget_s or passes == 0:
        k, d = run(stride)
        n += k
        dt += d
        passes += 1
        if stride > 1:
            break
    what = "the whole workload" if stride == 1 else f"every {stride}th ray of each batch"
    out = {"value": round(n / dt / 1e6, 4), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{passes} pass(es) over {what} ({n} rays, {dt:.1f} s): the oracle's BVH "
                     "traversal over the engine's BVH2 with the triangle test transcribed from "
                     "primitive.glsl:239-284"}
    if engine_primary_hits is not None:
        # the engine's primary hits (the origins of the step's secondary rays)
        # against the oracle's traversal, every ray
        _, rays, prev, _ = batches[0]
        expect = pyoracle.bvh_trace(layout, nodes, prims, rays, prev, mode=0, threads=threads)
        out["primary_hits_equal_oracle"] = bool(
            np.ascontiguousarray(engine_primary_hits).tobytes() == expect.tobytes())
    return out


def linear_loop_rate(tris, batches, max_rays: int = 256) -> float:
    """Brute-force rate of the reference's own algorithm (every triangle per ray)."""
    from oracle import pyoracle

    r = batches[0][1][:: max(1, len(batches[0][1]) // max_rays)][:max_rays]
    t0 = time.perf_counter()
    pyoracle.trace_geometry(tris, r)
    return len(r) / (time.perf_counter() - t0) / 1e6


# --------------------------------------------------------------------------
# Reference arm: the reference's traversal restated on the CPU (the oracle),
# over a BVH the oracle builds itself; the engine library is never loaded
# --------------------------------------------------------------------------

def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    from oracle import pyoracle

    if args.workload not in WORKLOAD_NAMES:
        print(json.dumps({"impl": "reference", "unavailable":
                          f"the CPU reference arm covers {sorted(WORKLOAD_NAMES)}, not {args.workload}"}))
        return
    pyoracle.lib()
    threads = pyoracle.hardware_threads()
    trees = {}

    def oracle_tree(tris):
        if "nodes" not in trees:
            t0 = time.perf_counter()
            trees["nodes"], trees["prims"] = pyoracle.bvh_build(tris)
            trees["build_s"] = time.perf_counter() - t0
        return trees["nodes"], trees["prims"]

    def primary_hits(tris, rays):
        nodes, prims = oracle_tree(tris)
        return pyoracle.bvh_trace(0, nodes, prims, rays, threads=threads)

    tris, batches, cfg = make_workload(args.workload, primary_hits)
    nodes, prims = oracle_tree(tris)
    total = sum(len(b[1]) for b in batches)
    times = []
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for _, rays, prev, mode in batches:
            pyoracle.bvh_trace(0, nodes, prims, rays, prev, mode=mode, threads=threads)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
    value = args.steps * total / sum(times) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * statistics.mean(times), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "setup": {"bvh": "the oracle's own binned-SAH BVH2 (oracle/bvh_build_oracle.c)",
                      "bvh_nodes": int(len(nodes)), "bvh_build_s": round(trees["build_s"], 2),
                      "secondaries_from": "the oracle's own primary hits" if args.workload == "sphere" else None},
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"every ray of the workload ({total} per step) each step, traced by "
                                       "the oracle's BVH traversal (the triangle test of "
                                       "primitive.glsl:239-284 in trace.glsl:9-98's closest / any-hit "
                                       "rules) on all host cores"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# Engine arm
# --------------------------------------------------------------------------

def measure_plain(args, ctx, dev, name: str, world: int, lite: bool = False) -> dict:
    """One workload through the plain trace calls: the step (every batch one
    launch, in order) timed with CUDA events, the per-launch figures and the
    roofline of the dominant launch, e2e with pinned host buffers; unless
    `lite`, also the host-memory and staged e2e routes, the batched form of
    the step, and the CPU baseline."""
    import torch

    import igx_raytracing_gb300 as igx
    from igx_raytracing_gb300 import BVH
    from igx_raytracing_gb300.dist import max_over_ranks

    def engine_primary_hits(tris, rays):
        scene = ctx.create_scene(tris)
        hits = scene.trace_geometry(rays)
        scene.close()
        engine_primary_hits.hits = hits
        return hits

    engine_primary_hits.hits = None
    tris, batches, cfg = make_workload(name, engine_primary_hits)
    t0 = time.perf_counter()
    bvh = BVH.build(tris)
    build_s = time.perf_counter() - t0
    scene = ctx.create_scene(bvh=bvh)
    info = scene.info

    # device-resident inputs and outputs
    dev_batches = []
    for bname, rays, prev, mode in batches:
        d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
        d_prev = None if prev is None else torch.from_numpy(prev.view(np.int32).copy()).to(dev)
        out = (torch.empty((len(rays), 4), dtype=torch.float32, device=dev) if mode == 0
               else torch.empty(len(rays), dtype=torch.int32, device=dev))
        dev_batches.append((bname, d_rays, d_prev, mode, out))
    total_rays = sum(len(b[1]) for b in batches)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    # launch shape: the engine's autotuner on this step's batches (unless a
    # layout is forced); the plain launches below then run with it
    items = [(scene, d_rays, d_prev, out, mode) for _, d_rays, d_prev, mode, out in dev_batches]
    tuned = tuned_batch = None
    saved_params = ctx.launch_params
    tune_s = 0.0
    if args.layout is None and not args.no_tune:
        t0 = time.perf_counter()
        # the plain launches as the step issues them (one per batch, in order)
        tuned, _ = ctx.autotune(items, reps=5, force=True, plain=True)
        # and, for the batched figure, the shape of one launch over all batches
        if len(items) > 1 and not lite:
            tuned_batch, _ = ctx.autotune(items, reps=3, force=True)
        tune_s = time.perf_counter() - t0
        ctx.set_launch_params(**tuned)
    # one launch shape for every batch, or each batch its own (the tuner run
    # on that batch alone), whichever runs the whole step faster
    shapes = [dict(ctx.launch_params)] * len(items)
    per_batch_shapes = False

    # The shadow rays and their prev_hit come from the primary hits, not from
    # the bounce launch queued before them: that launch is flagged
    # IGXRT_TRACE_INDEPENDENT and may start while the bounce launch drains.
    indep = [i > 0 and bname == "shadow" for i, (bname, *_rest) in enumerate(dev_batches)]

    def use_shape(i):
        if per_batch_shapes:
            ctx.set_launch_params(**shapes[i])

    def step(events=None, overlap=True):
        for i, (bname, d_rays, d_prev, mode, out) in enumerate(dev_batches):
            if events is not None:
                events[i][0].record(stream)
            use_shape(i)
            f = ctx.trace_closest if mode == 0 else ctx.trace_any
            f(scene, d_rays, d_prev, out=out, independent=overlap and indep[i])
            if events is not None:
                events[i][1].record(stream)

    def quick_step_ms(reps=10):
        for _ in range(3):
            step()
        ms = []
        for s in range(reps):
            flush.fill_(float(s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    if tuned is not None and len(items) > 1:
        t0 = time.perf_counter()
        per = [ctx.autotune([it], reps=5, force=True, plain=True)[0] for it in items]
        ctx.set_launch_params(**tuned)
        if any(p != tuned for p in per):
            one_ms = quick_step_ms()
            shapes, per_batch_shapes = per, True
            per_ms = quick_step_ms()
            if per_ms >= one_ms:
                shapes, per_batch_shapes = [dict(tuned)] * len(items), False
                ctx.set_launch_params(**tuned)
        tune_s += time.perf_counter() - t0
    layouts = [sh["layout"] for sh in shapes]
    layout = layouts[0]

    for _ in range(args.warmup):
        step()
        step(overlap=False)
    torch.cuda.synchronize()
    ctx.sync()

    nb = len(dev_batches)
    # the timed steps: events at step boundaries only (an event between two
    # launches would keep the second from starting early)
    sev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    clocks = ClockSampler(dev.index or 0, tag=f"_{name}")
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    region = timed_region_start()
    wall0 = time.perf_counter()
    for s in range(args.steps):
        flush.fill_(float(s))  # evict the BVH and rays from L2 between steps
        sev[s][0].record(stream)
        step()
        sev[s][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    timed_region_end(region)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    ctx.sync()
    # each rank traces its own replica of the workload (weak scaling); the
    # slowest rank defines the step time
    step_ms = max_over_ranks(float(np.mean([e0.elapsed_time(e1) for e0, e1 in sev])), dev)
    value = world * total_rays / (step_ms / 1e3) / 1e6

    # each launch alone (events around every launch, no overlap), for the
    # per-batch figures and the roofline of the dominant launch
    ev = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(nb)]
          for _ in range(args.steps)]
    for s in range(args.steps):
        flush.fill_(float(s))
        step(ev[s], overlap=False)
    torch.cuda.synchronize()
    ctx.sync()
    launch_ms = np.array([[ev[s][i][0].elapsed_time(ev[s][i][1]) for i in range(nb)]
                          for s in range(args.steps)])
    serial_step_ms = float(launch_ms.sum(axis=1).mean())

    # the same step through the batched engine: all batches in one persistent,
    # graph-captured launch (its own tuned shape), for the batched-vs-plain figure
    batched = None
    if len(dev_batches) > 1 and not lite:
        batch = ctx.create_batch(items, params=tuned_batch or ctx.launch_params)
        for _ in range(args.warmup):
            batch.launch()
        bts = []
        for s in range(args.steps):
            flush.fill_(float(s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            batch.launch()
            e1.record(stream)
            e1.synchronize()
            bts.append(e0.elapsed_time(e1))
        ctx.sync()
        batch.close()
        bms = max_over_ranks(statistics.mean(bts), dev)
        batched = {"ms_per_step": round(bms, 4), "mrays_s": round(world * total_rays / (bms / 1e3) / 1e6, 3),
                   "over_plain": round(step_ms / bms, 3), "launches_per_step": 1}
        if tuned_batch:
            batched["launch"] = tuned_batch

    # roofline: algorithmic bytes per launch from the instrumented kernel
    peaks = measured_peaks()
    per_batch = []
    for i, (bname, rays, prev, mode) in enumerate(batches):
        nf, pf = ctx.count_fetches(scene, rays, prev, mode=mode, layout=layouts[i])
        b = algorithmic_bytes(nf, pf, mode, prev is not None, layouts[i])
        ms = float(launch_ms[:, i].mean())
        per_batch.append({"batch": bname, "rays": len(rays), "mode": "any" if mode else "closest",
                          "layout": LAYOUT_NAMES[layouts[i]],
                          "ms": round(ms, 4), "bytes": b, "nodes_per_ray": round(float(nf.mean()), 3),
                          "prims_per_ray": round(float(pf.mean()), 3),
                          "gbs": round(b / (ms / 1e3) / 1e9, 1),
                          "mrays_s": round(len(rays) / (ms / 1e3) / 1e6, 1)})
    dom = max(per_batch, key=lambda x: x["ms"])
    achieved = dom["bytes"] / (dom["ms"] / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                "traffic": traffic_from_profiles(cfg["workload"], dom["batch"], LAYOUT_IDS[dom["layout"]]),
                "kernel": f"trace_kernel<{dom['layout']},{dom['mode']}> ({dom['batch']})",
                "peak_source": peaks["source"], "bytes_per_launch": dom["bytes"]}
    step_bytes = sum(b["bytes"] for b in per_batch)

    # e2e: the same rays through the C ABI from pinned host buffers
    host = []
    h2d = d2h = 0
    for i, (bname, rays, prev, mode) in enumerate(batches):
        hr = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory()
        hp = torch.from_numpy(prev.view(np.int32).copy()).pin_memory() if prev is not None else None
        ho = (torch.empty((len(rays), 4), dtype=torch.float32) if mode == 0
              else torch.empty(len(rays), dtype=torch.int32)).pin_memory()
        host.append((hr, hp, mode, ho, indep[i]))
        h2d += len(rays) * RAY_BYTES + (len(prev) * PREV_BYTES if prev is not None else 0)
        d2h += len(rays) * (HIT_BYTES if mode == 0 else OCC_BYTES)

    def e2e_async_step():
        # pinned tensors take the stream-ordered call: the kernels read the
        # rays and write the results in host memory, one synchronization per
        # step (the shadow launch independent of the bounce launch, as above)
        for i, (hr, hp, mode, ho, ind) in enumerate(host):
            use_shape(i)
            f = ctx.trace_closest if mode == 0 else ctx.trace_any
            f(scene, hr, hp, out=ho, independent=ind)
        stream.synchronize()

    def e2e_host_call_step():
        # numpy views of the same pinned memory: IGXRT_TRACE_HOST_MEMORY calls,
        # each returning once its results are in host memory
        for i, (hr, hp, mode, ho, _) in enumerate(host):
            use_shape(i)
            r = hr.numpy().view(igx.RAY_DTYPE).reshape(-1)
            pv = hp.numpy().view(np.uint32) if hp is not None else None
            if mode == 0:
                ctx.trace_closest(scene, r, pv, out=ho.numpy().view(igx.HIT_DTYPE).reshape(-1))
            else:
                ctx.trace_any(scene, r, pv, out=ho.numpy().view(np.uint32))

    spread = []  # (fastest, slowest) step of each route, ms

    def e2e_ms_per_step(step_fn):
        for _ in range(args.warmup):
            step_fn()
        times = []
        for _ in range(args.steps):
            flush.fill_(0.0)  # no ray or result of the last step stays in L2
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step_fn()
            times.append(time.perf_counter() - t0)
        spread.append((round(1000 * min(times), 3), round(1000 * max(times), 3)))
        return max_over_ranks(1000 * statistics.mean(times), dev)

    mrays = lambda ms: round(world * total_rays / (ms / 1e3) / 1e6, 3)
    e2e_ms = e2e_ms_per_step(e2e_async_step)
    e2e = {"value": mrays(e2e_ms), "unit": UNIT, "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 3), "ms_min_max": spread[0],
           "route": "pinned host tensors through the stream-ordered calls: the kernels read "
                    "the rays and write the results in host memory over NVLink-C2C; one "
                    "synchronization per step"}
    if not lite:
        host_call_ms = e2e_ms_per_step(e2e_host_call_step)
        ctx.stage_host_arrays = True  # IGXRT_TRACE_STAGED: copy up, trace, copy down
        staged_ms = e2e_ms_per_step(e2e_host_call_step)
        ctx.stage_host_arrays = False
        e2e["host_calls"] = {"value": mrays(host_call_ms), "ms_per_step": round(host_call_ms, 3),
                             "ms_min_max": spread[1],
                             "route": "IGXRT_TRACE_HOST_MEMORY calls on the same pinned memory, "
                                      "each returning with its results in host memory"}
        e2e["staged"] = {"value": mrays(staged_ms), "ms_per_step": round(staged_ms, 3),
                         "ms_min_max": spread[2],
                         "route": "IGXRT_TRACE_STAGED: copy up, trace, copy down, per call"}

    setup = {"layout": LAYOUT_NAMES[layout] if not per_batch_shapes else [LAYOUT_NAMES[l] for l in layouts],
             "launch": ctx.launch_params if not per_batch_shapes else shapes, "bvh_build_s": round(build_s, 2),
             "bvh2_nodes": info["bvh2_nodes"], "sah_cost": round(info["sah_cost"], 2),
             "parallelism": (f"replicas x{world}: every rank traces the whole step on its own GPU "
                             "(weak scaling)") if world > 1 else "single gpu"}
    if tuned is not None:
        setup["launch_chosen_by"] = (
            f"igxrt_autotune with IGXRT_TUNE_PLAIN on the step's batches, "
            + ("then on each batch alone: one shape per launch, set before it, ran the step faster"
               if per_batch_shapes else "one shape for every launch")
            + f" ({tune_s:.1f} s)")
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg, "setup": setup, "roofline": roofline,
            "roofline_step": {"bytes": step_bytes, "achieved": round(step_bytes / (step_ms / 1e3) / 1e9, 1),
                              "unit": "GB/s", "frac": round(step_bytes / (step_ms / 1e3) / 1e9 / peaks["hbm_gbs"], 4)},
            "batches": per_batch, "e2e": e2e, "gpu_launches": args.steps * nb, "clocks": clk,
            "wall_s_timed_region": round(wall, 3)}
    if any(indep):
        line["launches"] = {"independent": [b[0] for b, f in zip(dev_batches, indep) if f],
                            "sum_of_launches_alone_ms": round(serial_step_ms, 4),
                            "what": "shadow launch queued with IGXRT_TRACE_INDEPENDENT after the bounce "
                                    "launch (both read the primary hits only); value times whole steps"}
    if batched is not None:
        line["batched"] = batched
    if not lite and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(bvh, batches, layout=0, engine_primary_hits=engine_primary_hits.hits)
        line["cpu_baseline"]["linear_loop_mrays_s"] = round(linear_loop_rate(tris, batches), 6)
    # free this workload's device memory before the next one
    del dev_batches, items, host, flush
    scene.close()
    bvh.close()
    ctx.set_launch_params(**saved_params)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return line


SUB_KEYS = ("value", "unit", "ms_per_step", "steps", "warmup", "config", "setup", "roofline", "batches",
            "e2e", "clocks", "gpu_launches")


def run_engine(args, rank: int, world: int, local_rank: int):
    import torch

    import igx_raytracing_gb300 as igx

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = igx.Context(local_rank)
    if args.layout is not None:
        ctx.set_launch_params(layout=args.layout)
    line = measure_plain(args, ctx, dev, args.workload, world)
    # the workload's other targets in the same run: the 1M- and 2M-triangle
    # incoherent workloads (the roofline target is on the 1M variant), the
    # 64-scene batch against 64 plain launches, and a serving run
    if args.workload == "sphere" and world == 1 and not args.no_extras:
        for sub in ("incoherent1m", "incoherent"):
            log(f"bench: {sub}")
            s = measure_plain(args, ctx, dev, sub, world, lite=True)
            line[sub] = {k: s[k] for k in SUB_KEYS if k in s}
        line["incoherent1m"]["target"] = {
            "what": "roofline.frac >= 0.5 on 1M random triangles with 4M incoherent rays",
            "met": bool(line["incoherent1m"]["roofline"]["frac"] >= 0.5)}
        log("bench: batch")
        line["batch"] = measure_batch(args, ctx, dev, world)
        log("bench: serve")
        line["serve"] = measure_serve(args, ctx, local_rank, world, args.serve_seconds)
        line["gpu_launches"] += (line["incoherent1m"]["gpu_launches"] + line["incoherent"]["gpu_launches"]
                                 + line["batch"]["gpu_launches"] + line["serve"]["gpu_launches"])
        line["sub_objects"] = ("incoherent1m, incoherent, batch and serve: each measured in this run with "
                               "its own clock record; gpu_launches counts every timed launch of all of them")
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_batch(args, ctx, dev, world: int) -> dict:
    """64 scenes (triangles log-uniform in [1K, 512K]) with ray batches
    log-uniform in [4K, 2M] (half pinhole primaries, half incoherent): one
    autotuned, graph-captured persistent launch against 64 sequential plain
    launches of the same items on one stream."""
    import torch

    from igx_raytracing_gb300 import BVH, scenes
    from igx_raytracing_gb300.dist import max_over_ranks

    ntris, nrays = scenes.workload_batch_plan(64)
    t0 = time.perf_counter()
    items, host_rays, owned = [], [], []
    for i, (nt, nr) in enumerate(zip(ntris, nrays)):
        tris = scenes.random_triangles(int(nt), scenes.seed_for(4, i))
        bvh = BVH.build(tris)
        scene = ctx.create_scene(bvh=bvh)
        bvh.close()
        rays = scenes.batch_rays(i, int(nr))
        d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
        out = torch.empty((len(rays), 4), dtype=torch.float32, device=dev)
        items.append((scene, d_rays, None, out, 0))
        host_rays.append(rays)
        owned.append(scene)
    setup_s = time.perf_counter() - t0
    total_rays = int(sum(len(r) for r in host_rays))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    plain_params = ctx.launch_params

    t0 = time.perf_counter()
    tuned, tuned_ms = ctx.autotune(items, reps=2, force=True)
    tune_s = time.perf_counter() - t0

    def timed(fn, steps):
        ts = []
        for s in range(steps):
            flush.fill_(float(s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return ts

    def sequential():
        for scene, d_rays, _, out, _ in items:
            ctx.trace_closest(scene, d_rays, None, out=out)

    batch = ctx.create_batch(items, params=tuned)
    for _ in range(args.warmup):
        sequential()
        batch.launch()
    torch.cuda.synchronize()
    seq_ms = statistics.mean(timed(sequential, args.steps))
    ctx.set_launch_params(**tuned)
    seq_tuned_ms = statistics.mean(timed(sequential, args.steps))
    ctx.set_launch_params(**plain_params)
    clocks = ClockSampler(dev.index or 0, tag="_batch")
    clocks.start()
    region = timed_region_start()
    bat = timed(batch.launch, args.steps)
    timed_region_end(region)
    clk = clocks.stop()
    bat_ms = max_over_ranks(statistics.mean(bat), dev)
    ctx.sync()
    # the batch's results equal the plain launches' (checked bit for bit here
    # on a few items; the test suite checks items against the oracle)
    # (compared as integers: a miss stores prim 0xFFFFFFFF, a NaN bit pattern)
    ref = [items[i][3].clone() for i in range(0, 64, 16)]
    sequential()
    torch.cuda.synchronize()
    same = all(torch.equal(ref[k].view(torch.int32), items[i][3].view(torch.int32))
               for k, i in enumerate(range(0, 64, 16)))

    # roofline over the whole batch launch
    peaks = measured_peaks()
    layout = tuned["layout"]
    bytes_total = 0
    for (scene, _, _, _, _), rays in zip(items, host_rays):
        nf, pf = ctx.count_fetches(scene, rays, None, mode=0, layout=layout)
        bytes_total += algorithmic_bytes(nf, pf, 0, False, layout)
    achieved = bytes_total / (bat_ms / 1e3) / 1e9

    # e2e from pinned host memory: a batch whose items are the pinned arrays
    # (the kernel reads the rays and writes the hits in place over
    # NVLink-C2C); then the copy route: rays up, the device batch, hits down
    pinned = [torch.from_numpy(r.view(np.float32).reshape(-1, 8).copy()).pin_memory() for r in host_rays]
    hits_host = [torch.empty((len(r), 4), dtype=torch.float32).pin_memory() for r in host_rays]
    batch_h = ctx.create_batch([(it[0], hr, None, hh, 0) for it, hr, hh in zip(items, pinned, hits_host)],
                               params=tuned)

    def copied():
        for (scene, d_rays, _, out, _), hr in zip(items, pinned):
            d_rays.copy_(hr, non_blocking=True)
        batch.launch()
        for (scene, d_rays, _, out, _), hh in zip(items, hits_host):
            hh.copy_(out, non_blocking=True)

    e2e_ms = statistics.mean(timed(batch_h.launch, args.steps))
    same_h = all(torch.equal(hh.view(torch.int32), out.cpu().view(torch.int32))
                 for (_, _, _, out, _), hh in zip(items, hits_host))
    copied_ms = statistics.mean(timed(copied, args.steps))
    batch_h.close()
    batch.close()
    wl = "batch_64_scenes_1k_512k_tris_4k_2m_rays"
    out = {"value": round(world * total_rays / (bat_ms / 1e3) / 1e6, 3), "unit": UNIT,
           "ms_per_step": round(bat_ms, 4), "steps": args.steps, "warmup": args.warmup,
           "config": {"workload": wl, "scenes": 64, "triangles": int(ntris.sum()),
                      "rays_per_step": total_rays, "l2": L2_NOTE},
           "setup": {"autotuned": tuned, "autotune_s": round(tune_s, 2), "setup_s": round(setup_s, 1)},
           "plain_sequential": {"ms_per_step": round(seq_ms, 4),
                                "mrays_s": round(total_rays / (seq_ms / 1e3) / 1e6, 3), "params": plain_params},
           "plain_sequential_tuned": {"ms_per_step": round(seq_tuned_ms, 4),
                                      "mrays_s": round(total_rays / (seq_tuned_ms / 1e3) / 1e6, 3)},
           "batched_over_plain": round(seq_ms / bat_ms, 3),
           "batched_over_plain_tuned": round(seq_tuned_ms / bat_ms, 3),
           "target": {"what": "one batched launch faster than 64 sequential plain launches",
                      "met": bool(seq_ms > bat_ms)},
           "results_equal_plain": bool(same),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                        "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                        "traffic": traffic_from_profiles(wl, "batch", layout),
                        "kernel": f"batch_kernel<{LAYOUT_NAMES[layout]}>", "peak_source": peaks["source"],
                        "bytes_per_launch": int(bytes_total)},
           "e2e": {"value": round(world * total_rays / (e2e_ms / 1e3) / 1e6, 3), "unit": UNIT,
                   "h2d_bytes_per_step": total_rays * RAY_BYTES,
                   "d2h_bytes_per_step": total_rays * HIT_BYTES, "ms_per_step": round(e2e_ms, 3),
                   "route": "batch items in pinned host memory, read and written in place by the kernel",
                   "results_equal_device_batch": bool(same_h),
                   "copied": {"value": round(world * total_rays / (copied_ms / 1e3) / 1e6, 3),
                              "ms_per_step": round(copied_ms, 3),
                              "route": "rays copied up, device batch, hits copied down"}},
           "gpu_launches": args.steps,
           "clocks": clk}
    del items, pinned, hits_host, flush
    for s in owned:
        s.close()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def run_batch_bench(args, rank: int, world: int, local_rank: int):
    import torch

    import igx_raytracing_gb300 as igx

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = igx.Context(local_rank)
    out = measure_batch(args, ctx, dev, world)
    ctx.close()
    if rank != 0:
        return
    line = {"metric": METRIC, "n_gpus": world, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic"}
    line.update(out)
    print(json.dumps(line), flush=True)


def _device_overlap(times) -> dict:
    """From the batch kernels' own %globaltimer intervals: pairs of batches on
    different streams that ran at the same time, and the time during which
    two or more batch kernels ran."""
    iv = sorted((int(t["start_ns"]), int(t["end_ns"]), int(t["stream"])) for t in times)
    pairs = 0
    for i in range(len(iv)):
        for j in range(i + 1, len(iv)):
            if iv[j][0] >= iv[i][1]:
                break
            pairs += iv[j][2] != iv[i][2]
    events = sorted([(s, 1) for s, _, _ in iv] + [(e, -1) for _, e, _ in iv])
    depth, last, busy, multi = 0, 0, 0, 0
    for t, d in events:
        if depth >= 1:
            busy += t - last
        if depth >= 2:
            multi += t - last
        depth += d
        last = t
    return {"batches": len(iv), "overlapping_pairs": int(pairs), "busy_ms": round(busy / 1e6, 3),
            "two_or_more_kernels_ms": round(multi / 1e6, 3),
            "source": "each batch kernel's first CTA start and last warp exit (%globaltimer), "
                      "igxrt_server_batch_times"}


WARMUP_S = 1.0  # serving: seconds of the request stream replayed once before the measured run


def measure_serve(args, ctx, device: int, world: int, duration: float) -> dict:
    """32 resident scenes (10K-2M triangles), Poisson arrivals at `--rate`
    requests/s for `duration` s; each request names a scene, 1K-1M rays
    (log-uniform), closest or any hit.  The requests are submitted by the
    server's native pacer (igxrt_server_replay) at their scheduled arrival
    times, and latency runs from that time to the results in host memory.
    The engine's server (admission under a 24 GiB cap, continuous batching,
    large requests sliced) against a plain server that traces each request
    with one launch in arrival order, both fed the same request stream, each
    after replaying the stream's first WARMUP_S seconds once unmeasured."""
    import torch

    import igx_raytracing_gb300 as igx
    from igx_raytracing_gb300 import BVH, scenes

    rng = np.random.default_rng(scenes.seed_for(5))
    ntris = scenes.log_uniform_ints(rng, 10_000, 2_000_000, 32)
    t0 = time.perf_counter()
    sc, pools = [], []
    pool_rays = 1 << 20
    for i, nt in enumerate(ntris):
        bvh = BVH.build(scenes.random_triangles(int(nt), scenes.seed_for(5, i)))
        sc.append(ctx.create_scene(bvh=bvh))
        bvh.close()
        r = scenes.batch_rays(1000 + i, pool_rays)
        pr = torch.empty(pool_rays * 8, dtype=torch.float32).pin_memory().numpy()
        pr[:] = r.view(np.float32).reshape(-1)
        pools.append(pr.view(igx.RAY_DTYPE))
    setup_s = time.perf_counter() - t0
    # the request stream
    n_req = int(args.rate * duration)
    gaps = rng.exponential(1.0 / args.rate, n_req)
    arrivals = np.cumsum(gaps)
    scene_of = rng.integers(0, 32, n_req)
    counts = scenes.log_uniform_ints(rng, 1000, 1_000_000, n_req)
    modes = rng.integers(0, 2, n_req)
    offsets = rng.integers(0, pool_rays - counts + 1)
    # results land in a pinned ring of 1 GiB (several hundred ms of results
    # at the offered rate; nothing here reads them back)
    out_ring = torch.empty(256 << 20, dtype=torch.float32).pin_memory().numpy()
    ring_words = len(out_ring)

    def requests(ids):
        reqs, pos = [], 0
        for k in range(n_req):
            words = int(counts[k]) * (4 if modes[k] == 0 else 1)
            pos = (pos + 3) & ~3  # hit records need 16-byte alignment
            if pos + words > ring_words:
                pos = 0
            view = out_ring[pos:pos + words]
            pos += words
            out = view.view(igx.HIT_DTYPE) if modes[k] == 0 else view.view(np.uint32)
            rays = pools[scene_of[k]][offsets[k]:offsets[k] + counts[k]]
            reqs.append((ids[scene_of[k]], rays, None, int(modes[k]), out))
        return reqs

    n_warm = int(args.rate * WARMUP_S)

    def serve_pass(opts: dict, with_clocks: bool):
        srv = igx.Server(ctx, memory_cap_bytes=24 << 30, **opts)
        ids = [srv.add_scene(s) for s in sc]
        reqs = requests(ids)
        # warm-up: the stream's first WARMUP_S seconds once, not measured
        # (the server's threads, its arena and the host cores come up to speed)
        for t in srv.replay(reqs[:n_warm], arrivals[:n_warm]):
            srv.wait(t)
        clocks = ClockSampler(device, interval_ms=args.serve_clock_ms, tag="_serve")
        if with_clocks and args.serve_clock_ms > 0:
            clocks.start()
        tickets = srv.replay(reqs, arrivals)
        lat = np.zeros(n_req)
        first, last = float("inf"), 0.0
        for k, t in enumerate(tickets):
            w = srv.wait(t)
            lat[k] = 1e3 * (w["completed"] - w["arrival"])
            first, last = min(first, w["arrival"]), max(last, w["completed"])
        clk = (clocks.stop() if args.serve_clock_ms > 0 else {"sm_mhz": None, "reasons": ["not sampled"]}) \
            if with_clocks else None
        st = srv.stats()
        st["span_s"] = last - first
        times = srv.batch_times()
        srv.close()
        return st, lat, clk, times

    def timeline(lat, window_s=1.0):
        # per window of arrival time: how many requests, their p50, p99 and
        # max latency; a stall of the host shows as a window where every size
        # class is late at once
        out = []
        edges = np.arange(0.0, float(arrivals[-1]) + window_s, window_s)
        for lo in edges[:-1]:
            m = (arrivals >= lo) & (arrivals < lo + window_s)
            if m.any():
                out.append([round(float(lo), 1), int(m.sum()), round(float(np.percentile(lat[m], 50)), 3),
                            round(float(np.percentile(lat[m], 99)), 3), round(float(lat[m].max()), 3)])
        return out

    def pct(lat, q):
        return round(float(np.percentile(lat, q)), 3)

    def classes(lat):
        out = {}
        for name, lo, hi in (("lt10k", 0, 10_000), ("10k_100k", 10_000, 100_000), ("ge100k", 100_000, 1 << 40)):
            m = (counts >= lo) & (counts < hi)
            if m.any():
                out[name] = {"n": int(m.sum()), "p50_ms": round(float(np.percentile(lat[m], 50)), 3),
                             "p99_ms": round(float(np.percentile(lat[m], 99)), 3)}
        return out

    engine_opts = {"streams": args.streams}
    st, srv_lat, clk, times = serve_pass(engine_opts, True)
    served = float(counts.sum()) / st["span_s"] / 1e6
    # plain: the same native server launching one whole request at a time, in
    # arrival order, one launch in flight (no coalescing, slicing or overlap)
    plain_opts = {"streams": 1, "max_batch_requests": 1, "slice_rays": 0xFFFFFFFF}
    pst, plain_lat, _, _ = serve_pass(plain_opts, False)
    plain_span = pst["span_s"]
    offered = float(counts.sum()) / float(arrivals[-1]) / 1e6
    for s in sc:
        s.close()
    return {"value": round(world * served, 3), "unit": UNIT,
            "config": {"workload": "serve_32_scenes_poisson", "scenes": 32, "triangles": int(ntris.sum()),
                       "rate_req_s": args.rate, "duration_s": duration, "requests": n_req,
                       "rays_offered": int(counts.sum()), "offered_mrays_s": round(offered, 3),
                       "memory_cap_gib": 24},
            "setup": {"setup_s": round(setup_s, 1), "launch": ctx.launch_params,
                      "server": dict(engine_opts, slice_rays="default (256K)", max_batch_rays="default (1M)")},
            "latency_from": "each request's scheduled arrival time (submitted by the server's native "
                            "pacer, igxrt_server_replay) to its results in host memory",
            "serving": {"p50_ms": pct(srv_lat, 50), "p99_ms": pct(srv_lat, 99),
                        "mean_ms": round(float(srv_lat.mean()), 3), "max_ms": round(float(srv_lat.max()), 3),
                        "warmup_s": WARMUP_S,
                        "batches": st["batches"], "peak_memory_gib": round(st["peak_memory_bytes"] / 2**30, 3),
                        "peak_pending": st["peak_pending"], "rejected": st["rejected"],
                        "by_size": classes(srv_lat),
                        "timeline": {"columns": ["from_s", "requests", "p50_ms", "p99_ms", "max_ms"],
                                     "windows": timeline(srv_lat)}},
            "device_overlap": _device_overlap(times),
            "plain_server": {"p50_ms": pct(plain_lat, 50), "p99_ms": pct(plain_lat, 99),
                             "mrays_s": round(float(counts.sum()) / plain_span / 1e6, 3),
                             "batches": pst["batches"], "by_size": classes(plain_lat),
                             "mode": "same server, one whole request per launch, one launch in flight"},
            "e2e": {"value": round(world * served, 3), "unit": UNIT,
                    "h2d_bytes_per_step": int(counts.sum() * RAY_BYTES // n_req),
                    "d2h_bytes_per_step": int(sum(int(c) * (HIT_BYTES if m == 0 else OCC_BYTES)
                                                  for c, m in zip(counts, modes)) // n_req),
                    "route": "requests from pinned host memory through the server (copies, batched "
                             "launch, copies back), per request"},
            "gpu_launches": int(st["batches"]),
            "clocks": clk}


def run_serve_bench(args, rank: int, world: int, local_rank: int):
    import torch

    import igx_raytracing_gb300 as igx

    torch.cuda.set_device(local_rank)
    ctx = igx.Context(local_rank)
    # the client thread's GIL slices stay short while the native pacer runs
    sys.setswitchinterval(1e-4)
    out = measure_serve(args, ctx, local_rank, world, args.duration)
    ctx.close()
    if rank != 0:
        return
    line = {"metric": METRIC, "n_gpus": world, "steps": out["config"]["requests"], "warmup": 8,
            "ms_per_step": round(1e3 * args.duration / max(1, out["config"]["requests"]), 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic"}
    line.update(out)
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# The passes beside the plain queries: shadow mask, G-buffer, mixed
# primitives, moving geometry
# --------------------------------------------------------------------------

def _event_ms(torch, fn, steps: int, flush, stream) -> list:
    """CUDA-event time of fn() per step, L2 flushed before each."""
    ts = []
    region = timed_region_start()
    for s in range(steps):
        flush.fill_(float(s))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    timed_region_end(region)
    return ts


def _line(args, world, value, ms, cfg, **extra) -> dict:
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg}
    line.update(extra)
    return line


def _roofline(achieved_bytes: int, ms: float, kernel: str, traffic=None) -> dict:
    peaks = measured_peaks()
    gbs = achieved_bytes / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": round(gbs, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(gbs / peaks["hbm_gbs"], 4), "traffic": traffic, "kernel": kernel,
            "peak_source": peaks["source"], "bytes_per_launch": int(achieved_bytes)}


def run_pass_bench(args, rank: int, world: int, local_rank: int):
    """--workload gbuffer | shadowmask on the 1M-triangle sphere at 1080p.

    gbuffer: igxrt_trace_gbuffer, the reference's raygen.comp (camera rays
    made in the trace kernel, closest hit, then the dirObject and uvNormal
    encodings; the e2e figure writes host images in place with the tile
    kernel); compared with igxrt_camera_rays + igxrt_trace_closest (no
    encodings).
    shadowmask: igxrt_trace_shadow_mask, nv_all.shadow.comp's any-hit rays
    toward the point light packed into ballot words (one sample); compared
    with igxrt_trace_any on the same rays (one word per ray)."""
    import torch

    import igx_raytracing_gb300 as igx
    from igx_raytracing_gb300 import BVH, scenes

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    ctx = igx.Context(local_rank)
    tris, _ = scenes.workload_sphere_primary()
    bvh = BVH.build(tris)
    scene = ctx.create_scene(bvh=bvh)
    w, h = 1920, 1080
    cam = scenes.camera_record(w, h, eye=(0.0, -3.0, 0.0), target=(0.0, 0.0, 0.0))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    rays = ctx.camera_rays(cam)
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
    hits_h = ctx.trace_closest(scene, rays)
    hit = hits_h["prim"] != 0xFFFFFFFF
    layout = ctx.launch_params["layout"]
    cfg = {"triangles": len(tris), "width": w, "height": h, "layout": LAYOUT_NAMES[layout],
           "launch": ctx.launch_params, "l2": "256 MiB buffer written between timed steps"}

    if args.workload == "gbuffer":
        d_do = torch.empty((h, w, 4), dtype=torch.float32, device=dev)
        d_uv = torch.zeros((h, w, 4), dtype=torch.float32, device=dev)
        fused = lambda: ctx.trace_gbuffer(scene, cam, d_do, d_uv)
        d_hits = torch.empty((w * h, 4), dtype=torch.float32, device=dev)
        split = lambda: (ctx.camera_rays(cam, out=d_rays), ctx.trace_closest(scene, d_rays, out=d_hits))
        for _ in range(args.warmup):
            fused()
            split()
        torch.cuda.synchronize()
        clocks = ClockSampler(local_rank)
        clocks.start()
        ms = statistics.mean(_event_ms(torch, fused, args.steps, flush, stream))
        clk = clocks.stop()
        split_ms = statistics.mean(_event_ms(torch, split, args.steps, flush, stream))
        nf, pf = ctx.count_fetches(scene, rays, None, mode=0, layout=layout)
        # per pixel: the trace's hit record written and read back by the
        # encoding kernel (16 + 16 B), dirObject written (16 B); on a hit also
        # uvNormal (16 B) and the hit triangle's normals (48 B); no ray is read
        b = int(48 * len(rays) + (16 + 48) * int(hit.sum()) + NODE_BYTES[layout] * int(nf.sum(dtype=np.int64))
                + PRIM_BYTES * int(pf.sum(dtype=np.int64)))
        hdo = torch.empty((h, w, 4), dtype=torch.float32).pin_memory().numpy()
        huv = torch.zeros((h, w, 4), dtype=torch.float32).pin_memory().numpy()
        ctx.trace_gbuffer(scene, cam, hdo, huv)
        e2e = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            ctx.trace_gbuffer(scene, cam, hdo, huv)
            e2e.append(time.perf_counter() - t0)
        e2e_ms = 1000 * statistics.mean(e2e)
        n = w * h
        line = _line(args, world, world * n / (ms / 1e3) / 1e6, ms,
                     dict(cfg, workload="gbuffer_sphere_1m_1080p", rays_per_step=n),
                     roofline=_roofline(b, ms, f"trace_kernel<{LAYOUT_NAMES[layout]},closest,camera> + "
                                               "gbuffer_encode_kernel",
                                        traffic_from_profiles("gbuffer_sphere_1m_1080p", "gbuffer", layout)),
                     e2e={"value": round(world * n / (e2e_ms / 1e3) / 1e6, 3), "unit": UNIT,
                          "h2d_bytes_per_step": 64, "d2h_bytes_per_step": 32 * n,
                          "ms_per_step": round(e2e_ms, 3)},
                     split={"ms_per_step": round(split_ms, 4),
                            "mrays_s": round(n / (split_ms / 1e3) / 1e6, 3),
                            "what": "igxrt_camera_rays + igxrt_trace_closest (hits, no encodings)",
                            "fused_over_split": round(split_ms / ms, 3)},
                     gpu_launches=args.steps, clocks=clk)
    else:
        # one shadow ray per pixel toward the light from the primary hit;
        # missed pixels cast none (their ray words are never read)
        prim = rays.copy()
        bounce, shadow, prev = scenes.secondary_rays(tris, prim, hits_h, scenes.SPHERE_LIGHT,
                                                     scenes.seed_for(2, 50))
        pix_rays = np.zeros(w * h, dtype=igx.RAY_DTYPE)
        pix_rays[hit] = shadow
        obj = hits_h["prim"].astype(np.uint32)
        d_pix = torch.from_numpy(pix_rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
        d_obj = torch.from_numpy(obj.view(np.int32).copy()).to(dev)
        words = ((w + 15) // 16) * ((h + 1) // 2)
        d_mask = torch.empty(words, dtype=torch.int32, device=dev)
        d_sh = torch.from_numpy(shadow.view(np.float32).reshape(-1, 8).copy()).to(dev)
        d_prev = torch.from_numpy(prev.view(np.int32).copy()).to(dev)
        d_occ = torch.empty(len(shadow), dtype=torch.int32, device=dev)
        if not args.no_tune:
            # the pass's trace launch takes the context's shape: tune it on
            # the same any-hit rays
            tuned, _ = ctx.autotune([(scene, d_sh, d_prev, d_occ, 1)], reps=5, force=True, plain=True)
            ctx.set_launch_params(**tuned)
            layout = tuned["layout"]
            cfg = dict(cfg, layout=LAYOUT_NAMES[layout], launch=ctx.launch_params,
                       launch_chosen_by="igxrt_autotune with IGXRT_TUNE_PLAIN on the pass's any-hit rays")
        fused = lambda: ctx.trace_shadow_mask(scene, d_pix, d_obj, w, h, 1, out=d_mask)
        plain = lambda: ctx.trace_any(scene, d_sh, d_prev, out=d_occ)
        for _ in range(args.warmup):
            fused()
            plain()
        torch.cuda.synchronize()
        clocks = ClockSampler(local_rank)
        clocks.start()
        ms = statistics.mean(_event_ms(torch, fused, args.steps, flush, stream))
        clk = clocks.stop()
        plain_ms = statistics.mean(_event_ms(torch, plain, args.steps, flush, stream))
        nf, pf = ctx.count_fetches(scene, shadow, prev, mode=1, layout=layout)
        # per traced ray: ray (32 B) + its pixel's object (4 B, the prevHit);
        # every pixel's object word is read, every mask word written
        n = int(hit.sum())
        b = int(32 * n + 4 * w * h + 4 * words + NODE_BYTES[layout] * int(nf.sum(dtype=np.int64))
                + PRIM_BYTES * int(pf.sum(dtype=np.int64)))
        # pinned host copies of the pass's inputs and mask
        h_pix = torch.from_numpy(pix_rays.view(np.float32).reshape(-1, 8).copy()).pin_memory().numpy()
        h_pix = h_pix.view(igx.RAY_DTYPE).reshape(-1)
        h_obj = torch.from_numpy(obj.view(np.int32).copy()).pin_memory().numpy().view(np.uint32)
        hmask = torch.empty(words, dtype=torch.int32).pin_memory().numpy().view(np.uint32)
        ctx.trace_shadow_mask(scene, h_pix, h_obj, w, h, 1, out=hmask)
        e2e = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            ctx.trace_shadow_mask(scene, h_pix, h_obj, w, h, 1, out=hmask)
            e2e.append(time.perf_counter() - t0)
        e2e_ms = 1000 * statistics.mean(e2e)
        line = _line(args, world, world * n / (ms / 1e3) / 1e6, ms,
                     dict(cfg, workload="shadowmask_sphere_1m_1080p_1_sample", rays_per_step=n,
                          light=list(scenes.SPHERE_LIGHT)),
                     roofline=_roofline(b, ms, f"shadow pass: compact + trace_kernel<{LAYOUT_NAMES[layout]},any> + pack",
                                        traffic_from_profiles("shadowmask_sphere_1m_1080p_1_sample", "pass", layout)),
                     e2e={"value": round(world * n / (e2e_ms / 1e3) / 1e6, 3), "unit": UNIT,
                          "h2d_bytes_per_step": 36 * w * h, "d2h_bytes_per_step": 4 * words,
                          "ms_per_step": round(e2e_ms, 3)},
                     plain={"ms_per_step": round(plain_ms, 4),
                            "mrays_s": round(n / (plain_ms / 1e3) / 1e6, 3),
                            "what": "igxrt_trace_any on the same rays (one word per ray, no packing)"},
                     gpu_launches=args.steps, clocks=clk)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            mode = 0 if args.workload == "gbuffer" else 1
            sample = [("camera" if mode == 0 else "shadow", rays if mode == 0 else shadow,
                       None if mode == 0 else prev, mode)]
            line["cpu_baseline"] = cpu_baseline(bvh, sample, layout=0)
        print(json.dumps(line), flush=True)


def run_mixed_bench(args, rank: int, world: int, local_rank: int):
    """--workload mixed: 1M triangles, 64K spheres, 64K cubes and 4 planes
    (the reference's four primitive types, trace.glsl:22-46) in one tree,
    4M incoherent rays, closest hit."""
    import torch

    import igx_raytracing_gb300 as igx
    from igx_raytracing_gb300 import BVH, scenes

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    ctx = igx.Context(local_rank)
    sc = scenes.workload_mixed()
    rays = scenes.incoherent_rays(4_194_304, scenes.seed_for(6, 1))
    t0 = time.perf_counter()
    bvh = BVH.build_mixed(sc["tris"], sc["spheres"], sc["cubes"], sc["planes"])
    build_s = time.perf_counter() - t0
    scene = ctx.create_scene(bvh=bvh)
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
    out = torch.empty((len(rays), 4), dtype=torch.float32, device=dev)
    tuned_by = "default launch shape"
    if not args.no_tune:
        tuned, _ = ctx.autotune([(scene, d_rays, None, out, 0)], reps=5, force=True, plain=True)
        ctx.set_launch_params(**tuned)
        tuned_by = "igxrt_autotune with IGXRT_TUNE_PLAIN on the rays"
    layout = ctx.launch_params["layout"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    fn = lambda: ctx.trace_closest(scene, d_rays, out=out)
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    ms = statistics.mean(_event_ms(torch, fn, args.steps, flush, stream))
    clk = clocks.stop()
    nf, pf = ctx.count_fetches(scene, rays, None, mode=0, layout=layout)
    planes = len(sc["planes"])
    b = algorithmic_bytes(nf, pf, 0, False, layout) + 16 * planes * len(rays)
    hrays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).pin_memory().numpy().view(igx.RAY_DTYPE).reshape(-1)
    hout = torch.empty((len(rays), 4), dtype=torch.float32).pin_memory().numpy().view(igx.HIT_DTYPE).reshape(-1)
    ctx.trace_closest(scene, hrays, out=hout)
    e2e = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.trace_closest(scene, hrays, out=hout)
        e2e.append(time.perf_counter() - t0)
    e2e_ms = 1000 * statistics.mean(e2e)
    n = len(rays)
    cfg = {"workload": "mixed_1m_tris_64k_spheres_64k_cubes_4_planes_4m_incoherent",
           "triangles": len(sc["tris"]), "spheres": len(sc["spheres"]), "cubes": len(sc["cubes"]),
           "planes": planes, "rays_per_step": n, "layout": LAYOUT_NAMES[layout],
           "launch": ctx.launch_params, "launch_chosen_by": tuned_by, "bvh_build_s": round(build_s, 2),
           "l2": "256 MiB buffer written between timed steps"}
    line = _line(args, world, world * n / (ms / 1e3) / 1e6, ms, cfg,
                 roofline=_roofline(b, ms, f"trace_kernel<{LAYOUT_NAMES[layout]},closest,mixed>",
                                    traffic_from_profiles(cfg["workload"], "mixed", layout)),
                 e2e={"value": round(world * n / (e2e_ms / 1e3) / 1e6, 3), "unit": UNIT,
                      "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 16 * n,
                      "ms_per_step": round(e2e_ms, 3)},
                 fetches={"nodes_per_ray": round(float(nf.mean()), 3), "prims_per_ray": round(float(pf.mean()), 3)},
                 gpu_launches=args.steps, clocks=clk)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            from oracle import pyoracle

            sample = rays[:: max(1, n // 64)][:64]
            t0 = time.perf_counter()
            pyoracle.trace_geometry_mixed(sample, None, **sc)
            dt = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": round(len(sample) / dt / 1e6, 6), "unit": UNIT,
                                    "cores": pyoracle.hardware_threads(), "kind": "port",
                                    "sample": f"{len(sample)} rays through the oracle's linear loop over all "
                                              "objects (the reference's trace.glsl:22-46 order)"}
        print(json.dumps(line), flush=True)


def run_dynamic_bench(args, rank: int, world: int, local_rank: int):
    """--workload dynamic: the 1M-triangle sphere deforms every frame (the
    reference re-uploads moving geometry per frame, niels_scene.cpp:61-70).
    A step is one frame: new positions (device-resident) -> igxrt_scene_refit
    -> 1080p primaries.  Beside it: the same frame with a full GPU rebuild
    (igxrt_scene_create_gpu) instead of the refit.  e2e: the positions come
    from pinned host memory every frame and the hits go back to it."""
    import torch

    import igx_raytracing_gb300 as igx
    from igx_raytracing_gb300 import BVH, scenes
    from igx_raytracing_gb300.dist import max_over_ranks

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    ctx = igx.Context(local_rank)
    tris, rays = scenes.workload_sphere_primary()
    frames = []
    for k in range(4):  # a breathing, twisting sphere
        f = tris.copy()
        for v in ("p0", "p1", "p2"):
            p = f[v].astype(np.float64)
            s = 1.0 + 0.05 * math.sin(0.7 * k) * np.sin(3.0 * p[:, 2] + k)
            f[v] = (p * s[:, None]).astype(np.float32)
        frames.append(torch.from_numpy(f.view(np.float32).reshape(-1, 12).copy()).to(dev))
    t0 = time.perf_counter()
    bvh = BVH.build(tris)
    host_build_s = time.perf_counter() - t0
    scene = ctx.create_scene(bvh=bvh)
    layout = ctx.launch_params["layout"]
    d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
    out = torch.empty((len(rays), 4), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    counter = {"k": 0}

    def refit_frame():
        scene.refit(frames[counter["k"] % len(frames)])
        counter["k"] += 1
        ctx.trace_closest(scene, d_rays, out=out)

    def rebuild_frame():
        g = ctx.create_scene_gpu(frames[counter["k"] % len(frames)])
        counter["k"] += 1
        ctx.trace_closest(g, d_rays, out=out)
        torch.cuda.synchronize()
        g.close()

    for _ in range(args.warmup):
        refit_frame()
        rebuild_frame()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    ms = statistics.mean(_event_ms(torch, refit_frame, args.steps, flush, stream))
    clk = clocks.stop()
    refit_only = statistics.mean(_event_ms(torch, lambda: scene.refit(frames[0]), args.steps, flush, stream))
    trace_only = statistics.mean(_event_ms(torch, lambda: ctx.trace_closest(scene, d_rays, out=out),
                                           args.steps, flush, stream))
    rebuild_ms = statistics.mean(_event_ms(torch, rebuild_frame, args.steps, flush, stream))
    # end to end: each frame's positions come from pinned host memory (the
    # refit copies them up with IGXRT_TRACE_HOST_MEMORY) and its hits go to
    # pinned host memory in place; the frame's camera rays stay resident
    host_frames = [f.cpu().pin_memory() for f in frames]
    host_out = torch.empty((len(rays), 4), dtype=torch.float32).pin_memory()

    def e2e_frame():
        f = host_frames[counter["k"] % len(frames)]
        counter["k"] += 1
        scene.refit(f.numpy().view(igx.TRIANGLE_DTYPE).reshape(-1))
        ctx.trace_closest(scene, d_rays, out=host_out)
        stream.synchronize()

    for _ in range(args.warmup):
        e2e_frame()
    e2e_s = []
    for _ in range(args.steps):
        flush.fill_(0.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_frame()
        e2e_s.append(time.perf_counter() - t0)
    e2e_ms = max_over_ranks(1000 * statistics.mean(e2e_s), dev)
    e2e_spread = (round(1000 * min(e2e_s), 3), round(1000 * max(e2e_s), 3))

    nf, pf = ctx.count_fetches(scene, rays, None, mode=0, layout=layout)
    n = len(rays)
    b = algorithmic_bytes(nf, pf, 0, False, layout)
    # a frame: the refit's scan, records, nodes and BVH8 passes, then the trace
    si = scene.info
    refit_launches = 2 + (si["bvh2_nodes"] + si["bvh4_nodes"] > 0) + (si["bvh8_nodes"] > 0) + 1
    cfg = {"workload": "dynamic_sphere_1m_refit_1080p_primary", "triangles": len(tris),
           "rays_per_step": n, "layout": LAYOUT_NAMES[layout], "launch": ctx.launch_params,
           "frames": len(frames), "host_sah_build_s": round(host_build_s, 3),
           "l2": "256 MiB buffer written between timed steps"}
    line = _line(args, world, world * n / (ms / 1e3) / 1e6, ms, cfg,
                 roofline=_roofline(b, trace_only, f"trace_kernel<{LAYOUT_NAMES[layout]},closest> (frame rays)",
                                    traffic_from_profiles(cfg["workload"], "frame", layout)),
                 frame={"refit_ms": round(refit_only, 4), "trace_ms": round(trace_only, 4),
                        "refit_plus_trace_ms": round(ms, 4),
                        "gpu_rebuild_plus_trace_ms": round(rebuild_ms, 4),
                        "frames_per_s_refit": round(1e3 / ms, 1),
                        "frames_per_s_gpu_rebuild": round(1e3 / rebuild_ms, 1)},
                 e2e={"value": round(world * n / (e2e_ms / 1e3) / 1e6, 3), "unit": UNIT,
                      "h2d_bytes_per_step": int(host_frames[0].numel() * 4),
                      "d2h_bytes_per_step": int(host_out.numel() * 4), "ms_per_step": round(e2e_ms, 4),
                      "ms_min_max": e2e_spread, "frames_per_s": round(1e3 / e2e_ms, 1),
                      "route": "positions from pinned host memory through igxrt_scene_refit "
                               "(IGXRT_TRACE_HOST_MEMORY: copied up, then refit), hits written in place "
                               "to pinned host memory; camera rays resident; one synchronization per frame"},
                 gpu_launches=args.steps * refit_launches, clocks=clk)
    if rank == 0:
        print(json.dumps(line), flush=True)


def _free_port() -> int:
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="sphere",
                    choices=["sphere", "small", "incoherent", "incoherent1m", "batch", "serve",
                             "gbuffer", "shadowmask", "mixed", "dynamic"])
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--layout", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--no-extras", action="store_true",
                    help="sphere: leave out the incoherent, batch and serve sub-objects")
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="sphere: seconds of arrivals in the serve sub-object")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve: requests per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    ap.add_argument("--streams", type=int, default=2, help="serve: batches in flight")
    ap.add_argument("--serve-clock-ms", type=int, default=250,
                    help="serve: nvidia-smi sampling interval during the serving pass (0: none)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        # start one rank per GPU, as torchrun does for N > 1
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
               os.path.abspath(__file__)] + sys.argv[1:]
        raise SystemExit(subprocess.call(cmd))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world != args.gpus:
        raise SystemExit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}: launch one rank per GPU")
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(local_rank)  # each rank's collectives on its own GPU
        torch.distributed.init_process_group("nccl")
    if args.workload == "batch":
        run_batch_bench(args, rank, world, local_rank)
    elif args.workload == "serve":
        run_serve_bench(args, rank, world, local_rank)
    elif args.workload in ("gbuffer", "shadowmask"):
        run_pass_bench(args, rank, world, local_rank)
    elif args.workload == "mixed":
        run_mixed_bench(args, rank, world, local_rank)
    elif args.workload == "dynamic":
        run_dynamic_bench(args, rank, world, local_rank)
    else:
        run_engine(args, rank, world, local_rank)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
