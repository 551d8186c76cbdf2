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

value: Mrays/s over all rays of a step, inputs resident in device memory,
CUDA-event time per step (L2 flushed between steps).  e2e: the same rays
through the C ABI with pinned host buffers (uploads and downloads inside the
timed region).  --impl reference times the CPU transcription of the
reference's traversal (the oracle's BVH traversal over the same BVH) on all
host cores.
"""
from __future__ import annotations

import argparse
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
NODE_BYTES = {0: 64, 1: 128}
PRIM_BYTES = 48


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------
# Workloads: a list of batches (rays, prev, mode) over one triangle set
# --------------------------------------------------------------------------

def make_workload(name: str, ctx=None):
    from igx_raytracing_gb300 import scenes

    if name == "small":
        tris, rays = scenes.workload_small()
        return tris, [("primary", rays, None, 0)], {"workload": "heightfield_4k_256x256_primary",
                                                    "triangles": len(tris)}
    if name in ("incoherent", "incoherent1m"):
        nt = 2_097_152 if name == "incoherent" else 1_048_576
        tris, rays = scenes.workload_incoherent(nt, 4_194_304, variant=0 if name == "incoherent" else 1)
        return tris, [("incoherent", rays, None, 0)], {
            "workload": f"random_{nt // 1048576 if nt >= 1048576 else nt}m_tris_4m_incoherent_rays",
            "triangles": nt}
    if name == "sphere":
        tris, prim = scenes.workload_sphere_primary()
        # secondaries start at the primary hits found by the engine (the
        # parity tests check those hits against the oracle)
        assert ctx is not None
        scene = ctx.create_scene(tris)
        hits = scene.trace_geometry(prim)
        scene.close()
        bounce, shadow, prev = scenes.secondary_rays(tris, prim, hits, scenes.SPHERE_LIGHT,
                                                     scenes.seed_for(2, 50))
        return tris, [("primary", prim, None, 0), ("bounce", bounce, prev, 0),
                      ("shadow", shadow, prev, 1)], {
            "workload": "sphere_1m_1080p_primary_bounce_shadow", "triangles": len(tris)}
    raise SystemExit(f"unknown workload {name}")


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


def traffic_from_profiles(workload: str, batch: str):
    """DRAM bytes per launch from a committed ncu summary, if one exists."""
    p = os.path.join(REPO, "profiles", "dram_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(workload, {}).get(batch)


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(REPO, "gpurun_out", f"clocks_dev{device}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

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

def cpu_baseline(bvh, batches, budget_s: float = 12.0, layout: int = 0) -> dict:
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
    return {"value": round(n / dt / 1e6, 4), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{passes} pass(es) over {what} ({n} rays, {dt:.1f} s): the oracle's BVH "
                      "traversal over the engine's BVH2 with the triangle test transcribed from "
                      "primitive.glsl:239-284"}


def linear_loop_rate(tris, batches, max_rays: int = 256) -> float:
    """Brute-force rate of the reference's own algorithm (every triangle per ray)."""
    from oracle import pyoracle

    r = batches[0][1][:: max(1, len(batches[0][1]) // max_rays)][:max_rays]
    t0 = time.perf_counter()
    pyoracle.trace_geometry(tris, r)
    return len(r) / (time.perf_counter() - t0) / 1e6


# --------------------------------------------------------------------------
# Reference arm
# --------------------------------------------------------------------------

def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    from igx_raytracing_gb300 import BVH, scenes
    from oracle import pyoracle

    pyoracle.lib()
    if args.workload == "sphere":
        # primary hits come from the oracle's own traversal here (no GPU use)
        tris, prim = scenes.workload_sphere_primary()
        bvh = BVH.build(tris)
        nodes, prims = bvh.arrays(0)
        hits = pyoracle.bvh_trace(0, nodes, prims, prim)
        bounce, shadow, prev = scenes.secondary_rays(tris, prim, hits, scenes.SPHERE_LIGHT,
                                                     scenes.seed_for(2, 50))
        batches = [("primary", prim, None, 0), ("bounce", bounce, prev, 0), ("shadow", shadow, prev, 1)]
        cfg = {"workload": "sphere_1m_1080p_primary_bounce_shadow", "triangles": len(tris)}
    else:
        tris, batches, cfg = make_workload(args.workload)
        bvh = BVH.build(tris)
    threads = pyoracle.hardware_threads()
    nodes, prims = bvh.arrays(0)
    total = sum(len(b[1]) for b in batches)
    stride = max(1, total // 200000)
    times = []
    nrays = 0
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        n = 0
        for _, rays, prev, mode in batches:
            off = step % stride
            r = rays[off::stride]
            p = None if prev is None else prev[off::stride]
            pyoracle.bvh_trace(0, nodes, prims, r, p, mode=mode, threads=threads)
            n += len(r)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
            nrays += n
    value = nrays / sum(times) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * statistics.mean(times), 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(cfg, rays_per_step=total, sample_stride=stride),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads,
                             "kind": "port",
                             "sample": f"each step traces every {stride}th ray of the workload "
                                       "with the oracle's BVH traversal (a transcription of "
                                       "primitive.glsl:239-284 / trace.glsl:9-98) on all cores"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# Engine arm
# --------------------------------------------------------------------------

def run_engine(args, rank: int, world: int, local_rank: int):
    import torch

    import igx_raytracing_gb300 as igx
    from igx_raytracing_gb300 import BVH

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    ctx = igx.Context(local_rank)
    if args.layout is not None:
        ctx.set_launch_params(layout=args.layout)
    layout = ctx.launch_params["layout"]

    tris, batches, cfg = make_workload(args.workload, ctx)
    t0 = time.perf_counter()
    bvh = BVH.build(tris)
    build_s = time.perf_counter() - t0
    scene = ctx.create_scene(bvh=bvh)
    info = scene.info

    # device-resident inputs and outputs
    dev_batches = []
    for name, rays, prev, mode in batches:
        d_rays = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(dev)
        d_prev = None if prev is None else torch.from_numpy(prev.view(np.int32).copy()).to(dev)
        out = (torch.empty((len(rays), 4), dtype=torch.float32, device=dev) if mode == 0
               else torch.empty(len(rays), dtype=torch.int32, device=dev))
        dev_batches.append((name, d_rays, d_prev, mode, out))
    total_rays = sum(len(b[1]) for b in batches)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(events=None):
        for i, (name, d_rays, d_prev, mode, out) in enumerate(dev_batches):
            if events is not None:
                events[i][0].record(stream)
            if mode == 0:
                ctx.trace_closest(scene, d_rays, d_prev, out=out)
            else:
                ctx.trace_any(scene, d_rays, d_prev, out=out)
            if events is not None:
                events[i][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ctx.sync()

    nb = len(dev_batches)
    ev = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(nb)]
          for _ in range(args.steps)]
    clocks = ClockSampler(local_rank)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    for s in range(args.steps):
        flush.fill_(float(s))  # evict the BVH and rays from L2 between steps
        step(ev[s])
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    ctx.sync()
    launch_ms = np.array([[ev[s][i][0].elapsed_time(ev[s][i][1]) for i in range(nb)]
                          for s in range(args.steps)])
    step_ms = float(launch_ms.sum(axis=1).mean())
    if world > 1:
        t = torch.tensor([step_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms = float(t.item())
    value = world * total_rays / (step_ms / 1e3) / 1e6

    # roofline: algorithmic bytes per launch from the instrumented kernel
    peaks = measured_peaks()
    per_batch = []
    for i, (name, rays, prev, mode) in enumerate(batches):
        nf, pf = ctx.count_fetches(scene, rays, prev, mode=mode, layout=layout)
        b = algorithmic_bytes(nf, pf, mode, prev is not None, layout)
        ms = float(launch_ms[:, i].mean())
        per_batch.append({"batch": name, "rays": len(rays), "mode": "any" if mode else "closest",
                          "ms": round(ms, 4), "bytes": b, "nodes_per_ray": round(float(nf.mean()), 3),
                          "prims_per_ray": round(float(pf.mean()), 3),
                          "gbs": round(b / (ms / 1e3) / 1e9, 1),
                          "mrays_s": round(len(rays) / (ms / 1e3) / 1e6, 1)})
    dom = max(per_batch, key=lambda x: x["ms"])
    achieved = dom["bytes"] / (dom["ms"] / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                "traffic": traffic_from_profiles(cfg["workload"], dom["batch"]),
                "kernel": f"trace_kernel<{'bvh4' if layout else 'bvh2'},{dom['mode']}> ({dom['batch']})",
                "peak_source": peaks["source"]}
    step_bytes = sum(b["bytes"] for b in per_batch)

    # e2e: the same rays through the C ABI from pinned host buffers
    host = []
    h2d = d2h = 0
    for name, rays, prev, mode in batches:
        hr = torch.empty(len(rays) * 8, dtype=torch.float32, pin_memory=True).numpy()
        hr[:] = rays.view(np.float32).reshape(-1)
        hp = None
        if prev is not None:
            hp = torch.empty(len(prev), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
            hp[:] = prev
        ho = (torch.empty(len(rays) * 4, dtype=torch.float32, pin_memory=True).numpy()
              .view(igx.HIT_DTYPE) if mode == 0
              else torch.empty(len(rays), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32))
        host.append((hr.view(igx.RAY_DTYPE), hp, mode, ho))
        h2d += len(rays) * RAY_BYTES + (len(prev) * PREV_BYTES if prev is not None else 0)
        d2h += len(rays) * (HIT_BYTES if mode == 0 else OCC_BYTES)

    def e2e_step():
        for hr, hp, mode, ho in host:
            if mode == 0:
                ctx.trace_closest(scene, hr, hp, out=ho)
            else:
                ctx.trace_any(scene, hr, hp, out=ho)

    for _ in range(args.warmup):
        e2e_step()
    e2e_times = []
    for _ in range(args.steps):
        flush.fill_(0.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = 1000 * statistics.mean(e2e_times)
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = world * total_rays / (e2e_ms / 1e3) / 1e6

    if rank != 0:
        return
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": dict(cfg, rays_per_step=total_rays, layout="bvh4" if layout else "bvh2",
                           launch=ctx.launch_params, bvh_build_s=round(build_s, 2),
                           bvh2_nodes=info["bvh2_nodes"], sah_cost=round(info["sah_cost"], 2),
                           l2="256 MiB buffer written between timed steps",
                           parallelism=f"replicas x{world}" if world > 1 else "single gpu"),
            "roofline": roofline,
            "roofline_step": {"bytes": step_bytes, "achieved": round(step_bytes / (step_ms / 1e3) / 1e9, 1),
                              "unit": "GB/s", "frac": round(step_bytes / (step_ms / 1e3) / 1e9 / peaks["hbm_gbs"], 4)},
            "batches": per_batch,
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 3)},
            "gpu_launches": args.steps * nb,
            "clocks": clk,
            "wall_s_timed_region": round(wall, 3)}
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(bvh, batches, layout=0)
        line["cpu_baseline"]["linear_loop_mrays_s"] = round(linear_loop_rate(tris, batches), 6)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="sphere",
                    choices=["sphere", "small", "incoherent", "incoherent1m"])
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--layout", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    run_engine(args, rank, world, local_rank)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
