"""Benchmark of the GB300 tile matching-and-placement path (one JSON line on rank 0).

Workload: the recommended-settings mosaic -- target 3840x2880 (32 blobs),
1500 materials with aspect drawn from {1:1, 4:3, 3:4} at long side 256 (the
4:3 ones pass the aspect filter), grid 80x60, max usage 3, adjacency weight
0.25, colour strength 0.4, 32 annealing chains x 2000 iterations, 48x48
output tiles.  Synthetic, seeded inputs (there are no image files).

A step is one whole generate_mosaic job: palette ingestion (material Lab,
thumbnail means), the similarity database, cell Lab, the k-nearest scan,
greedy placement, the annealing chains and the colour-adjusted composite.

  value  tiles placed per second with the inputs resident in device memory
         (mg_plan_run), device time per step from CUDA events on the library's
         stream, L2 flushed (512 MB write) between steps.
  e2e    the same metric through mg_generate from pinned host buffers: host
         wall time per call, including the uploads and the download of the
         output image and grid.

--impl reference times the CPU restatement of the reference's path (the
reference crate itself cannot be built here: no Rust toolchain) on the host
cores with all threads.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "mosaic-art-rust_gb300"))
sys.path.insert(0, str(REPO))

METRIC = "tiles placed/sec"
WORKLOAD = "recommended"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0 -> same as --steps")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def read_peaks():
    try:
        return json.loads((REPO / "MEASURED_PEAKS.json").read_text()), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload_inputs(name: str, rank: int, allocator=None):
    from mosaic_gpu import job

    cfg = job.WORKLOADS[name]
    if rank:
        cfg = job.scaled(cfg, seed=cfg.seed + 7919 * rank)
    return job.make_inputs(cfg, allocator)


def algorithmic(inp, palette_size: int, sel_px: int):
    """Algorithmic bytes (or candidates) per launch of each stage."""
    cfg = inp.cfg
    N = cfg.grid_w * cfg.grid_h
    cw, ch = cfg.target_w // cfg.grid_w, cfg.target_h // cfg.grid_h
    tw, th = inp.tile
    P = palette_size
    k = min(P, 100)
    return {
        "palette_lab": 3 * sel_px + 16 * P + (3 * tw * th * P + 4 * P if cfg.color_strength > 0 else 0),
        "similarity": 4 * P * P,
        "cell_lab": 3 * cw * ch * N + 16 * N + 4 * N,
        "nearest": 16 * N + 16 * P + 8 * k * N,
        "greedy": 8 * k * N + 4 * N,
        "anneal": 4 * N * (cfg.chains + 1) + 16 * P,
        "composite": 3 * tw * th * N * 2 + 4 * N + 16 * N,
    }


STAGES = ["palette_lab", "similarity", "cell_lab", "nearest", "greedy", "anneal", "composite"]
KERNEL_OF_STAGE = {"palette_lab": "region_stats_kernel", "similarity": "similarity_full_kernel",
                   "cell_lab": "region_stats_kernel", "nearest": "nearest_kernel", "greedy": "greedy_kernel",
                   "anneal": "anneal_kernel", "composite": "composite_kernel"}


def traffic_from_profiles(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    path = REPO / "profiles" / "dram_traffic.txt"
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def cpu_baseline(inp, seconds: float = 10.0):
    import oracle.binding as ob

    cores = os.cpu_count() or 1
    n = inp.cfg.grid_w * inp.cfg.grid_h
    runs, t_total = 0, 0.0
    while t_total < seconds and runs < 12:
        t0 = time.perf_counter()
        ob.generate(inp, threads=cores)
        t_total += time.perf_counter() - t0
        runs += 1
    return {"value": n * runs / t_total, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": f"{runs} full {inp.cfg.name} jobs ({n} cells each) on the C++ restatement of the reference "
                      f"path; material Lab and chains across {cores} threads, cells and greedy walk sequential"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import oracle.binding as ob

    inp = workload_inputs(args.workload, 0)
    cores = os.cpu_count() or 1
    n = inp.cfg.grid_w * inp.cfg.grid_h
    for _ in range(args.warmup):
        ob.generate(inp, threads=cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ob.generate(inp, threads=cores)
        times.append(time.perf_counter() - t0)
    ms = 1000 * statistics.mean(times)
    value = n / (ms / 1000)
    line = {"metric": METRIC, "value": value, "unit": "tiles/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "cells": n, "palette": 1500, "grid": "80x60",
                       "chains": inp.cfg.chains, "iterations": inp.cfg.iterations},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "tiles/s", "cores": cores, "kind": "port",
                             "sample": f"each step one full {args.workload} job on the C++ restatement of the "
                                       f"reference path (the Rust crate cannot be built: no toolchain)"},
            "e2e": {"value": value, "unit": "tiles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local):
    import ctypes as C

    import numpy as np
    import torch

    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    lib = capi.load()
    ctx = capi.Context(local)
    inp = workload_inputs(args.workload, rank, allocator=lib.mg_host_alloc)
    holder = job.RequestHolder(inp, stream=rank)
    cfg = inp.cfg
    N = cfg.grid_w * cfg.grid_h

    # ---- device-resident steps ------------------------------------------------------------
    plan = job.Plan(ctx, holder)
    stream = torch.cuda.ExternalStream(lib.mg_ctx_stream(ctx.h), device=torch.device("cuda", local))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=torch.device("cuda", local))
    for _ in range(args.warmup):
        plan.run()
    capi.check(lib.mg_ctx_sync(ctx.h))
    res, grid, image = plan.read()
    P = res.palette_size
    n_m = len(inp.mats)
    ws = (C.c_int * n_m)(*[int(v) for v in inp.mats.w])
    hs = (C.c_int * n_m)(*[int(v) for v in inp.mats.h])
    sel = (C.c_int * n_m)()
    cnt = lib.mg_select_palette(ws, hs, n_m, cfg.target_w / cfg.target_h, cfg.aspect_tolerance,
                                cfg.max_materials or n_m, sel)
    assert cnt == P
    sel_px = int(sum(int(inp.mats.w[i]) * int(inp.mats.h[i]) for i in sel[:P]))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stage_ms = np.zeros((args.steps, 8))
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    launches0 = lib.mg_kernel_launches()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)          # L2 flush between steps, outside the events
            starts[i].record(stream)
        plan.run()
        with torch.cuda.stream(stream):
            ends[i].record(stream)
        stage_ms[i] = plan.stage_ms()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = int(lib.mg_kernel_launches() - launches0)
    clk = clocks.stop()
    step_ms = float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    if dist:
        t = torch.tensor([step_ms], device=torch.device("cuda", local))
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
        step_ms = float(t.item())
    value = world * N / (step_ms / 1000.0)

    # ---- end to end through mg_generate from pinned host buffers -----------------------
    out_img = np.ctypeslib.as_array(C.cast(lib.mg_host_alloc(image.nbytes), C.POINTER(C.c_uint8)),
                                    shape=(image.nbytes,)).reshape(image.shape)
    out_grid = np.zeros(N, np.int32)
    e2e_steps = args.e2e_steps or args.steps
    for _ in range(2):
        job.generate(ctx, holder, out_img, out_grid)
    if dist:
        dist.barrier()
    times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        r2, g2, im2 = job.generate(ctx, holder, out_img, out_grid)
        times.append(time.perf_counter() - t0)
    e2e_ms = 1000 * statistics.mean(times)
    if dist:
        t = torch.tensor([e2e_ms], device=torch.device("cuda", local))
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    tw, th = inp.tile
    h2d = int(inp.target.nbytes + 3 * sel_px + P * tw * th * 3)
    d2h = int(out_img.nbytes + out_grid.nbytes)
    same = bool(np.array_equal(g2, grid) and np.array_equal(im2, image))

    # ---- roofline of the dominant kernel --------------------------------------------------
    peaks, peak_kind = read_peaks()
    mean_stage = stage_ms.mean(axis=0)
    alg = algorithmic(inp, P, sel_px)
    dom = max(range(7), key=lambda s: mean_stage[s])
    dom_name = STAGES[dom]
    achieved = alg[dom_name] / (mean_stage[dom] / 1000.0) / 1e9
    stages = {STAGES[s]: {"ms": round(float(mean_stage[s]), 4),
                          "gbs": round(alg[STAGES[s]] / max(mean_stage[s], 1e-9) / 1e6, 1)} for s in range(7)}
    line = {
        "metric": METRIC, "value": value, "unit": "tiles/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": args.workload, "cells": N, "palette_in": len(inp.mats), "palette": P,
                   "grid": f"{cfg.grid_w}x{cfg.grid_h}", "chains": cfg.chains, "iterations": cfg.iterations,
                   "tile": f"{tw}x{th}", "l2": "flushed (512 MB write) between steps",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": world * N / (e2e_ms / 1000.0), "unit": "tiles/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "matches_device_run": same},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": KERNEL_OF_STAGE[dom_name], "stage": dom_name,
                     "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 6), "peak_source": peak_kind,
                     "traffic": traffic_from_profiles(KERNEL_OF_STAGE[dom_name]),
                     "algorithmic_bytes": alg[dom_name]},
        "stages": stages,
        "clocks": clk,
        "wall_s_timed": round(wall, 3),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(inp)
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
