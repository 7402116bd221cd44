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
         stream, L2 flushed (512 MB write) between steps.  The K timed steps
         are repeated in passes until about a second of load has run, so the
         clock sampler sees the clocks under load; every pass is timed.
  e2e    the same metric through mg_generate from pinned host buffers: host
         wall time per call, including the uploads and the download of the
         output image and grid.

With one GPU the same line also carries the two serving patterns (batches of
uneven mosaics, a request stream) and the large single mosaic, each measured
in this run on the current build:
  batched  256 uneven mosaics over one resident 10 000-material palette
           (mosaics/s, against the same mosaics one single-mosaic batch after
           another, the plain path)
  served   Poisson arrivals at 50, 200 and 800 req/s over a resident
           20 000-material palette (p50/p99, saturated mosaics/s, against one
           request per batch and one batch in flight, the plain path)
  large    7680x5760 target, 5000 materials, 179x134 cells, 64 chains x
           100 000 iterations (tiles/s; the Lab reductions' and composite's
           GB/s; k-nearest candidates per second)

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
    ap.add_argument("--served-seconds", type=float, default=2.0, help="offered-load run length (served)")
    ap.add_argument("--served-saturated", type=int, default=512, help="requests queued at once (served)")
    ap.add_argument("--served-pool", type=int, default=64, help="distinct targets (served)")
    ap.add_argument("--served-scale", type=float, default=1.0, help="shrinks the cell range (served)")
    ap.add_argument("--served-arena-gb", type=int, default=8, help="pinned output arena (served)")
    ap.add_argument("--batched-mosaics", type=int, default=256, help="mosaics in the batch (batched; fewer for profiling)")
    ap.add_argument("--min-timed-s", type=float, default=1.0, help="repeat the K timed steps until this much load ran")
    ap.add_argument("--no-patterns", action="store_true", help="leave the batched/served/large sub-records out")
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


def bench_config(cfg, palette_in: int, palette: int, tile, world: int) -> dict:
    """The workload as both arms name it (same keys, same values)."""
    return {"workload": cfg.name, "cells": cfg.grid_w * cfg.grid_h, "palette_in": palette_in, "palette": palette,
            "grid": f"{cfg.grid_w}x{cfg.grid_h}", "chains": cfg.chains, "iterations": cfg.iterations,
            "tile": f"{tile[0]}x{tile[1]}", "max_usage": cfg.max_usage, "adjacency_weight": cfg.weight,
            "color_strength": cfg.color_strength, "l2": "flushed (512 MB write) between steps",
            "parallelism": f"replicas x{world}"}


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
                   "cell_lab": "region_stats_kernel", "nearest": "nearest_kernel", "greedy": "greedy_pair_kernel",
                   "anneal": "anneal_cta_kernel", "composite": "composite_kernel"}
# Stages that are chains of dependent decisions (their bytes are a lower bound;
# the limit is the latency of one decision), and the data-parallel ones.
SEQUENTIAL = {"greedy": "latency of one placement decision (row-major walk, sequential by definition)",
              "anneal": "latency of one round of 16 proposals per chain (32 chains, sequential within a chain)"}
DATA_PARALLEL = ["palette_lab", "nearest", "similarity", "composite"]


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


FILE_ENDS_CHILD = r"""
import json, sys, time
import numpy as np
sys.path.insert(0, sys.argv[2])
from mosaic_gpu import _capi as capi
target = np.load(sys.argv[1])
t0 = time.perf_counter()
data = capi.png_encode(target, level=1, threads=0)
enc_ms = 1000 * (time.perf_counter() - t0)
out = np.empty(target.shape, np.uint8)
dec_ms = float("inf")
for _ in range(3):
    t0 = time.perf_counter()
    capi.png_decode(data, out)
    dec_ms = min(dec_ms, 1000 * (time.perf_counter() - t0))
t0 = time.perf_counter()
jdata = capi.jpeg_encode(target, quality=75, threads=0)
jenc_ms = 1000 * (time.perf_counter() - t0)
jdec_ms = float("inf")
for _ in range(3):
    t0 = time.perf_counter()
    back = capi.image_decode(jdata)
    jdec_ms = min(jdec_ms, 1000 * (time.perf_counter() - t0))
print(json.dumps({"png_bytes": len(data), "encode_ms": round(enc_ms, 2), "decode_ms": round(dec_ms, 2),
                  "round_trip_exact": bool(np.array_equal(out, target)),
                  "jpeg": {"bytes": len(jdata), "quality": 75, "encode_ms": round(jenc_ms, 2),
                           "decode_ms": round(jdec_ms, 2), "decoded_shape_ok": back.shape == target.shape}}))
"""


def file_ends(target):
    """The path's file ends on this machine's host cores, beside the step (not
    part of `value` or `e2e`): the workload's target encoded as PNG (level 1,
    all threads) and decoded back (best of three), with the round trip checked;
    and as JPEG (quality 75, the crate's default for a .jpg output) and decoded
    back.  Run in a child process so that nothing in it can cost the bench line."""
    import numpy as np

    info = {"what": "PNG encode (level 1, all host threads) and decode of the target; JPEG (quality 75) the same",
            "pixels_bytes": int(target.nbytes), "host_threads": os.cpu_count()}
    try:
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "target.npy")
            np.save(path, np.ascontiguousarray(target))
            r = subprocess.run([sys.executable, "-c", FILE_ENDS_CHILD, path, str(REPO / "mosaic-art-rust_gb300")],
                               capture_output=True, text=True, timeout=120)
        if r.returncode != 0:
            return {**info, "error": f"exit {r.returncode}: {r.stderr.strip()[-200:]}"}
        return {**info, **json.loads(r.stdout.strip().splitlines()[-1])}
    except Exception as e:
        return {**info, "error": str(e)[:200]}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import oracle.binding as ob

    inp = workload_inputs(args.workload, 0)
    cores = os.cpu_count() or 1
    n = inp.cfg.grid_w * inp.cfg.grid_h
    palette = None
    for _ in range(max(args.warmup, 1)):
        palette = ob.generate(inp, threads=cores)["p"]
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
            "config": bench_config(inp.cfg, len(inp.mats), int(palette), inp.tile, world),
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
    clocks = ClockSampler(local)

    def timed_pass():
        """Exactly K steps between a barrier + synchronize on both sides."""
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        st = np.zeros((args.steps, 8))
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xFF)          # L2 flush between steps, outside the events
                starts[i].record(stream)
            plan.run()
            with torch.cuda.stream(stream):
                ends[i].record(stream)
            st[i] = plan.stage_ms()
        torch.cuda.synchronize()
        return [s.elapsed_time(e) for s, e in zip(starts, ends)], st

    clocks.start()
    wall0 = time.perf_counter()
    launches0 = lib.mg_kernel_launches()
    step_times, stage_rows, passes = [], [], 0
    while True:  # K steps per pass; passes until about a second of load has run
        t, st = timed_pass()
        step_times += t
        stage_rows.append(st)
        passes += 1
        if time.perf_counter() - wall0 >= args.min_timed_s or passes >= 1000:
            break
    wall = time.perf_counter() - wall0
    launches = int(lib.mg_kernel_launches() - launches0)
    clk = clocks.stop()
    stage_ms = np.concatenate(stage_rows)
    step_ms = float(np.mean(step_times))
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
    # cell Lab runs on a second stream beside palette Lab and similarity: its
    # stage time is only the part that outlasts them, not a kernel duration
    stages["cell_lab"] = {"ms": stages["cell_lab"]["ms"], "gbs": None,
                          "note": "runs beside palette_lab and similarity; ms is the part that outlasts them"}
    line = {
        "metric": METRIC, "value": value, "unit": "tiles/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(cfg, len(inp.mats), P, (tw, th), world),
        "timed_passes": {"passes": passes, "steps_per_pass": args.steps,
                         "ms_per_step_per_pass": [round(float(np.mean(step_times[i * args.steps:(i + 1) * args.steps])), 4)
                                                  for i in range(passes)][:20]},
        "e2e": {"value": world * N / (e2e_ms / 1000.0), "unit": "tiles/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "matches_device_run": same},
        "gpu_launches": launches // passes,
        "roofline": {"bound": "hbm", "kernel": KERNEL_OF_STAGE[dom_name], "stage": dom_name,
                     "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 6), "peak_source": peak_kind,
                     "traffic": traffic_from_profiles(KERNEL_OF_STAGE[dom_name]),
                     "algorithmic_bytes": alg[dom_name],
                     "limit": SEQUENTIAL.get(dom_name, "HBM bandwidth"),
                     "us_per_unit": round(1000.0 * mean_stage[dom] / N, 4) if dom_name == "greedy" else None},
        "roofline_data_parallel": (lambda d: {
            "bound": "hbm", "kernel": KERNEL_OF_STAGE[d], "stage": d,
            "achieved": round(alg[d] / (mean_stage[STAGES.index(d)] / 1000.0) / 1e9, 2), "peak": peaks["hbm_gbs"],
            "unit": "GB/s",
            "frac": round(alg[d] / (mean_stage[STAGES.index(d)] / 1000.0) / 1e9 / peaks["hbm_gbs"], 4),
            "traffic": traffic_from_profiles(KERNEL_OF_STAGE[d]), "algorithmic_bytes": alg[d]})(
            max(DATA_PARALLEL, key=lambda d: mean_stage[STAGES.index(d)])),
        "stages": stages,
        "clocks": clk,
        "wall_s_timed": round(wall, 3),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(inp)
    if rank == 0 and world == 1:
        line["file_ends"] = file_ends(inp.target)
    plan.close()
    del flush
    if rank == 0 and world == 1 and not args.no_patterns and args.workload == WORKLOAD:
        # the batched and served patterns and the large mosaic, on this GPU, in this run
        for key, fn in (("batched", lambda: measure_batched(args, 0, 1, local, ctx)),
                        ("served", lambda: measure_served(args, 0, 1, local, ctx)),
                        ("large", lambda: measure_large(args, local, ctx))):
            try:
                line[key] = fn()
            except Exception as e:  # a sub-record never costs the headline line
                line[key] = {"error": f"{type(e).__name__}: {str(e)[:300]}"}
            torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def run_batched(args, rank, world, local):
    from mosaic_gpu import _capi as capi

    ctx = capi.Context(local)
    line = measure_batched(args, rank, world, local, ctx)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def measure_batched(args, rank, world, local, ctx):
    """256 uneven mosaics over one resident 10 000-material palette: the batched
    pipeline (cell statistics and k-nearest over every cell, every walk in one
    launch, every chain in one launch, adjustment and composite; graph replay)
    against the same mosaics run one single-mosaic batch after another (the
    plain path)."""
    import ctypes as C

    import numpy as np
    import torch

    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    lib = capi.load()
    t0 = time.perf_counter()
    specs, mats, thumbs = job.batched_workload(n=args.batched_mosaics, seed=20251203 + 7919 * rank,
                                               allocator=lib.mg_host_alloc)
    gen_s = time.perf_counter() - t0
    pal = job.Palette(ctx, mats, thumbs, 32, 32, target_aspect=4 / 3, build_similarity=True)
    reqs = job.batched_requests(specs)
    n = len(reqs)
    cells = int(sum(s.gw * s.gh for s in specs))
    batch = job.Batch(ctx, pal, reqs)
    stream = torch.cuda.ExternalStream(lib.mg_ctx_stream(ctx.h), device=torch.device("cuda", local))
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=torch.device("cuda", local))
    for _ in range(max(args.warmup, 3)):
        batch.run()
    capi.check(lib.mg_ctx_sync(ctx.h))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = lib.mg_kernel_launches()
    stage = []
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
            starts[i].record(stream)
        batch.run()
        with torch.cuda.stream(stream):
            ends[i].record(stream)
        stage.append(batch.stage_ms())
    torch.cuda.synchronize()
    clk = clocks.stop()
    # graph replays launch the captured kernels without passing the host-side counter
    launches = max(int(lib.mg_kernel_launches() - launches0), batch.launches() * args.steps)
    step_ms = float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    # plain path: the same mosaics, one single-mosaic batch after another
    singles = [job.Batch(ctx, pal, [r]) for r in reqs]
    for _ in range(3):  # tune, capture, replay
        for b in singles:
            b.run()
    capi.check(lib.mg_ctx_sync(ctx.h))
    plain = []
    for rep in range(2):
        with torch.cuda.stream(stream):
            flush.fill_(rep)
            s0 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
        for b in singles:
            b.run()
        with torch.cuda.stream(stream):
            s1 = torch.cuda.Event(enable_timing=True)
            s1.record(stream)
        torch.cuda.synchronize()
        plain.append(s0.elapsed_time(s1))
    plain_ms = float(np.mean(plain))
    same = all(np.array_equal(batch.read(i, want_image=False)[1], singles[i].read(0, want_image=False)[1])
               for i in range(0, n, 17))
    for b in singles:
        b.close()
    # end to end from pinned host buffers to pinned host buffers (one
    # mg_generate_batch call; the targets are read in place)
    tw = 32
    outs = []
    for s in specs:
        g = np.ctypeslib.as_array(C.cast(lib.mg_host_alloc(4 * s.gw * s.gh), C.POINTER(C.c_int32)), shape=(s.gw * s.gh,))
        im = np.ctypeslib.as_array(C.cast(lib.mg_host_alloc(3 * s.gw * s.gh * tw * tw), C.POINTER(C.c_uint8)),
                                   shape=(s.gh * tw, s.gw * tw, 3))
        outs.append((g, im))
    e2e = []
    for _ in range(3):
        t1 = time.perf_counter()
        job.generate_batch(ctx, pal, reqs, outputs=outs)
        e2e.append(time.perf_counter() - t1)
    e2e = e2e[1:]
    e2e_s = float(np.mean(e2e))
    h2d = int(sum(s.target.nbytes for s in specs))
    d2h = int(sum(s.gw * s.gh * tw * tw * 3 + s.gw * s.gh * 4 for s in specs))
    line = {"metric": "mosaics/sec (batched)", "value": n / (step_ms / 1000.0), "unit": "mosaics/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched", "mosaics": n, "cells": cells, "palette": pal.size,
                       "grid_widths": "log-uniform 20..160, 4:3", "px_per_cell": 32, "chains": 8,
                       "iterations": 5000, "l2": "flushed (512 MB write) between steps",
                       "tuning": batch.tuning(), "input_generation_s": round(gen_s, 2)},
            "tiles_per_s": cells / (step_ms / 1000.0),
            "plain": {"ms_per_pass": plain_ms, "mosaics_per_s": n / (plain_ms / 1000.0),
                      "what": "the same mosaics, one single-mosaic batch (graph-replayed) after another"},
            "batched_over_plain": plain_ms / step_ms, "batched_equals_plain": same,
            "stages_ms": {k: round(float(v), 3) for k, v in zip(["cells", "nearest", "walks_chains", "composite",
                                                                 "total"], np.mean(stage, axis=0))},
            "e2e": {"value": n / e2e_s, "unit": "mosaics/s", "ms_per_step": 1000 * e2e_s,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk}
    batch.close()
    pal.close()
    return line


class _Arena:
    """Pinned output buffers handed out in submission order and released in the
    same order (results are collected in submission order)."""

    def __init__(self, lib, nbytes: int):
        import ctypes as C
        import threading
        from collections import deque

        import numpy as np

        addr = lib.mg_host_alloc(nbytes)
        if not addr:
            raise MemoryError(f"pinned arena of {nbytes} bytes")
        self.lib, self.addr = lib, addr
        self.buf = np.ctypeslib.as_array(C.cast(addr, C.POINTER(C.c_uint8)), shape=(nbytes,))
        self.n, self.head = nbytes, 0
        self.live = deque()
        self.cv = threading.Condition()

    def _fit(self, size: int):
        if not self.live:
            return 0 if size <= self.n else None
        tail = self.live[0][0]
        if self.head > tail:  # free: [head, n) and [0, tail)
            if self.head + size <= self.n:
                return self.head
            return 0 if size < tail else None
        return self.head if self.head + size < tail else None  # free: [head, tail)

    def take(self, size: int):
        size = (size + 63) & ~63
        with self.cv:
            start = self._fit(size)
            while start is None:
                self.cv.wait()
                start = self._fit(size)
            self.live.append((start, start + size))
            self.head = start + size
            return self.buf[start:start + size]

    def close(self):
        self.buf = None
        if self.addr:
            self.lib.mg_host_free(self.addr)
            self.addr = None

    def release(self):
        with self.cv:
            self.live.popleft()
            if not self.live:
                self.head = 0
            self.cv.notify_all()


def _serve(server, pool, stream, arrivals, arena, tile, keep=()):
    """Submit stream[j] at arrivals[j] seconds (a submitting thread), collect every
    result in order; latency = result on the host - scheduled arrival."""
    import threading

    import numpy as np

    from mosaic_gpu import _capi as capi

    n = len(stream)
    tickets, sub_t, views = [None] * n, [0.0] * n, [None] * n
    ready = [threading.Event() for _ in range(n)]
    t0 = time.perf_counter() + 0.01

    def submitter():
        for j in range(n):
            dt = t0 + arrivals[j] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            p, m = stream[j]
            spec = pool[p]
            gb = spec.gw * spec.gh * 4
            buf = arena.take(gb + spec.gw * spec.gh * tile * tile * 3)
            grid = buf[:gb].view(np.int32)
            image = buf[gb:gb + spec.gw * spec.gh * tile * tile * 3]
            views[j] = (grid, image)
            sub_t[j] = time.perf_counter()
            tickets[j] = server.submit(m, grid, image)
            ready[j].set()

    th = threading.Thread(target=submitter)
    th.start()
    lat, done, kept = [], [], {}
    for j in range(n):
        ready[j].wait()
        st, res, ms = server.wait(tickets[j])
        if st != capi.MG_OK:
            raise RuntimeError(f"request {j} failed with status {st}")
        if j in keep:
            kept[j] = views[j][0].copy()
        arena.release()
        fin = sub_t[j] + ms / 1000.0
        lat.append(1000.0 * (fin - (t0 + arrivals[j])))
        done.append(fin)
    th.join()
    span = max(done) - (t0 + float(arrivals[0]))
    lag = max(sub_t[j] - (t0 + arrivals[j]) for j in range(n))
    cells = sum(pool[p].gw * pool[p].gh for p, _ in stream)
    return {"requests": n, "mosaics_per_s": n / span, "tiles_per_s": cells / span,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "max_submit_lag_ms": 1000.0 * lag}, kept


def run_served(args, rank, world, local):
    from mosaic_gpu import _capi as capi

    ctx = capi.Context(local)
    line = measure_served(args, rank, world, local, ctx)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def measure_served(args, rank, world, local, ctx):
    """The served stream: Poisson arrivals of mixed-size requests (cells
    log-uniform 500..50 000 at 4:3, 24 px per cell, max usage 5, weight 0.25,
    colour 0.4, 2000 iterations x 4 chains) over one resident palette of 20 000
    128x128 materials with its 20 000 x 20 000 similarity matrix, admitted by the
    server (3 slots, batches of up to 64, 120 GB budget) at 50, 200 and 800
    req/s, beside the plain path (the same loop with one slot and one request
    per batch: one request per launch sequence, nothing overlapped) and the CPU
    restatement of the reference path.  value: served mosaics/s with every
    request queued at once (the saturated rate); results go from pinned host
    targets to pinned host outputs."""
    import numpy as np

    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    lib = capi.load()
    seed = 20251203 + 7919 * rank
    t0 = time.perf_counter()
    pool, mats, thumbs = job.served_workload(n_targets=args.served_pool, seed=seed, allocator=lib.mg_host_alloc,
                                             scale=args.served_scale)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    pal = job.Palette(ctx, mats, thumbs, 24, 24, target_aspect=4 / 3, build_similarity=True)
    pal_s = time.perf_counter() - t0
    tile = 24
    arena = _Arena(lib, args.served_arena_gb << 30)
    loads = [50.0, 200.0, 800.0]
    secs = args.served_seconds
    max_n = int(max(loads) * secs)
    stream = job.served_stream(pool, max(max_n, args.served_saturated), seed)
    srv = job.Server(ctx, pal, slots=3, max_batch=64, memory_budget_bytes=120 << 30)
    _serve(srv, pool, stream[:32], np.zeros(32), arena, tile)  # warm-up
    launches0 = lib.mg_kernel_launches()
    clocks = ClockSampler(local)
    clocks.start()
    sat_n = args.served_saturated
    sat, kept = _serve(srv, pool, stream[:sat_n], np.zeros(sat_n), arena, tile, keep=(0, 1, 2, sat_n - 1))
    clk = clocks.stop()
    launches = int(lib.mg_kernel_launches() - launches0)
    offered = {}
    for k, rate in enumerate(loads):
        n = int(rate * secs)
        arr = job.poisson_arrivals(rate, n, seed + k)
        offered[f"{int(rate)}"], _ = _serve(srv, pool, stream[:n], arr, arena, tile)
    st = srv.stats()
    srv.close()
    # plain path: one slot, one request per batch
    plain_srv = job.Server(ctx, pal, slots=1, max_batch=1, memory_budget_bytes=120 << 30)
    _serve(plain_srv, pool, stream[:8], np.zeros(8), arena, tile)
    plain_n = max(16, sat_n // 4)
    plain_sat, kept_plain = _serve(plain_srv, pool, stream[:plain_n], np.zeros(plain_n), arena, tile, keep=(0, 1, 2))
    plain_offered = {}
    cap = plain_sat["mosaics_per_s"]
    for k, rate in enumerate(loads):
        n = min(int(rate * secs), max(8, int(cap * secs)))
        arr = job.poisson_arrivals(rate, n, seed + k)
        plain_offered[f"{int(rate)}"], _ = _serve(plain_srv, pool, stream[:n], arr, arena, tile)
    plain_srv.close()
    same = all(np.array_equal(kept[j], kept_plain[j]) for j in (0, 1, 2))
    # CPU restatement of the reference path on the request nearest the median size
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        import oracle.binding as ob

        cores = os.cpu_count() or 1
        cells = sorted(pool[p].gw * pool[p].gh for p, _ in stream[:sat_n])
        med = cells[len(cells) // 2]
        spec = min(pool, key=lambda s: abs(s.gw * s.gh - med))
        cfg = job.JobConfig("served", spec.w, spec.h, 8, len(mats), 128, 0, spec.gw, spec.gh, 5, 0.25, 0.4, 2000, 4,
                            tile, tile, seed=seed)
        tc = time.perf_counter()
        ob.generate(job.Inputs(cfg, spec.target, mats, thumbs), threads=cores)
        dt = time.perf_counter() - tc
        cpu = {"value": 1.0 / dt, "unit": "mosaics/s", "cores": cores, "kind": "port",
               "sample": f"one {spec.gw}x{spec.gh} request (median size) with the 20 000-material palette on "
                         f"the C++ restatement of the reference path, which ingests the palette and builds "
                         f"the similarity matrix per request as the reference's generator does"}
    value = sat["mosaics_per_s"]
    cells = sum(pool[p].gw * pool[p].gh for p, _ in stream[:sat_n])
    h2d = int(sum(pool[p].target.nbytes for p, _ in stream[:sat_n]))
    d2h = int(sum(pool[p].gw * pool[p].gh * (4 + tile * tile * 3) for p, _ in stream[:sat_n]))
    line = {"metric": "served mosaics/sec", "value": value, "unit": "mosaics/s", "n_gpus": world,
            "steps": 1, "warmup": 1, "ms_per_step": 1000.0 * sat_n / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "served", "palette": pal.size, "similarity": f"{pal.size}x{pal.size} fp32",
                       "pool_targets": len(pool), "cells": "log-uniform 500..50000, 4:3", "px_per_cell": tile,
                       "chains": 4, "iterations": 2000, "max_usage": 5, "slots": 3, "max_batch": 64,
                       "budget_gb": 120, "saturated_requests": sat_n, "saturated_cells": cells,
                       "offered_seconds": secs, "l2": "inputs larger than L2 (20 000-material palette, "
                       "1.6 GB similarity)", "input_generation_s": round(gen_s, 2),
                       "palette_build_s": round(pal_s, 3)},
            "saturated": sat, "offered": offered, "server_stats": st,
            "plain": {"saturated": plain_sat, "offered": plain_offered,
                      "what": "the same loop with one slot and one request per batch"},
            "served_over_plain": value / plain_sat["mosaics_per_s"], "served_equals_plain": same,
            "e2e": {"value": value, "unit": "mosaics/s", "ms_per_step": 1000.0 * sat_n / value,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk, "cpu_baseline": cpu}
    pal.close()
    arena.close()
    return line


def measure_large(args, local, ctx, steps: int = 3):
    """The large single mosaic at full size (7680x5760 target, 128 blobs; 5000
    materials 128x128; 179x134 cells; max usage 8; 64 chains x 100 000
    iterations; 32x32 tiles): the device-resident plan timed per stage with CUDA
    events (L2 flushed between steps), and the figures that configuration is
    quoted on -- GB/s of the two Lab reductions and of the composite, and
    k-nearest candidates (cells x palette) per second.  The cell reduction runs
    beside the material reduction inside the plan, so it is also timed alone
    here on the resident target (mg_cells_lab_noalloc on the same stream)."""
    import ctypes as C

    import numpy as np
    import torch

    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    lib = capi.load()
    dev = torch.device("cuda", local)
    t0 = time.perf_counter()
    inp = workload_inputs("large", 0, allocator=lib.mg_host_alloc)
    gen_s = time.perf_counter() - t0
    cfg = inp.cfg
    N = cfg.grid_w * cfg.grid_h
    holder = job.RequestHolder(inp)
    plan = job.Plan(ctx, holder)
    stream = torch.cuda.ExternalStream(lib.mg_ctx_stream(ctx.h), device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    for _ in range(3):
        plan.run()
    capi.check(lib.mg_ctx_sync(ctx.h))
    res, grid, image = plan.read()
    P = res.palette_size
    sel_px = int(sum(int(w) * int(h) for w, h in zip(inp.mats.w, inp.mats.h)))  # 1:1 materials: all kept
    clocks = ClockSampler(local)
    clocks.start()
    times, stages = [], []
    for i in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 0xFF)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
        plan.run()
        with torch.cuda.stream(stream):
            b.record(stream)
        stages.append(plan.stage_ms())
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    # the cell reduction alone, device-resident target
    cw, ch = cfg.target_w // cfg.grid_w, cfg.target_h // cfg.grid_h
    d_img = torch.from_numpy(np.ascontiguousarray(inp.target)).to(dev)
    d_lab = torch.empty((N, 4), dtype=torch.float32, device=dev)
    d_rgb = torch.empty((N, 4), dtype=torch.uint8, device=dev)
    cell_ms = []
    with torch.cuda.stream(stream):
        for i in range(4):
            flush.fill_(i & 0xFF)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            capi.check(lib.mg_cells_lab_noalloc(C.c_void_p(d_img.data_ptr()), cfg.target_w, cfg.target_h,
                                                3 * cfg.target_w, cfg.grid_w, cfg.grid_h,
                                                C.c_void_p(d_lab.data_ptr()), C.c_void_p(d_rgb.data_ptr()),
                                                C.c_void_p(lib.mg_ctx_stream(ctx.h))))
            b.record(stream)
            torch.cuda.synchronize()
            if i:
                cell_ms.append(a.elapsed_time(b))
    clk = clocks.stop()
    # end to end from pinned host buffers
    out_img = np.ctypeslib.as_array(C.cast(lib.mg_host_alloc(image.nbytes), C.POINTER(C.c_uint8)),
                                    shape=(image.nbytes,)).reshape(image.shape)
    out_grid = np.zeros(N, np.int32)
    job.generate(ctx, holder, out_img, out_grid)
    e2e = []
    for _ in range(2):
        t1 = time.perf_counter()
        _, g2, im2 = job.generate(ctx, holder, out_img, out_grid)
        e2e.append(time.perf_counter() - t1)
    same = bool(np.array_equal(g2, grid) and np.array_equal(im2, image))
    plan.close()
    peaks, peak_kind = read_peaks()
    hbm = peaks["hbm_gbs"]
    st = np.mean(stages, axis=0)
    step_ms = float(np.mean(times))
    alg = algorithmic(inp, P, sel_px)
    cell_bytes = 3 * cw * ch * N + 20 * N
    cms = float(np.mean(cell_ms))

    def gbs(nbytes, ms):
        v = nbytes / (ms / 1000.0) / 1e9
        return {"gbs": round(v, 1), "frac_of_measured_hbm": round(v / hbm, 4), "ms": round(ms, 4), "bytes": int(nbytes)}

    tw, th = inp.tile
    out = {"metric": METRIC, "value": N / (step_ms / 1000.0), "unit": "tiles/s", "ms_per_step": step_ms,
           "steps": steps, "config": bench_config(cfg, len(inp.mats), P, (tw, th), 1),
           "stages_ms": {k: round(float(v), 4) for k, v in zip(STAGES + ["total"], st)},
           "material_lab": gbs(alg["palette_lab"], float(st[0])),
           "cell_lab": {**gbs(cell_bytes, cms), "what": "cell reduction alone on the resident target (it overlaps "
                                                      "the material reduction inside the step)"},
           "composite": gbs(alg["composite"], float(st[6])),
           "similarity": gbs(alg["similarity"], float(st[1])),
           "nearest": {"candidates_per_s": N * P / (float(st[3]) / 1000.0), "ms": round(float(st[3]), 4),
                       "what": "cells x palette per second of the k-nearest stage (the bucket-grid search "
                               "computes far fewer distances than that)"},
           "greedy_us_per_cell": round(1000.0 * float(st[4]) / N, 4),
           "anneal_proposals_per_s": cfg.chains * cfg.iterations / (float(st[5]) / 1000.0),
           "e2e": {"value": N / float(np.mean(e2e)), "unit": "tiles/s", "ms_per_step": 1000.0 * float(np.mean(e2e)),
                   "h2d_bytes_per_step": int(inp.target.nbytes + 3 * sel_px + P * tw * th * 3),
                   "d2h_bytes_per_step": int(out_img.nbytes + out_grid.nbytes), "matches_device_run": same},
           "peak_source": peak_kind, "input_generation_s": round(gen_s, 2), "clocks": clk}
    if not args.no_cpu_baseline:
        import oracle.binding as ob

        cores = os.cpu_count() or 1
        tc = time.perf_counter()
        ob.generate(inp, threads=cores)
        dt = time.perf_counter() - tc
        out["cpu_baseline"] = {"value": N / dt, "unit": "tiles/s", "cores": cores, "kind": "port",
                               "sample": "one full large job on the C++ restatement of the reference path"}
    return out


def run_large(args, rank, world, local):
    from mosaic_gpu import _capi as capi

    ctx = capi.Context(local)
    line = measure_large(args, local, ctx, steps=args.steps)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload == "batched":
        run_batched(args, rank, world, local)
    elif args.workload == "served":
        run_served(args, rank, world, local)
    elif args.workload == "large-figures":
        run_large(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
