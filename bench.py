"""Benchmark of the Kerr null-geodesic batch tracer (geodesics/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload 1080p|c1|batch64]

A step traces every pixel of the workload once. Default workload: one 1920x1080 frame, a=0.998,
r_obs=1000 M, theta=60 deg, alpha in +-20 M with square pixels, disk ISCO..30 M, mixed precision
(FP32 Dormand-Prince, rtol 1e-6) -- the frame the headline metric is quoted on. The inputs are
frame descriptors (the pixel index is the ray), so every launch recomputes all 2,073,600 rays.

`value`   geodesics/s with the descriptor already on the device: CUDA events on the launching stream
          around each step (set-up, FP64 launch, sort, trace, rescue), L2 flushed between steps.
`e2e`     the same through bhk_trace_frames_host: host descriptors in, host SoA outputs back
          (pinned), wall clock per call.
`roofline` the tracer kernel against the measured FP32 FMA peak: accepted steps x FLOPs per step
          (counted from the kernel source) / kernel time (CUDA events inside the library).
`cpu_baseline` the reference integrator (its RK4 loop shape at its product tolerance 1e-2, which
          meets the 1e-4 accuracy bar) on all host cores, a bounded sample of the same frame.

--impl reference times that CPU implementation alone (rank 0) on the same workload and metric.
Multi-GPU (torchrun): every rank traces its own copy of the workload (replicas, weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "geodesics/s"
REF_TOL = 1e-2          # reference product tolerance (src/trajectory.cpp:261); meets the 1e-4 bar
# DRAM bytes (read + write) of one tracer launch from ncu, by workload: the 960x540 capture of
# profiles/trace_kernel_1080p_mixed.md (14.61 MB) scaled by rays to the full frame.
NCU_TRAFFIC = {"1080p": 58.4e6}
SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def workload(name: str, scale: int = 1):
    from black_simulation_gb300 import bhk
    if name == "1080p":
        w, h = 1920 // scale, 1080 // scale
        return [bhk.frame_c2(w, h)], bhk.TraceOpts("mixed", rtol=1e-6), dict(
            workload=f"{w}x{h} frame, a=0.998, r_obs=1000M, theta=60deg, alpha +-20M, disk ISCO-30M",
            rays=w * h, precision="mixed FP32/FP64", rtol=1e-6)
    if name == "c1":
        return [bhk.frame_c1()], bhk.TraceOpts("fp64", rtol=1e-10), dict(
            workload="128x128 frame, a=0.9, r_obs=50M, theta=80deg, alpha,beta +-15M, disk ISCO-20M",
            rays=128 * 128, precision="fp64", rtol=1e-10)
    if name == "batch64":
        frames = batch64_frames()
        return frames, bhk.TraceOpts("mixed", rtol=1e-6, use_graph=True), dict(
            workload="64 seeded frames, width U[256,2048], 16:9 or 1:1, a U[0,0.998], theta U[5,89]deg, "
                     "r_obs log-U[20,1000]M, half-width 1.2x shadow radius", rays=sum(f.rays for f in frames),
            precision="mixed FP32/FP64", rtol=1e-6)
    raise SystemExit(f"unknown workload {name}")


def batch64_frames(seed: int = 20261203):
    """64 frames of uneven size, spin and pose from one seeded generator."""
    from black_simulation_gb300 import bhk
    rng = np.random.Generator(np.random.PCG64(seed))
    frames = []
    for _ in range(64):
        w = int(rng.integers(256, 2049))
        h = int(round(w * 9 / 16)) if rng.random() < 0.5 else w
        a = float(rng.uniform(0.0, 0.998))
        th = math.radians(float(rng.uniform(5.0, 89.0)))
        r = float(math.exp(rng.uniform(math.log(20.0), math.log(1000.0))))
        ca, cb = bhk.critical_curve(a, r, th, 200)
        half = 1.2 * float(np.max(np.hypot(ca, cb)))
        hb = half * h / w
        frames.append(bhk.Frame(a, r, th, w, h, -half, half, -hb, hb, 0.0, 30.0))
    return frames


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.rows = []
        self.proc = None
        self.index = index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={SMI_FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows),
                "power_w_max": max((float(r[3]) for r in self.rows if r[3].replace(".", "").isdigit()), default=None)}


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if n_gpus > 0 else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sample_rays(frames, stride: int):
    """Strided pixel sample of the frames: (a, r_obs, theta_obs, alpha, beta) arrays."""
    cols = []
    for f in frames:
        col = np.arange(f.width)
        row = np.arange(f.height)
        al = f.alpha_lo + (col + 0.5) * (f.alpha_hi - f.alpha_lo) / f.width
        be = f.beta_hi - (row + 0.5) * (f.beta_hi - f.beta_lo) / f.height
        A, B = np.meshgrid(al, be)
        A, B = A.ravel()[::stride], B.ravel()[::stride]
        cols.append((np.full(len(A), f.a), np.full(len(A), f.r_obs), np.full(len(A), f.theta_obs), A, B,
                     f.r_disk_out))
    return cols


def cpu_reference_rate(frames, target_s: float = 12.0, threads: int | None = None):
    """Reference RK4 loop (oracle port) at its product tolerance on all host cores: rays/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    if not os.path.exists(po.LIB_ORACLE):
        po.build()
    O = po.Oracle()
    threads = threads or os.cpu_count() or 1
    total = sum(f.rays for f in frames)
    stride = max(1, total // 2048)
    done, elapsed = 0, 0.0
    while True:
        t0 = time.perf_counter()
        n = 0
        for a, r, th, al, be, r_out in sample_rays(frames, stride):
            sc = po.scene(a=float(a[0]), r_obs=float(r[0]), theta_obs_deg=math.degrees(th[0]), r_disk_out=r_out,
                          tol=REF_TOL, method=po.RK4, max_steps=2_000_000)
            O.trace_rays(sc, a, r, th, al, be, nthreads=threads)
            n += len(a)
        dt = time.perf_counter() - t0
        done += n
        elapsed += dt
        if elapsed >= target_s * 0.3 or stride == 1:
            break
        stride = max(1, int(stride * dt / (target_s * 0.7)))
    return done / elapsed, done, elapsed, threads


def run_reference(args):
    world, rank, _ = dist_setup(0)
    if rank != 0:
        return
    frames, _, cfg = workload(args.workload, args.scale)
    cfg = {k: v for k, v in cfg.items() if k not in ("precision", "rtol")}
    rates = []
    for i in range(args.warmup + args.steps):
        rate, n, dt, threads = cpu_reference_rate(frames, target_s=max(2.0, 30.0 / (args.warmup + args.steps)))
        if i >= args.warmup:
            rates.append((rate, n, dt))
    value = float(np.mean([r[0] for r in rates]))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * np.mean([r[2] for r in rates]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {**cfg, "tolerance": REF_TOL, "accuracy": "reference RK4 at its product tolerance 1e-2: "
                   "r_disk 8e-5, g 1.6e-5, exit angle 1.1e-5 rad vs the FP64 oracle"},
        "cpu_baseline": {"value": value, "unit": "rays/s", "cores": threads, "kind": "port",
                         "sample": f"{rates[0][1]} strided pixels of the workload per step"},
        "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ours(args):
    import torch
    from black_simulation_gb300 import bhk, build
    build.build()
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    frames, opts, cfg = workload(args.workload, args.scale)
    n_rays = sum(f.rays for f in frames)
    ctx = bhk.Context(local)
    work_stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(work_stream)
    if args.block or args.chunk or args.buckets or args.reg_budget:
        opts.block, opts.chunk, opts.sort_buckets, opts.reg_budget = args.block, args.chunk, args.buckets, args.reg_budget
        tuned = {"block": args.block, "chunk": args.chunk, "sort_buckets": args.buckets, "reg_budget": args.reg_budget}
    else:
        tuned = ctx.autotune(frames, opts) if args.autotune else None
    out = bhk.alloc_outputs(n_rays, dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MB > 129 MB L2
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        ctx.trace_frames(frames, opts, out=out)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kernel_ms, acc_steps, rej_steps, rescued = [], [], [], []
    barrier(world)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    with Clocks(local) as clk:
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            ctx.trace_frames(frames, opts, out=out)
            ev[i][1].record(stream)
            st = ctx.stats()
            kernel_ms.append(st["kernel_ms"])
            acc_steps.append(st["accepted_steps"])
            rej_steps.append(st["rejected_steps"])
            rescued.append(st["rescued"])
        torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = max_over_ranks(float(np.mean(step_ms)), world, dev)
    value = world * n_rays / (ms * 1e-3)
    # end to end through the host-buffer C-ABI call
    pinned = {k: torch.empty(n_rays, dtype=v.dtype, pin_memory=True) for k, v in out.items()}
    e2e_t = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, status = ctx.trace_frames_host(frames, opts, out=pinned)
        if i >= args.warmup:
            e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.mean(e2e_t)), world, dev)
    d2h = sum(v.numel() * v.element_size() for v in pinned.values())
    h2d = len(frames) * bhk.C.sizeof(bhk.FrameDescC)
    peak = bhk.fp32_fma_peak_tflops(local)
    fps = bhk.flops_per_step()
    k_ms = float(np.mean(kernel_ms))
    achieved = float(np.mean(acc_steps)) * fps / (k_ms * 1e-3) / 1e12
    counts = {k: int(v) for k, v in zip(*np.unique(pinned["outcome"].numpy(), return_counts=True))}
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if opts.precision == "mixed" else "f64", "data": "synthetic",
        "config": {**cfg, "parallelism": f"replicas x{world}", "l2": "flushed (256 MB write) between steps",
                   "block": (tuned or {}).get("block"), "chunk": (tuned or {}).get("chunk"),
                   "sort_buckets": (tuned or {}).get("sort_buckets"), "reg_budget": (tuned or {}).get("reg_budget"),
                   "status": status,
                   "outcomes": {"captured": counts.get(1, 0), "disk": counts.get(2, 0),
                                "escaped": counts.get(3, 0), "unfinished": counts.get(0, 0)},
                   "mean_accepted_steps_per_ray": float(np.mean(acc_steps)) / n_rays,
                   "rejected_fraction": float(np.sum(rej_steps)) / max(1.0, float(np.sum(acc_steps) + np.sum(rej_steps))),
                   "rescued_rays": int(np.mean(rescued)), "wall_s": wall},
        "e2e": {"value": world * n_rays / e2e_s, "unit": "rays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "traffic": NCU_TRAFFIC.get(args.workload) if args.scale == 1 else None,
                     "peak_source": "measured FP32 FMA throughput (bhk_fp32_fma_peak) in this run",
                     "kernel_ms": k_ms, "flops_per_step": fps},
        "gpu_launches": 7 * args.steps,
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        rate, n, dt, threads = cpu_reference_rate(frames, target_s=15.0)
        line["cpu_baseline"] = {"value": rate, "unit": "rays/s", "cores": threads, "kind": "port",
                                "sample": f"{n} strided pixels of the workload, reference RK4 at tolerance 1e-2, "
                                          f"{dt:.1f} s"}
    ctx.close()
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="1080p", choices=["1080p", "c1", "batch64"])
    ap.add_argument("--autotune", action="store_true", default=True)
    ap.add_argument("--no-autotune", dest="autotune", action="store_false")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--scale", type=int, default=1, help="divide the frame size (profiling captures)")
    ap.add_argument("--block", type=int, default=0, help="fixed launch shape instead of autotuning")
    ap.add_argument("--chunk", type=int, default=0)
    ap.add_argument("--buckets", type=int, default=0)
    ap.add_argument("--reg-budget", type=int, default=0)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
