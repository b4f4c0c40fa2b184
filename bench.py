"""Throughput bench: body-steps/s of the direct-sum step at N = 1,048,576.

Workload (one GPU): N = 1,048,576 bodies uniform in [0,1)^3 at rest, log-normal(0, 0.5)
masses summing to 1, softened law eps = 1e-3, G = 1, FP32, semi-implicit Euler
dt = 1e-3, no wrap. A "step" is one full update (accelerate + integrate) of all bodies.

Printed JSON line (rank 0):
  value           body-steps/s with the bodies resident in HBM, timed on the device with
                  CUDA events around each step on the launching stream; L2 is flushed
                  between steps (outside the events) by writing 256 MiB.
  e2e             the same metric through the C ABI with host buffers: every step uploads
                  the Body array from pinned host memory, steps, and downloads it again.
  roofline        the direct-sum kernel against the measured FP32 FFMA peak
                  (nbody_cuda_calibrate_fp32): 20 flop per pair (the GPU Gems 3 ch. 31
                  convention), N^2 pairs per launch, divided by the kernel's own average
                  event-timed duration.
  cpu_baseline    the reference's CPU brute force (oracle/_ref, built from the reference's
                  sources) where it loads, else the oracle's C restatement, on all host
                  cores, timed on a bounded sample of targets against all N sources.

``--impl reference`` times only the CPU implementation (same workload, metric and
units) and prints its own line.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N = 1 << 20
EPS = 1e-3
DT = 1e-3
METRIC = "body-steps/s N=1M direct & 16M BH θ=0.5; compensated vs plain FP32 at err≤1e-6"
WORKLOAD = ("direct-sum step, N=1048576 uniform unit cube at rest, log-normal(0,0.5) masses "
            "summing to 1, softened eps=1e-3, G=1, dt=1e-3, FP32, semi-implicit Euler")
FLOP_PER_PAIR = 20


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


# --- clocks ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        rows = [r for r in csv.reader(io.StringIO(self.out or "")) if len(r) >= 9]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for name, val in zip(names, r[5:9]):
                if val.strip() == "Active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# --- CPU baseline -------------------------------------------------------------------------

def cpu_brute_force_rate(bodies: np.ndarray, seconds: float = 10.0):
    """Pairs/s of the reference CPU brute force (or its restatement) on all host cores,
    timed on a bounded sample of targets against all sources."""
    from oracle import oracle as O
    n = len(bodies)
    threads = O.threads()
    use_ref = O.ref_available()
    kind = "reference" if use_ref else "port"

    def run(k):
        tg = np.linspace(0, n - 1, k).astype(np.int64)
        t0 = time.perf_counter()
        if use_ref:
            # the reference solver runs over all of its bodies; give it k targets + all
            # sources by timing k/n of a full sweep through the targets-only restated path
            # is not possible, so time its own accelerate on a k-body prefix scaled below.
            sub = bodies[:k]
            O.ref_brute_force(sub, 1.0, nthreads=threads)
            dt = time.perf_counter() - t0
            return k * k, dt
        O.brute_force_targets(bodies, 1.0, tg, nthreads=threads)
        dt = time.perf_counter() - t0
        return k * n, dt

    if use_ref:
        k = 2048
        pairs, dt = run(k)
        while dt < seconds / 4 and k < n:
            k = min(n, int(k * max(1.5, min(4.0, np.sqrt(seconds / max(dt, 1e-3))))))
            pairs, dt = run(k)
        sample = f"CpuBruteForceSolver::accelerate on the first {k} bodies (all {k}x{k} pairs)"
    else:
        k = 64
        pairs, dt = run(k)
        while dt < seconds / 4:
            k = int(k * min(8.0, max(2.0, seconds / max(dt, 1e-3))))
            pairs, dt = run(k)
        sample = f"{k} sampled targets x all {n} sources (restated reference brute force)"
    return pairs / dt, threads, kind, sample, dt


# --- the GPU arm ----------------------------------------------------------------------------

def bench_gpu(args):
    import torch

    # A dedicated stream: the context queues on it and the timing events are recorded on
    # it (torch's default stream has handle 0, which would not be this stream).
    torch.cuda.set_device(env_rank()[2])
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        return _bench_gpu(args, stream)


def _bench_gpu(args, stream):
    import torch

    from nbody_gb300 import native, scenes

    rank, world, local = env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    st, why = native.probe()
    if st != native.OK:
        raise SystemExit(f"no usable GB300: {why}")

    bodies = scenes.uniform_cube(N, seed=1003)
    p = native.params(dt=DT, G=1.0, eps2=EPS * EPS, law=native.LAW_SOFTENED, size=0.0, wrap=False)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    ctx = native.Context(native.LAYOUT_SOA)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload_bodies(bodies)
    s_tf, p_tf = ctx.calibrate_fp32()
    fp32_peak = max(s_tf, p_tf)

    def one_step():
        ctx.update(p, 1)

    for _ in range(args.warmup):
        flush.zero_()
        one_step()
    torch.cuda.synchronize()

    # --- device-timed steps (value) ---
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = ctx.launches()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            one_step()
            ends[k].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ctx.synchronize()
    launches = ctx.launches() - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = N * args.steps * world / (total_ms * 1e-3)

    # --- the dominant kernel alone (accelerate), for the roofline ---
    acc_starts = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    acc_ends = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    for k in range(3):
        flush.zero_()
        acc_starts[k].record(stream)
        ctx.accelerate(p)
        acc_ends[k].record(stream)
    torch.cuda.synchronize()
    ctx.synchronize()
    acc_ms = statistics.mean(s.elapsed_time(e) for s, e in zip(acc_starts, acc_ends))
    cfg = ctx.last_direct_config()
    pairs = float(N) * N
    achieved_tf = FLOP_PER_PAIR * pairs / (acc_ms * 1e-3) / 1e12

    # --- end to end through the C ABI with host buffers ---
    host = torch.from_numpy(bodies).pin_memory()
    host_np = host.numpy()
    e2e_steps = max(1, min(args.steps, 5))
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.upload_bodies(host_np)
        ctx.update(p, 1)
        ctx.download_bodies(into=host_np)
    t1 = time.perf_counter()
    e2e_value = N * e2e_steps * world / (t1 - t0)
    ctx.close()

    line = None
    if rank == 0:
        cpu_rate, cores, kind, sample, cpu_s = cpu_brute_force_rate(bodies, seconds=args.cpu_seconds)
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "body-steps/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_per_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic (seeded Philox): uniform unit cube, log-normal masses",
            "config": {"workload": WORKLOAD, "n_bodies": N, "eps": EPS, "dt": DT, "law": "softened",
                       "precision": "fp32", "layout": "soa", "parallelism": "replicas only",
                       "l2": "flushed between steps (256 MiB write outside the timed events)",
                       "launch": cfg},
            "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": N * 48,
                    "d2h_bytes_per_step": N * 48, "steps": e2e_steps,
                    "path": "nbody_cuda_upload_bodies + nbody_cuda_update + nbody_cuda_download_bodies, pinned host Body[]"},
            "roofline": {"bound": "fp32", "kernel": "direct_fp32_kernel", "achieved": achieved_tf,
                         "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved_tf / fp32_peak,
                         "peak_source": "measured FFMA/FFMA2 chains on this GPU (nbody_cuda_calibrate_fp32)",
                         "peak_scalar_ffma": s_tf, "peak_packed_ffma2": p_tf,
                         "flop_per_pair": FLOP_PER_PAIR, "pairs_per_launch": pairs,
                         "kernel_ms": acc_ms, "traffic": None},
            "cpu_baseline": {"value": cpu_rate / N, "unit": "body-steps/s", "cores": cores, "kind": kind,
                             "sample": sample + f"; {cpu_s:.1f} s; body-steps/s = pairs/s / N",
                             "pairs_per_s": cpu_rate},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
        }
    if world > 1:
        torch.distributed.destroy_process_group()
    return line


def bench_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return None
    from nbody_gb300 import scenes
    bodies = scenes.uniform_cube(N, seed=1003)
    per_step = []
    info = None
    for k in range(args.warmup + args.steps):
        rate, cores, kind, sample, dt = cpu_brute_force_rate(bodies, seconds=args.cpu_seconds / 2)
        info = (cores, kind, sample)
        if k >= args.warmup:
            per_step.append(N / rate)     # seconds for one full body-step of all N bodies
    total = sum(per_step)
    value = N * args.steps / total
    cores, kind, sample = info
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "body-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Philox): uniform unit cube, log-normal masses",
        "config": {"workload": WORKLOAD, "n_bodies": N, "eps": EPS, "dt": DT,
                   "note": "reference CPU brute force uses its own radius-cutoff law (no softening); "
                           "same pair count and arithmetic class"},
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": cores, "kind": kind,
                         "sample": sample + " per step; body-steps/s = pairs/s / N"},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        line = bench_reference(args)
    else:
        import __graft_entry__
        __graft_entry__.build()
        line = bench_gpu(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
