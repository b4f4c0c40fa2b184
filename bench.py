"""Throughput bench: body-steps/s of the direct-sum step at N = 1,048,576, plus the
compensated form, the FP64 form, Barnes-Hut at N = 16,777,216 and the small configs.

Headline workload (one GPU): N = 1,048,576 bodies uniform in [0,1)^3 at rest, log-normal
(0, 0.5) masses summing to 1, softened law eps = 1e-3, G = 1, FP32, semi-implicit Euler
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
  compensated     the same workload in the split-precision form: body-steps/s, its ratio
                  to plain FP32, and the median / p99 relative acceleration error of each
                  form against FP64 on 65,536 sampled targets (the FP64 reference is the
                  GPU FP64 form, itself checked against the CPU oracle on 512 targets).
  barnes_hut_16m  N = 16,777,216 exponential disk + Hernquist halo, eps = 0.005,
                  dt = 2.5e-4, FP32 tree forces + compensated integration, at reference-
                  convention theta 0.5 and 0.75 and conventional theta 0.5 and 0.75
                  (reference theta 2 and 4/3), each with both walks (per target, per
                  group with interaction lists): steps/s, interactions, the device time of
                  the build and of the traversal (nbody_cuda_bh_stage_ms), the build's
                  compulsory bytes against the measured HBM copy bandwidth, the traversal's
                  interactions (20 flop each) against the FFMA peak, and the median / p99
                  relative error against the FP64 direct sum on 4096 sampled targets. Its
                  "drift_100_steps" object runs config 5's 100 steps and reports the energy
                  and momentum drift from nbody_cuda_energy at both ends.
                  Its "transfer" object times the host transfer paths (staged, mapped,
                  direct) for all 16.8M Body records against the copy engine's pinned
                  bandwidth, and one frame of update + state(). Its "cpu_reference_bh"
                  object times one full step of the restated CPU Barnes-Hut on the same
                  bodies on all host cores.
  configs         configs 1 (N = 4096 Plummer, 100 steps) and 2 (2 x 131072 Plummer BH,
                  both theta conventions and walks, with FP64 errors on 4096 sampled
                  targets), each beside the reference's CPU solver (restated, softened law)
                  on the same bodies and host cores (all 100 steps of config 1; one step
                  of config 2), and config 4 (512 batched systems).
  scene_generators util::disk and util::cube on the device at N = 16,777,216, against the
                  reference's serial generator on 1,048,576 bodies.
  ray_query       Tree::query over the exported tree of 1,048,576 bodies: picking rays
                  and full walks per second, against the walk on one host core.
  cpu_baseline    the reference's CPU brute force, restated in the oracle (speed build), with
                  the GPU arm's softened law, on all host cores, timed on a bounded sample
                  of targets against all N sources.

``--impl reference`` times only that CPU implementation on the same workload, metric and
units, a bounded sample of targets per step, and prints its own line.
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
N_SAMPLE = 65536
# ncu DRAM bytes (read + write) of one N = 2^20 direct-sum launch, by (targets per thread,
# block, packed mode, jsplit): the j-split partials stay mostly in L2, so traffic is far
# below the 16 MB x (1 + jsplit) the launch touches.
MEASURED_TRAFFIC = {(4, 256, 1, 4): 17975296 + 11777024, (4, 256, 2, 4): 18174976 + 12430080}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def measured_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return {}


# --- clocks ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.out = ""

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
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

def cpu_brute_force_rate(bodies: np.ndarray, seconds: float = 10.0, eps2: float = EPS * EPS):
    """Pairs/s of the reference's CPU brute force (CpuBruteForceSolver::accelerate,
    cpu_brute_force.h:17-43, restated in oracle/nbody_oracle.c) with the GPU arm's own
    softened law, on all host cores, timed on a bounded sample of the workload: k sampled
    targets against all n sources. The restatement is timed in its speed build (-O2, the
    reference's fastest build); the reference's own sources do not exist on the GPU host."""
    from oracle import oracle as O
    n = len(bodies)
    threads = O.threads()
    k = 64
    while True:
        tg = np.linspace(0, n - 1, k).astype(np.int64)
        t0 = time.perf_counter()
        O.brute_force_targets(bodies, 1.0, tg, nthreads=threads, law=O.LAW_SOFTENED, eps2=eps2, timing=True)
        dt = time.perf_counter() - t0
        if dt >= seconds / 4:
            break
        k = int(k * min(8.0, max(2.0, seconds / max(dt, 1e-3))))
    return k * n / dt, threads, "port", \
        f"{k} sampled targets x all {n} sources (restated reference brute force, softened law as the GPU arm), {dt:.1f} s"


def cpu_config1_seconds(bodies, steps, dt, eps2):
    """Seconds for `steps` whole updates (accelerate + integrate) of the reference's CPU
    brute force on all host cores: Sim::update (sim.cpp:307-313, Solver::update
    solver.h:59) over CpuBruteForceSolver, restated (speed build), with the GPU arm's
    softened law."""
    from oracle import oracle as O
    threads = O.threads()
    b = np.ascontiguousarray(bodies, np.float32).copy()
    tg = np.arange(len(b), dtype=np.int64)
    t0 = time.perf_counter()
    for _ in range(steps):
        b[:, 8:11] = O.brute_force_targets(b, 1.0, tg, nthreads=threads, law=O.LAW_SOFTENED, eps2=eps2, timing=True)
        b = O.integrate(b, dt, 10000.0, False)
    return time.perf_counter() - t0, threads, "port (restated CpuBruteForceSolver + integrate, softened law)"


def cpu_barnes_hut_rate(bodies, size, theta, eps2):
    """Seconds per step of the reference's CpuBarnesHutSolver (serial tree build + parallel
    traversal, cpu_barnes_hut.h:22-44), restated (speed build), with the GPU arm's softened
    law, on all host cores."""
    from oracle import oracle as O
    threads = O.threads()
    t0 = time.perf_counter()
    O.barnes_hut(bodies, size, theta, 1.0, nthreads=threads, law=O.LAW_SOFTENED, eps2=eps2, timing=True)
    return time.perf_counter() - t0, threads


# --- helpers for the GPU arm ------------------------------------------------------------------

def timed_steps(torch, stream, flush, fn, steps):
    """Per-step CUDA-event times (ms) on `stream`, L2 flushed between steps."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        flush.zero_()
        starts[k].record(stream)
        fn()
        ends[k].record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def rel_stats(acc, ref):
    d = np.linalg.norm(np.asarray(acc, np.float64) - ref, axis=1)
    r = d / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)
    return {"median": float(np.median(r)), "p99": float(np.percentile(r, 99)), "max": float(r.max())}


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
    for _ in range(args.warmup):
        flush.zero_()
        ctx.update(p, 1)
    torch.cuda.synchronize()
    s_tf, p_tf = ctx.calibrate_fp32()      # after warm-up: clocks are up
    fp32_peak = max(s_tf, p_tf)
    # the library's direct-sum autotuner picks the kernel shape (outside the timed region)
    tuned, tune_ms = ctx.direct_autotune(p)
    tune_table = [dict(native.Context.direct_variant(i), ms=round(float(t), 3)) for i, t in enumerate(tune_ms)]
    flush.zero_()
    ctx.update(p, 1)
    torch.cuda.synchronize()

    # --- device-timed steps (value) ---
    launches0 = ctx.launches()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        step_ms = timed_steps(torch, stream, flush, lambda: ctx.update(p, 1), args.steps)
    if world > 1:
        torch.distributed.barrier()
    ctx.synchronize()
    launches = ctx.launches() - launches0
    # replicas only: the slowest rank's time, every rank's bodies
    from nbody_gb300.replicas import whole_job_value
    value, total_ms, _ = whole_job_value(sum(step_ms), N, args.steps, device="cuda")
    ms_per_step = total_ms / args.steps

    # --- the dominant kernel alone (accelerate), for the roofline ---
    acc_ms = statistics.mean(timed_steps(torch, stream, flush, lambda: ctx.accelerate(p), 3))
    ctx.synchronize()
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

    extra = {}
    if rank == 0 and not args.quick:
        extra["compensated"] = bench_compensated(torch, stream, flush, native, bodies, args, value, fp32_peak)
        extra["barnes_hut_16m"] = bench_bh16m(torch, stream, flush, native, scenes, args)
        extra["configs"] = bench_small_configs(torch, stream, flush, native, scenes)
        extra["configs"]["config4_batched"] = bench_batched(torch, stream, flush, native, scenes,
                                                            float(N) * N / (acc_ms * 1e-3))
        extra["scene_generators"] = bench_scenes(torch, stream, native)
        extra["ray_query"] = bench_query(native, scenes)

    line = None
    if rank == 0:
        cpu_rate, cores, kind, sample = cpu_brute_force_rate(bodies, seconds=args.cpu_seconds)
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
                       "launch": cfg, "autotune": {"chosen": tuned, "accelerate_ms_per_shape": tune_table}},
            "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": N * 48,
                    "d2h_bytes_per_step": N * 48, "steps": e2e_steps,
                    "path": "nbody_cuda_upload_bodies + nbody_cuda_update + nbody_cuda_download_bodies, pinned host Body[]"},
            "roofline": {"bound": "fp32", "kernel": "direct_fp32_kernel", "achieved": achieved_tf,
                         "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved_tf / fp32_peak,
                         "peak_source": "measured FFMA/FFMA2 chains on this GPU (nbody_cuda_calibrate_fp32); "
                                        "MEASURED_PEAKS.json carries no FP32 figure",
                         "peak_scalar_ffma": s_tf, "peak_packed_ffma2": p_tf,
                         "flop_per_pair": FLOP_PER_PAIR, "pairs_per_launch": pairs,
                         "kernel_ms": acc_ms,
                         "traffic": MEASURED_TRAFFIC.get((cfg["targets_per_thread"], cfg["block"],
                                                          native.Context.direct_variant(tuned)["packed"],
                                                          cfg["jsplit"])),
                         "traffic_source": "constant: ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                           "N=2^20 launch of the chosen shape, captured earlier with the "
                                           "profiler, not measured in this run; null for a shape not captured"},
            "cpu_baseline": {"value": cpu_rate / N, "unit": "body-steps/s", "cores": cores, "kind": kind,
                             "sample": sample + "; body-steps/s = pairs/s / N", "pairs_per_s": cpu_rate},
            "clocks": clocks.summary(),
            "gpu_launches": launches,
        }
        line.update(extra)
    if world > 1:
        torch.distributed.destroy_process_group()
    return line


def bench_compensated(torch, stream, flush, native, bodies, args, fp32_value, fp32_peak):
    from oracle import oracle as O
    pc = native.params(dt=DT, G=1.0, eps2=EPS * EPS, law=native.LAW_SOFTENED, size=0.0,
                       precision=native.PREC_COMPENSATED)
    p32 = native.params(dt=DT, G=1.0, eps2=EPS * EPS, law=native.LAW_SOFTENED, size=0.0)
    p64 = native.params(dt=DT, G=1.0, eps2=EPS * EPS, law=native.LAW_SOFTENED, size=0.0,
                        precision=native.PREC_FP64)
    out = {}
    with native.Context() as ctx:
        ctx.set_stream(stream.cuda_stream)
        ctx.upload_bodies(bodies)
        # accuracy of each form, from the same initial state
        tg = np.random.default_rng(1003).choice(N, N_SAMPLE, replace=False)
        ctx.accelerate(p32)
        a32 = ctx.download_bodies()[tg, 8:11]
        ctx.accelerate(pc)
        ac = ctx.download_bodies()[tg, 8:11]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a64 = ctx.accel_sampled(p64, tg)
        t64 = time.perf_counter() - t0
        chk = a64[:512]
        ref = O.direct_f64(bodies[:, [0, 1, 2, 7]], 1.0, float(np.float32(EPS * EPS)), O.LAW_SOFTENED,
                           targets=tg[:512])
        fp64_check = float(np.max(np.linalg.norm(chk - ref, axis=1) / np.linalg.norm(ref, axis=1)))
        # throughput of the compensated step
        for _ in range(args.warmup):
            ctx.update(pc, 1)
        torch.cuda.synchronize()
        steps = max(3, args.steps // 2)
        ms = timed_steps(torch, stream, flush, lambda: ctx.update(pc, 1), steps)
        comp_value = N * steps / (sum(ms) * 1e-3)
        acc_ms = statistics.mean(timed_steps(torch, stream, flush, lambda: ctx.accelerate(pc), 2))
        fp64_peak = ctx.calibrate_fp64()
        cfg = ctx.last_direct_config()
    fp64_pairs = float(N_SAMPLE) * N
    out = {
        "value": comp_value, "unit": "body-steps/s", "ratio_vs_fp32": comp_value / fp32_value,
        "ms_per_step": sum(ms) / steps,
        "form": "FP64 origin + FP32 offsets, FP32 pair forces, Kahan over 64-source sub-tiles, FP64 chunk sums, "
                "Kahan-compensated integration",
        "err_vs_fp64": {"fp32": rel_stats(a32, a64), "compensated": rel_stats(ac, a64),
                        "targets": N_SAMPLE, "metric": "|a - a_fp64| / |a_fp64|",
                        "fp64_reference": "GPU FP64 form; max rel. diff. to the CPU FP64 oracle on 512 targets "
                                          f"= {fp64_check:.2e}"},
        "roofline": {"bound": "fp32", "achieved": FLOP_PER_PAIR * float(N) * N / (acc_ms * 1e-3) / 1e12,
                     "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": FLOP_PER_PAIR * float(N) * N / (acc_ms * 1e-3) / 1e12 / fp32_peak,
                     "kernel_ms": acc_ms, "launch": cfg},
        "fp64_form": {"pairs_per_s": fp64_pairs / t64, "seconds": t64, "targets": N_SAMPLE,
                      "peak_dfma_tflops": fp64_peak,
                      "note": "synchronous sampled call incl. upload/readback; ~20 DP flop per pair"},
    }
    return out


# Barnes-Hut opening parameters, in the reference's convention (accept when
# |com - x| > size * theta, bhtree.cpp:117-125): conventional theta = 1 / reference theta.
BH_THETAS = (("theta_0.5", 0.5), ("theta_0.75", 0.75), ("theta_conventional_0.5", 2.0),
             ("theta_conventional_0.75", 4.0 / 3.0))
# compulsory HBM bytes per body of the build (byte model): bounding box 16; Morton codes 16
# read + 12 written; sort: histogram 8, five 9-bit passes x 24, run ordering 12; gather and
# cell sums: order 4 + body 16 + sorted body 16 + prefix 32; radix tree: keys 8 + records 24;
# octree numbering 8; octree records ~70 (0.45 cells per body, each 64 B written and 84 B of
# ranges, prefixes and sums read, and the flags)
BUILD_BYTES_PER_BODY = 16 + 28 + (8 + 5 * 24 + 12) + (4 + 16 + 16 + 32) + (8 + 24) + 8 + 70


def bh_run(torch, stream, flush, native, ctx, bodies, p, steps, warmup, a64, tg, fp32_peak, hbm):
    """One Barnes-Hut configuration: the error of the first accelerate against the FP64 sums
    on the sampled targets, then `steps` timed update steps and the stage times."""
    n = len(bodies)
    ctx.upload_bodies(bodies)
    ctx.accelerate(p)
    err = rel_stats(ctx.download_bodies()[tg, 8:11], a64)
    stats = ctx.bh_stats()
    for _ in range(warmup):
        ctx.update(p, 1)
    torch.cuda.synchronize()
    ms = timed_steps(torch, stream, flush, lambda: ctx.update(p, 1), steps)
    stage = []
    for _ in range(3):
        ctx.update(p, 1)
        stage.append(ctx.bh_stage_ms())
    build_ms = statistics.mean(s[0] for s in stage)
    walk_ms = statistics.mean(s[1] for s in stage)
    ms_step = sum(ms) / steps
    inter = stats["interactions"]
    return {
        "steps_per_s": 1e3 / ms_step, "ms_per_step": ms_step, "body_steps_per_s": n * 1e3 / ms_step,
        "interactions_per_body": inter / n, "tree_cells": stats["cells"],
        "err_vs_fp64": dict(err, targets=len(tg)),
        "stage_ms": {"build": build_ms, "traversal": walk_ms, "integrate_and_rest": ms_step - build_ms - walk_ms,
                     "source": "nbody_cuda_bh_stage_ms (CUDA events), mean of 3 steps"},
        "roofline": {
            "build": {"bound": "hbm", "achieved": n * BUILD_BYTES_PER_BODY / (build_ms * 1e-3) / 1e9, "peak": hbm,
                      "unit": "GB/s", "frac": n * BUILD_BYTES_PER_BODY / (build_ms * 1e-3) / 1e9 / hbm,
                      "peak_source": "MEASURED_PEAKS.json hbm_gbs",
                      "bytes_model": f"{BUILD_BYTES_PER_BODY} B/body compulsory"},
            "traversal": {"bound": "fp32 (interactions at 20 flop each)",
                          "achieved": FLOP_PER_PAIR * inter / (walk_ms * 1e-3) / 1e12, "peak": fp32_peak,
                          "unit": "TFLOP/s", "frac": FLOP_PER_PAIR * inter / (walk_ms * 1e-3) / 1e12 / fp32_peak,
                          "peak_source": "measured FFMA/FFMA2 chains (nbody_cuda_calibrate_fp32)",
                          "interactions_per_s": inter / (walk_ms * 1e-3)},
        },
    }


def energy_drift(ctx, native, bodies, p, steps, e0=None):
    """Relative energy drift and momentum drift of `steps` update steps from `bodies`, from
    nbody_cuda_energy (FP32 pair terms, exact tile folds, FP64 totals) at both ends; e0 is
    the energy of `bodies` when already known (the same law and eps2)."""
    ctx.upload_bodies(bodies)
    if e0 is None:
        e0 = ctx.energy(p)
    t0 = time.perf_counter()
    ctx.update_graph(p, steps)
    ctx.synchronize()
    run_s = time.perf_counter() - t0
    e1 = ctx.energy(p)
    E0, E1 = e0["kinetic"] + e0["potential"], e1["kinetic"] + e1["potential"]
    m = bodies[:, 7].astype(np.float64)
    pscale = float(np.sum(m * np.linalg.norm(bodies[:, 4:7].astype(np.float64), axis=1)))
    return {"steps": steps, "run_s": run_s, "energy_start": E0, "energy_end": E1, "e0": e0,
            "energy_drift": (E1 - E0) / abs(E0),
            "momentum_drift": float(np.linalg.norm(e1["momentum"] - e0["momentum"]) / pscale),
            "momentum_scale": "sum_i m_i |v_i| at the start",
            "diagnostics": "nbody_cuda_energy: FP32 pair terms, tile sums folded exactly, FP64 totals"}


def bench_bh16m(torch, stream, flush, native, scenes, args):
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    t0 = time.perf_counter()
    b = scenes.disk_halo()
    gen_s = time.perf_counter() - t0
    n = len(b)
    eps2 = 0.005 ** 2
    tg = np.random.default_rng(5).choice(n, 4096, replace=False)
    res = {"n_bodies": n, "workload": "exponential disk 12,000,000 (R_d=3, z_0=0.3, circular v) + Hernquist "
                                      "halo 4,777,216 (a=10, m_halo = 5 m_disk), eps=0.005, dt=2.5e-4, "
                                      "FP32 tree forces + compensated integration, auto power-of-two root box",
           "generate_s": gen_s,
           "theta_convention": "keys theta_X use the reference's convention (accept when |com-x| > size*X, "
                               "bhtree.cpp:117-125); theta_conventional_X is the usual one (accept when "
                               "size/|com-x| < X), i.e. reference theta 1/X",
           "walks": {"target": "every target applies exactly the cells the reference's walk accepts for it",
                     "group": "one walk per 128 Morton-consecutive targets (split at the 3 largest Morton jumps), "
                              "cells accepted for a whole sub-group, interaction lists; each target's sources "
                              "refine its reference set"},
           "err_metric": "|a - a_fp64| / |a_fp64| of the first accelerate, 4096 sampled targets; FP64 = GPU FP64 "
                         "direct sum (nbody_cuda_accel_sampled)"}
    steps = max(5, args.steps)
    with native.Context() as ctx:
        ctx.set_stream(stream.cuda_stream)
        fp32_peak = max(ctx.calibrate_fp32())
        ctx.upload_bodies(b)
        a64 = ctx.accel_sampled(native.params(law=native.LAW_SOFTENED, eps2=eps2, precision=native.PREC_FP64), tg)
        for key, theta in BH_THETAS:
            entry = {"theta_reference": theta, "theta_conventional": 1.0 / theta, "per_walk": {}}
            for wname, walk in (("target", native.WALK_TARGET), ("group", native.WALK_GROUP)):
                p = native.params(mode=native.MODE_NLOGN, theta=theta, law=native.LAW_SOFTENED, eps2=eps2,
                                  dt=2.5e-4, size=0.0, tree_box=1, precision=native.PREC_COMPENSATED, walk=walk)
                entry["per_walk"][wname] = bh_run(torch, stream, flush, native, ctx, b, p, steps, args.warmup,
                                                  a64, tg, fp32_peak, hbm)
            # the headline fields: the faster walk (the group walk is at least as accurate)
            fast = min(entry["per_walk"], key=lambda w: entry["per_walk"][w]["ms_per_step"])
            entry = {**entry, "walk": fast, **entry["per_walk"][fast]}
            res[key] = entry
        # 100 steps (config 5) at conventional theta 0.5 and at reference theta 0.5, the faster
        # walk each, energy and momentum drift from the diagnostics at both ends
        res["drift_100_steps"] = {}
        e0 = None
        for key in ("theta_conventional_0.5", "theta_0.5"):
            theta = res[key]["theta_reference"]
            walk = native.WALK_GROUP if res[key]["walk"] == "group" else native.WALK_TARGET
            p = native.params(mode=native.MODE_NLOGN, theta=theta, law=native.LAW_SOFTENED, eps2=eps2, dt=2.5e-4,
                              size=0.0, tree_box=1, precision=native.PREC_COMPENSATED, walk=walk)
            d = energy_drift(ctx, native, b, p, 100, e0)
            e0 = d.pop("e0")
            res["drift_100_steps"][key] = dict(d, walk=res[key]["walk"])
        p = native.params(mode=native.MODE_NLOGN, theta=0.5, law=native.LAW_SOFTENED, eps2=eps2,
                          dt=2.5e-4, size=0.0, tree_box=1, precision=native.PREC_COMPENSATED)
        res["transfer"] = bench_transfer(torch, native, ctx, b, p)
    # one full step of the restated CPU Barnes-Hut on the same bodies, on all host cores:
    # the reference's fixed root box (centred at the origin), made a power of two that holds
    # every body; the GPU arm's softened law
    size = float(2.0 ** np.ceil(np.log2(2.0 * float(np.abs(b[:, :3]).max()))))
    cpu_s, cores = cpu_barnes_hut_rate(b, size, 0.5, eps2)
    res["cpu_reference_bh"] = {
        "theta": 0.5, "step_s": cpu_s, "cores": cores, "body_steps_per_s": n / cpu_s,
        "kind": "port (restated CpuBarnesHutSolver, cpu_barnes_hut.h:22-44: serial tree build, "
                "parallel traversal; softened law as the GPU arm)",
        "root_box": f"centred at the origin, edge {size:g}",
        "gpu_speedup": cpu_s / (res["theta_0.5"]["ms_per_step"] * 1e-3)}
    return res


def bench_transfer(torch, native, ctx, bodies, p, reps=3):
    """Host transfers of all N Body records (48 B each) on each path, against the copy
    engine's own pinned-memory bandwidth for the same bytes (the link roofline), and one
    frame of the reference's read-every-frame loop: update(dt) then state()."""
    n = len(bodies)
    nbytes = n * 48
    host = np.empty_like(bodies)

    def best(fn):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return min(ts)

    dev = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
    pin = torch.empty(nbytes // 4, dtype=torch.float32, pin_memory=True)
    ce_d2h = nbytes / best(lambda: (pin.copy_(dev, non_blocking=True), torch.cuda.synchronize())) / 1e9
    ce_h2d = nbytes / best(lambda: (dev.copy_(pin, non_blocking=True), torch.cuda.synchronize())) / 1e9
    del dev, pin
    info = ctx.transfer_info()
    out = {"n_bodies": n, "bytes": nbytes, "pageable_access": info["pageable"],
           "auto_resolves_to": {1: "staged", 2: "mapped", 3: "direct"}[info["resolved"]],
           "copy_engine_gbs": {"d2h_pinned": ce_d2h, "h2d_pinned": ce_h2d},
           "caller_memory": "pageable numpy array", "timing": "host wall clock, best of %d" % reps}
    names = {native.TRANSFER_STAGED: "staged", native.TRANSFER_MAPPED: "mapped", native.TRANSFER_DIRECT: "direct"}
    ctx.upload_bodies(bodies)
    for pol, name in names.items():
        try:
            ctx.set_transfer(pol)
        except native.NbodyError as e:
            out[name] = {"unavailable": str(e)}
            continue
        up = best(lambda: ctx.upload_bodies(bodies))
        down = best(lambda: ctx.download_bodies(into=host))
        pos = best(lambda: ctx.download_bodies(mask=native.READ_POSITIONS, into=host))
        out[name] = {"upload_ms": up * 1e3, "upload_gbs": nbytes / up / 1e9,
                     "download_ms": down * 1e3, "download_gbs": nbytes / down / 1e9,
                     "download_positions_ms": pos * 1e3,
                     "roofline": {"bound": "host link", "unit": "GB/s", "peak_source": "copy engine, same bytes",
                                  "download_frac": nbytes / down / 1e9 / ce_d2h,
                                  "upload_frac": nbytes / up / 1e9 / ce_h2d}}
    ctx.upload_bodies(bodies)
    frames = {}
    for pol, name in names.items():
        try:
            ctx.set_transfer(pol)
        except native.NbodyError:
            continue
        def frame():
            ctx.update(p, 1)
            ctx.prefetch(native.READ_ALL)       # the prediction of a read-every-frame caller
            ctx.download_bodies(into=host)
        frames[name] = best(frame) * 1e3
    ctx.set_transfer(native.TRANSFER_AUTO)
    frames["step_only"] = best(lambda: (ctx.update(p, 1), ctx.synchronize())) * 1e3
    out["frame_ms"] = frames
    out["frame_note"] = ("BH theta=0.5 step (compensated integration) + full Body readback into the caller's "
                         "array, per path; step_only is the same step without the readback")
    return out


def bench_scenes(torch, stream, native, reps=5):
    """util::disk and util::cube generated on the device at N = 16,777,216, against the
    reference's serial generator (oracle/_ref where it loads, else the oracle's bit-exact
    restatement) on a bounded sample of 1,048,576 bodies."""
    from oracle import oracle as O
    n = 1 << 24
    hbm = measured_peaks().get("hbm_gbs", 6800.0)
    out = {"n_bodies": n, "args": "the reference's defaults (disk: outer radius 250, central mass 4.1e6; cube: edge 500)"}
    with native.Context() as ctx:
        ctx.set_stream(stream.cuda_stream)
        for kind in ("disk", "cube"):
            gen = getattr(ctx, f"scene_{kind}")
            gen(n)
            torch.cuda.synchronize()
            ms = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                gen(n)
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            best = min(ms)
            out[kind] = {"device_ms": best, "bodies_per_s": n / (best * 1e-3),
                         "roofline": {"bound": "issue (integer mulmod jump-ahead, FP64 sin/cos/log)",
                                      "achieved": n * 48 / (best * 1e-3) / 1e9, "peak": hbm, "unit": "GB/s",
                                      "frac": n * 48 / (best * 1e-3) / 1e9 / hbm,
                                      "note": "48 B written per body against the measured HBM copy bandwidth"}}
    sample = 1 << 20
    ref = O.ref_lib() is not None
    t0 = time.perf_counter()
    if ref:
        O.ref_disk_range(np.zeros((sample, 12), np.float32), 0, sample)
    else:
        O.disk(sample)
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": sample / cpu_s, "unit": "bodies/s", "cores": 1,
                           "kind": "reference" if ref else "port",
                           "sample": "util::disk, 1,048,576 bodies (the reference's generator is serial)"}
    out["disk_speedup_vs_cpu"] = out["disk"]["bodies_per_s"] / out["cpu_baseline"]["value"]
    return out


def bench_query(native, scenes):
    """Tree::query for many rays over the exported Barnes-Hut tree of a 1,048,576-body
    Plummer sphere: picking rays (stop at the first body leaf) and full walks, through the
    C ABI with host ray and hit arrays, against the oracle's walk on one host core."""
    from oracle import oracle as O
    n = 1 << 20
    b = scenes.plummer(n, seed=2)
    g = np.random.default_rng(1)
    out = {"n_bodies": n}
    with native.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.accelerate(native.params(mode=native.MODE_NLOGN, theta=0.5, law=native.LAW_SOFTENED, eps2=1e-4,
                                     size=0.0, tree_box=1))
        t0 = time.perf_counter()
        nodes = ctx.tree_export()
        out["tree_nodes"] = len(nodes)
        out["export_ms"] = (time.perf_counter() - t0) * 1e3
        for name, nr, stop, mh in (("picking", 1 << 20, native.QUERY_FIRST_BODY, 64),
                                   ("full_walk", 1 << 16, native.QUERY_ALL, 256)):
            rays = np.concatenate([g.normal(0, 3, (nr, 3)), g.normal(0, 1, (nr, 3))], 1).astype(np.float32)
            ctx.tree_query(rays[:1024], stop, mh)
            t0 = time.perf_counter()
            _, counts = ctx.tree_query(rays, stop, mh)
            t = time.perf_counter() - t0
            k = 2000
            t0 = time.perf_counter()
            for r in range(k):
                O.tree_query(nodes, rays[r], stop, mh)
            tc = time.perf_counter() - t0
            out[name] = {"rays": nr, "ms": t * 1e3, "rays_per_s": nr / t, "mean_nodes_visited": float(counts.mean()),
                         "cpu_baseline": {"value": k / tc, "unit": "rays/s", "cores": 1, "kind": "port",
                                          "sample": "%d rays, the restated Tree::query walk" % k},
                         "speedup_vs_cpu": (nr / t) / (k / tc)}
    out["note"] = "wall clock of nbody_cuda_tree_query including the ray upload and hit download"
    return out


def fp64_euler_drift(bodies, eps2, dt, steps):
    """Relative energy drift of an FP64 semi-implicit Euler run (CPU oracle), for comparing
    the FP32 batched run's drift against FP64 arithmetic on the same system."""
    from oracle import oracle as O
    pos = bodies[:, :3].astype(np.float64)
    vel = bodies[:, 4:7].astype(np.float64)
    m = bodies[:, 7].astype(np.float64)
    ke, pe, _ = O.energy_f64(pos, vel, m, 1.0, eps2)
    e0 = ke + pe
    for _ in range(steps):
        vel = vel + O.direct_f64_pos(pos, m, 1.0, eps2) * dt
        pos = pos + vel * dt
    ke, pe, _ = O.energy_f64(pos, vel, m, 1.0, eps2)
    return abs((ke + pe - e0) / e0)


def bench_batched(torch, stream, flush, native, scenes, direct_pairs_per_s):
    """Config 4: 512 Plummer systems, N log-uniform in [64, 8192], eps 0.01, dt 1e-3, 1000
    steps: autotuned persistent kernel, each step replayed from a CUDA graph."""
    b, off = scenes.batch_plummer()
    sizes = np.diff(off)
    pairs = float(np.sum(sizes.astype(np.float64) ** 2))
    eps2 = float(np.float32(1e-4))
    p = native.params(mode=native.MODE_BATCHED, law=native.LAW_SOFTENED, eps2=1e-4, dt=1e-3, size=0.0)
    steps = 1000
    with native.Context() as ctx:
        ctx.set_stream(stream.cuda_stream)
        ctx.upload_bodies(b)
        ctx.set_systems(off)
        best, times = ctx.batch_autotune(p)
        e0 = ctx.system_energy(p)
        ctx.update_graph(p, 2)          # capture
        torch.cuda.synchronize()
        launches0 = ctx.launches()
        ms = timed_steps(torch, stream, flush, lambda: ctx.update_graph(p, steps), 1)[0]
        launches = ctx.launches() - launches0
        e1 = ctx.system_energy(p)
        cfg = ctx.batch_config(-1)
    E0, E1 = e0[:, 0] + e0[:, 1], e1[:, 0] + e1[:, 1]
    drift = np.abs((E1 - E0) / E0)
    small = np.argsort(sizes)[:6]
    # FP64 reference runs of the smallest systems over the same 1002 steps
    ref = {int(s): fp64_euler_drift(b[off[s]:off[s + 1]], eps2, 1e-3, steps + 2) for s in small}
    per_step_ms = ms / steps
    return {
        "systems": len(sizes), "bodies": int(off[-1]), "pairs_per_step": pairs,
        "steps": steps, "ms": ms, "ms_per_step": per_step_ms,
        "body_steps_per_s": float(off[-1]) * steps / (ms * 1e-3),
        "pairs_per_s": pairs / (per_step_ms * 1e-3),
        "ratio_vs_single_system_direct": pairs / (per_step_ms * 1e-3) / direct_pairs_per_s,
        "kernel_launches": launches,
        "autotune": {"best": best, "config": cfg, "accelerate_ms_per_config": [float(t) for t in times]},
        "energy_drift_fp64_diagnostics": {"median": float(np.median(drift)), "p99": float(np.percentile(drift, 99)),
                                          "max": float(drift.max())},
        "energy_drift_vs_fp64_run": {str(s): {"n": int(sizes[s]), "fp32_batched": float(drift[s]),
                                             "fp64_euler": ref[s]} for s in ref},
        "note": "512 log-uniform draws in [64, 8192] average ~0.86M bodies; this seed gives the total above",
    }


def bench_small_configs(torch, stream, flush, native, scenes):
    out = {}
    # config 1: N=4096 Plummer, 100 steps, FP32, eps 0.01, steps replayed from a CUDA graph
    b = scenes.plummer(4096, seed=1001)
    p = native.params(dt=1e-3, eps2=1e-4, law=native.LAW_SOFTENED, size=0.0)
    with native.Context() as ctx:
        ctx.set_stream(stream.cuda_stream)
        ctx.upload_bodies(b)
        ctx.update_graph(p, 3)
        torch.cuda.synchronize()
        ms = timed_steps(torch, stream, flush, lambda: ctx.update(p, 100), 1)[0]
        ms_graph = timed_steps(torch, stream, flush, lambda: ctx.update_graph(p, 100), 1)[0]
    # FP64 error of the first accelerate (all 4096 bodies, CPU FP64 oracle)
    from oracle import oracle as O
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED)
    with native.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.accelerate(p)
        err = rel_stats(ctx.download_bodies()[:, 8:11], a64)
    cpu_s, cores, kind = cpu_config1_seconds(b, 100, 1e-3, 1e-4)
    out["config1_plummer_4096"] = {"steps": 100, "ms_eager": ms, "ms_graph": ms_graph,
                                   "body_steps_per_s": 4096 * 100 / (min(ms, ms_graph) * 1e-3),
                                   "err_vs_fp64": dict(err, targets=4096),
                                   "cpu_100_steps_s": cpu_s, "cpu_body_steps_per_s": 4096 * 100 / cpu_s,
                                   "cpu_cores": cores, "cpu_kind": kind}
    # config 2: two Plummer spheres of 131072, eps 0.01, dt 5e-4, 200 steps, the reference's
    # fixed 64 box; reference theta 0.5 and conventional theta 0.5, both walks; FP64 errors
    # of the first accelerate on 4096 sampled targets (CPU FP64 oracle)
    b = scenes.two_plummer(131072)
    tg = np.random.default_rng(2).choice(len(b), 4096, replace=False)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED, targets=tg)
    c2 = {"n_bodies": len(b), "steps": 200, "err_metric": "|a - a_fp64| / |a_fp64|, 4096 sampled targets"}
    for key, theta in (("theta_0.5", 0.5), ("theta_conventional_0.5", 2.0)):
        entry = {"theta_reference": theta, "per_walk": {}}
        for wname, walk in (("target", native.WALK_TARGET), ("group", native.WALK_GROUP)):
            p = native.params(mode=native.MODE_NLOGN, theta=theta, dt=5e-4, eps2=1e-4, law=native.LAW_SOFTENED,
                              size=64.0, walk=walk)
            with native.Context() as ctx:
                ctx.set_stream(stream.cuda_stream)
                ctx.upload_bodies(b)
                ctx.accelerate(p)
                err = rel_stats(ctx.download_bodies()[tg, 8:11], a64)
                stats = ctx.bh_stats()
                ctx.update(p, 3)
                ctx.update_graph(p, 3)
                torch.cuda.synchronize()
                ms_eager = timed_steps(torch, stream, flush, lambda: ctx.update(p, 200), 1)[0]
                ms_graph = timed_steps(torch, stream, flush, lambda: ctx.update_graph(p, 200), 1)[0]
            ms = min(ms_eager, ms_graph)
            entry["per_walk"][wname] = {"ms": ms, "ms_eager": ms_eager, "ms_graph": ms_graph,
                                        "steps_per_s": 200 / (ms * 1e-3),
                                        "body_steps_per_s": len(b) * 200 / (ms * 1e-3),
                                        "interactions_per_body": stats["interactions"] / len(b),
                                        "err_vs_fp64": dict(err, targets=len(tg))}
        fast = min(entry["per_walk"], key=lambda w: entry["per_walk"][w]["ms"])
        c2[key] = {**entry, "walk": fast, **entry["per_walk"][fast]}
    cpu_s, cores = cpu_barnes_hut_rate(b, 64.0, 0.5, float(np.float32(1e-4)))
    c2.update({"cpu_reference_bh_step_s": cpu_s, "cpu_cores": cores,
               "cpu_kind": "port (restated CpuBarnesHutSolver, serial build, softened law), reference theta 0.5"})
    out["config2_two_plummer_bh"] = c2
    return out


def bench_reference(args):
    """The reference's CPU brute force (CpuBruteForceSolver::accelerate, cpu_brute_force.h:17-43,
    restated in the oracle, speed build) with the GPU arm's softened law, on all host cores.
    A step is a bounded sample of the workload: k targets spread over the N bodies, each
    summed against all N sources and integrated (physics.h:60-70); body-steps/s counts the k.
    ms_per_step is that sample's own time, so steps x ms_per_step is the timed region."""
    rank, world, _ = env_rank()
    if rank != 0:
        return None
    from nbody_gb300 import scenes
    from oracle import oracle as O
    bodies = scenes.uniform_cube(N, seed=1003)
    threads = O.threads()
    eps2 = EPS * EPS
    target_s = max(0.5, args.cpu_seconds / 5)

    def step(tg):
        acc = O.brute_force_targets(bodies, 1.0, tg, nthreads=threads, law=O.LAW_SOFTENED, eps2=eps2, timing=True)
        sub = bodies[tg].copy()
        sub[:, 8:11] = acc
        return O.integrate(sub, DT, 10000.0, False)

    k = 256
    while True:                 # size a step to about target_s seconds
        tg = np.linspace(0, N - 1, k).astype(np.int64)
        t0 = time.perf_counter()
        step(tg)
        dt = time.perf_counter() - t0
        if dt >= 0.5 * target_s or k >= N:
            break
        k = min(N, int(k * min(8.0, max(1.5, target_s / max(dt, 1e-3)))))
    tg = np.linspace(0, N - 1, k).astype(np.int64)
    for _ in range(args.warmup):
        step(tg)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step(tg)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = k * args.steps / total
    sample = (f"{k} targets spread over the {N} bodies, each against all {N} sources (restated reference "
              f"brute force, softened law as the GPU arm, speed build) and integrated, per step")
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
        "config": {"workload": WORKLOAD, "n_bodies": N, "eps": EPS, "dt": DT, "law": "softened",
                   "same_config": True, "bodies_per_step": k,
                   "note": "the GPU arm's workload and law; a step is a bounded sample of k of its N bodies"},
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": threads, "kind": "port",
                         "sample": sample, "pairs_per_s": k * N * args.steps / total},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--quick", action="store_true", help="headline workload only (for profiler captures)")
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
