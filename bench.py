"""Benchmark of the ray-integration hot path on GB300.

Workload (default): the plain FP64 drop-in case -- 65,536 rays over a
2,001 x 2,001 seamount grid at 50 m with a uniform (0.5, 0) m/s current grid,
dt = 1 s, 4,000 RK4 steps, full trajectories (10.5 GB per step).  One bench
step = one trace call over all rays.  Metric: ray-steps/s (one ray-step = one
RK4 step = four right-hand-side evaluations).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun each rank traces its own copy of the workload (rays are
independent, no collective; weak scaling) and rank 0 prints one JSON line.
`--impl reference` times the CPU restatement of the reference path on the
host cores instead (rank 0 only).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from mantaray_gb300.distributed import reduce_scalar  # noqa: E402

METRIC = "ray-steps/s"
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2

# Algorithmic work of one ray-step of the plain FP64 form over f64 grids:
# 4 stages x 3 fields (h, u, v) x 4 corners x 8 B of grid gathers, plus one
# stored 40 B output row (t, x, y, kx, ky).
GRID_BYTES_PER_RAY_STEP = 4 * 3 * 4 * 8
OUT_BYTES_PER_ROW = 5 * 8
# FP32 floating-point operations one ray-step of the batched kernel executes
# (FADD/FMUL = 1, FFMA = 2), counted by ncu on the 4,096^2 shelf-slope case
# with the current on the bathymetry's grid (92.0 FFMA, 36.0 FADD, 36.1 FMUL).
FP32_FLOP_PER_RAY_STEP = 256.2
# Algorithmic work of one ray-step (the reference's arithmetic, hand count from
# src/wave_ray_path.rs:118-216 plus the RK4 update): ~55 FP64 add/mul/div per
# right-hand side x 4 + ~53 for the update = 270 (36 transcendental calls not
# counted); its f32 interpolation adds ~440 FP32 operations (4 stages x 3
# bilinears of ~35 operations, plus index arithmetic).  The batched form does
# all of it in FP32: 710.
ALG_FP64_FLOP_PER_RAY_STEP = 270.0
ALG_FP32_FLOP_PER_RAY_STEP = 710.0
# FP64 floating-point operations one ray-step executes (DADD/DMUL = 1,
# DFMA = 2), per right-hand-side arithmetic, counted by ncu on the plain
# kernel over the seamount workload's whole 4,000-step horizon (20,480 of its
# rays, 79.3 M ray-steps; sm__sass_thread_inst_executed_op_d{add,mul,fma}_pred_on).
FP64_FLOP_PER_RAY_STEP = {"libm": 1399.1, "identity": 221.9}
# FP64-pipe instructions per ray-step (sm__inst_executed_pipe_fp64 x 32: warp
# instructions in lane slots, so lanes idle in a divergent warp count; same
# captures), of the build the 65,536-ray benchmark runs: identity with the
# lookup cache, libm without (its cached build does not fit one wave)
FP64_PIPE_INST_PER_RAY_STEP = {"libm": 974.4, "identity": 225.4}
# DRAM bytes (read + written) per stored trajectory row of the plain kernel
# on the seamount workload: ncu dram__bytes_read.sum + dram__bytes_write.sum
# of one launch over its 65,536 rays x 1,000 steps (55.5 MB read, 2,573.7 MB
# written: the 2.62 GB of stored rows, 20x L2, less what L2 still held at the
# end) over its 65,536 x 1,001 rows.  Scaled by rows (NaN padding included:
# a ray that stops early still writes its padding rows), not ray-steps.
K1_DRAM_BYTES_PER_ROW = (55537408 + 2573673472) / (65536 * 1001)
K1_DRAM_NOTE = ("ncu DRAM bytes of a 65,536-ray x 1,000-step launch of the same workload "
                "(55.5 MB read, 2,573.7 MB written) scaled by stored rows (rays x rows, NaN "
                "padding included); rows still in L2 at the end of that launch (at most 129 MB) "
                "are not counted")
# The same for the batched kernel on the shelf-slope field: one graph-replayed
# call on the field's generator at 4,096^2 (records 1.3 GB, 10x L2) with the
# 8,192^2 case's ray density, 5,466,581 rays traced to their ends (49.64 G
# ray-steps), launch 128 x 12, ordered: the sum over the call's K2 launches,
# by sweep length (0: one launch; in sweeps the bytes include the running
# rays' states written and read between sweeps).  Its rays spread over the
# field as the 8,192^2 case's do, so the bytes scale with ray-steps.
K2_SHELF_RAY_STEPS = 49640953115
K2_SHELF_DRAM_BYTES = {0: (1690693872640, 1447764224), 128: (98504049152, 28714596608),
                       256: (61612061696, 15217717760)}


def k2_shelf_dram(sweep_steps: int):
    """DRAM bytes per ray-step of the batched kernel on the shelf-slope field
    for a sweep length (the nearest captured one), and its note."""
    s = 0
    if sweep_steps > 0:
        s = min((k for k in K2_SHELF_DRAM_BYTES if k > 0), key=lambda k: abs(k - sweep_steps))
    rd, wr = K2_SHELF_DRAM_BYTES[s]
    return (rd + wr) / K2_SHELF_RAY_STEPS, (
        f"ncu DRAM bytes of one call of the same generator at 4,096^2 and the same ray density "
        f"({'one launch' if s == 0 else f'sweeps of {s} steps'}; {(rd + wr) / K2_SHELF_RAY_STEPS:.2f} B "
        f"per ray-step), scaled by this call's ray-steps")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--rays", type=int, default=65536)
    p.add_argument("--trace-steps", type=int, default=4000)
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="wall-time budget of the CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--math", default="identity", choices=["identity", "libm"],
                   help="right-hand-side arithmetic of the plain FP64 kernel")
    p.add_argument("--form", default="plain", choices=["plain", "batched", "adjoint"],
                   help="plain FP64 drop-in (default), the batched FP32 form, or the "
                        "differentiation form (adjoint vs forward time)")
    p.add_argument("--precision", type=int, default=64, choices=[64, 32],
                   help="adjoint form: FP64 or FP32 arithmetic")
    p.add_argument("--workload", default="seamount",
                   choices=["seamount", "planar_beach", "shelf_bump", "shelf_slope",
                            "multi_source"],
                   help="plain form: seamount (default), planar_beach, shelf_bump; batched "
                        "form: seamount, the 8192^2 shelf-slope case (graph-replayed calls "
                        "with varied ray counts) or the 8-scenario multi-source case")
    p.add_argument("--grid", type=int, default=None, help="grid points per axis override")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--launch", default=None,
                   help="batched form: fixed launch shape 'block,blocks_per_sm,rays_per_lane,"
                        "order[,staging[,sweep_steps]]' instead of the autotuner's")
    # the target measurements reported beside the plain form's line
    p.add_argument("--no-north-star", action="store_true",
                   help="plain form: skip the shelf-slope batched-vs-plain and adjoint-vs-"
                        "forward measurements reported in the line's north_star object")
    p.add_argument("--ns-rays", type=int, default=16777216,
                   help="shelf-slope: nominal rays per call (each call traces 0.5-1.5x)")
    p.add_argument("--ns-grid", type=int, default=8192, help="shelf-slope: grid points per axis")
    p.add_argument("--ns-steps", type=int, default=50000, help="shelf-slope: step horizon")
    p.add_argument("--ns-calls", type=int, default=6,
                   help="shelf-slope: timed graph-replayed calls")
    p.add_argument("--ns-warmup", type=int, default=2, help="shelf-slope: untimed calls")
    p.add_argument("--ns-plain-rays", type=int, default=1048576,
                   help="shelf-slope: rays of the plain FP64 form's rate measurement (2^20: "
                        "enough to fill the GPU as the rays end; 2^18 ran 13% slower)")
    p.add_argument("--ns-plain-chunk", type=int, default=2500,
                   help="shelf-slope: steps per plain FP64 launch (memory of full trajectories)")
    p.add_argument("--ns-error-rays", type=int, default=4096,
                   help="shelf-slope: rays of the endpoint-error comparison")
    p.add_argument("--ns-adjoint-calls", type=int, default=2,
                   help="differentiation case: timed forward and gradient calls per precision")
    p.add_argument("--ns-only", action="store_true",
                   help="print only the shelf-slope batched-vs-plain measurement (for profiling)")
    return p.parse_args()


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def cpu_sample(w, seconds: float, threads: int):
    """Times the oracle (CPU restatement of the reference path, OpenMP over
    rays) on successive batches of the workload's rays until `seconds` pass.
    After a first batch of 16 rays per thread the batches grow to fill the
    remaining time, so one long ray does not leave the other threads idle at
    the end of every batch.  Returns (ray-steps/s, description, seconds)."""
    from oracle import pyoracle

    ob = pyoracle.Bathymetry.grid(w.bx, w.by, w.depth)
    oc = pyoracle.Current.grid(w.cx, w.cy, w.u, w.v)
    batch = max(threads * 16, 256)
    done_rays = 0
    ray_steps = 0
    sizes = []
    t_start = time.perf_counter()
    i = 0
    while True:
        idx = np.arange(i, i + batch) % w.n
        t_b = time.perf_counter()
        traj, n_rows, _ = pyoracle.trace(ob, oc, w.x0[idx], w.y0[idx], w.kx0[idx], w.ky0[idx],
                                         w.t0, w.t_end, w.dt, threads=threads)
        t_b = time.perf_counter() - t_b
        ray_steps += int(np.sum(n_rows.astype(np.int64) - 1))
        done_rays += batch
        sizes.append(batch)
        i += batch
        elapsed = time.perf_counter() - t_start
        if elapsed >= seconds:
            break
        # next batch: about half the remaining time, within memory bounds
        rows = int(round((w.t_end - w.t0) / w.dt)) + 1
        cap = max(256, int(2e9 // (5 * 8 * rows)))
        batch = int(min(cap, max(batch, batch * 0.5 * (seconds - elapsed) / max(t_b, 1e-3))))
    desc = (f"{done_rays} of the workload's rays (batches of {min(sizes)} to {max(sizes)}) x up "
            f"to {int(round((w.t_end - w.t0) / w.dt))} steps with full trajectories, "
            f"{threads} OpenMP threads, {elapsed:.1f} s wall")
    return ray_steps / elapsed, desc, elapsed


def cpu_baseline(w, seconds: float) -> dict:
    """The cpu_baseline object: the oracle on all host cores for `seconds`,
    and on one core for a quarter of that (value_1thread)."""
    threads = cpu_threads()
    rate, desc, _ = cpu_sample(w, seconds, threads)
    rate1, desc1, _ = cpu_sample(w, max(seconds / 4.0, 1.0), 1)
    return {"value": rate, "unit": METRIC, "cores": threads, "kind": "port", "sample": desc,
            "value_1thread": rate1, "sample_1thread": desc1}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


PLAIN_WORKLOADS = ("seamount", "planar_beach", "shelf_bump")


def plain_workload(args):
    """The plain form's workload: the seamount case (default), the planar beach
    (1,024 rays x 2,000 steps) or the shelf-bump differentiation field traced
    forward (262,144 rays x 3,000 steps)."""
    from mantaray_gb300 import workloads as W

    if args.workload == "seamount":
        return W.seamount(n_rays=args.rays, steps=args.trace_steps)
    if args.workload == "planar_beach":
        return W.planar_beach(n_rays=args.rays if args.rays != 65536 else 1024)
    if args.workload == "shelf_bump":
        return W.shelf_bump(n_rays=args.rays if args.rays != 65536 else 262144,
                            steps=args.trace_steps if args.trace_steps != 4000 else 3000)
    raise SystemExit(f"--workload {args.workload} runs in the batched form only")


def grid_desc(w) -> str:
    return f"{w.depth.shape[1]}x{w.depth.shape[0]} f64 depth/u/v"


def reference_arm(args, rank: int, world: int):
    """The reference's CPU path (the oracle port: the Rust crate cannot be
    built here) on the host cores, each step a bounded sample."""
    if rank != 0:
        return
    w = plain_workload(args)
    threads = cpu_threads()
    per_step = max(args.cpu_seconds / 4.0, 1.0)
    for _ in range(args.warmup):
        cpu_sample(w, per_step / 4.0, threads)
    rates, descs, times = [], [], []
    for _ in range(args.steps):
        r, d, t = cpu_sample(w, per_step, threads)
        rates.append(r)
        descs.append(d)
        times.append(t)
    value = statistics.mean(rates)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": w.name, "rays": w.n, "grid": grid_desc(w), "dt": w.dt,
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": descs[-1]},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def gb300_arm(args, rank: int, world: int, local_rank: int):
    import torch

    import mantaray_gb300 as mr

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()

    w = plain_workload(args)
    b = mr.Bathymetry.grid(w.bx, w.by, w.depth)
    c = mr.Current.grid(w.cx, w.cy, w.u, w.v)
    rows = mr.num_steps(w.t0, w.t_end, w.dt) + 1
    n = w.n
    ins = [torch.from_numpy(a).to(dev) for a in (w.x0, w.y0, w.kx0, w.ky0)]
    traj = torch.empty((5, rows, n), dtype=torch.float64, device=dev)
    n_rows = torch.empty(n, dtype=torch.int32, device=dev)
    status = torch.empty(n, dtype=torch.uint8, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def one(math=args.math):
        mr.trace_device(b, c, *ins, w.t0, w.t_end, w.dt, traj, n_rows, status, math=math,
                        stream=stream)

    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()

    # ---- device-resident throughput (value) ----
    times = []
    launches = 0
    with ClockSampler(local_rank) as clocks:
        barrier()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.fill_(1.0)  # evict L2 between timed steps (not timed)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one()
            e1.record(stream)
            launches += 1
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        torch.cuda.synchronize()
        barrier()
    clock = clocks.summary()
    ray_steps = int(torch.sum(n_rows.to(torch.int64) - 1).item())
    local_t = sum(times)
    t_max = reduce_scalar(local_t, "max") if dist is not None else local_t
    total_ray_steps = ray_steps * args.steps * world
    value = total_ray_steps / t_max
    kernel_s = local_t / args.steps

    # ---- the other right-hand-side arithmetic, same workload (reported only) ----
    alt_math = "libm" if args.math == "identity" else "identity"
    one(alt_math)
    torch.cuda.synchronize()
    alt_times = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        one(alt_math)
        e1.record(stream)
        e1.synchronize()
        alt_times.append(e0.elapsed_time(e1) / 1e3)
    alt_rate = int(torch.sum(n_rows.to(torch.int64) - 1).item()) * args.steps / sum(alt_times)

    # ---- end-to-end through the C ABI with host buffers (e2e) ----
    e2e = None
    if not args.no_e2e:
        hin = [torch.from_numpy(a.copy()).pin_memory() for a in (w.x0, w.y0, w.kx0, w.ky0)]
        hout = torch.empty((5, rows, n), dtype=torch.float64, pin_memory=True)
        hout_np = hout.numpy()
        h_np = [t.numpy() for t in hin]
        mr.trace(b, c, *h_np, w.t_end - w.t0, w.dt, t0=w.t0, out=hout_np, math=args.math)  # warm-up
        barrier()
        e2e_times = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = mr.trace(b, c, *h_np, w.t_end - w.t0, w.dt, t0=w.t0, out=hout_np, math=args.math)
            e2e_times.append(time.perf_counter() - t0)
        barrier()
        e2e_local = sum(e2e_times)
        e2e_max = reduce_scalar(e2e_local, "max") if dist is not None else e2e_local
        e2e_steps = int(np.sum(res.n_rows.astype(np.int64) - 1))
        e2e = {"value": e2e_steps * args.steps * world / e2e_max, "unit": METRIC,
               "h2d_bytes_per_step": 4 * n * 8,
               "d2h_bytes_per_step": 5 * rows * n * 8 + n * 4 + n,
               "path": "mr_trace (C ABI), page-locked host buffers; the kernel stores "
                       "trajectories straight into host memory",
               "ms_per_step": 1e3 * e2e_local / args.steps}
        del hout, hin

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel (rk4_f64) ----
    L = mr._native.load()
    import ctypes

    fp64_peak = ctypes.c_double()
    mr._native.check(L.mr_measure_fma_peak(1, ctypes.byref(fp64_peak)))
    rs_per_s_kernel = ray_steps / kernel_s
    hbm_achieved = rs_per_s_kernel * (GRID_BYTES_PER_RAY_STEP + OUT_BYTES_PER_ROW) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # achieved = the algorithmic FP64 work of a ray-step (ALG_FP64_FLOP_PER_RAY_STEP)
    # x ray-steps per second of the kernel; the executed work (ncu) beside it
    fp64_achieved = rs_per_s_kernel * ALG_FP64_FLOP_PER_RAY_STEP / 1e12
    exec_flop = FP64_FLOP_PER_RAY_STEP[args.math]
    roofline = {"bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak.value,
                "unit": "TFLOP/s", "frac": fp64_achieved / fp64_peak.value,
                "peak_source": "measured: FP64 FMA-chain kernel on this GPU, this run",
                "flop_per_ray_step": ALG_FP64_FLOP_PER_RAY_STEP,
                "flop_note": "algorithmic: 4 x ~55 RHS + ~53 RK4-update FP64 add/mul/div per "
                             "ray-step (the reference's expressions); its 36 transcendental "
                             "calls are not counted",
                "executed_flop_per_ray_step": exec_flop,
                "executed_frac": rs_per_s_kernel * exec_flop / 1e12 / fp64_peak.value,
                "pipe_issue_frac": rs_per_s_kernel * FP64_PIPE_INST_PER_RAY_STEP[args.math]
                / (fp64_peak.value * 1e12 / 2.0),
                "pipe_issue_note": "FP64-pipe instructions/s (ncu count per ray-step) over the "
                                   "FMA-chain DFMA/s"}
    roofline["hbm"] = {"achieved": hbm_achieved, "peak": hbm_peak, "unit": "GB/s",
                       "frac": hbm_achieved / hbm_peak,
                       "bytes_per_ray_step": GRID_BYTES_PER_RAY_STEP + OUT_BYTES_PER_ROW,
                       "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"}
    # DRAM bytes of one launch: the algorithmic floor (the trajectory rows the
    # launch must store, NaN padding included) and the ncu count of a capture
    # whose stored rows dwarf L2, scaled by stored rows
    must_store = 5 * 8 * rows * n + n * 5
    roofline["traffic_floor"] = must_store
    if args.workload == "seamount":
        roofline["traffic"] = K1_DRAM_BYTES_PER_ROW * rows * n
        roofline["traffic_note"] = K1_DRAM_NOTE
    else:
        roofline["traffic"] = None
        roofline["traffic_note"] = "no ncu capture of this workload"
    if args.workload != "seamount":
        roofline["executed_note"] = "executed counts from ncu on the seamount workload"
    roofline["kernel_ms"] = 1e3 * kernel_s

    # free the headline's buffers before the target measurements
    del traj, n_rows, status, ins
    torch.cuda.empty_cache()
    north = None
    if not args.no_north_star and world == 1:
        north = {"batched_fp32": north_star_batched(args, dev, stream, flush),
                 "adjoint": north_star_adjoint(args, dev, stream)}

    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(w, args.cpu_seconds)

    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "form": "plain FP64 (rk4_f64), one launch per call",
                   "rays_per_gpu": n, "steps_per_ray": rows - 1, "grid": grid_desc(w),
                   "dt": w.dt, "stop_rule": "stage1", "math": args.math,
                   "other_math": {"math": alt_math, "value": alt_rate, "unit": METRIC},
                   "l2": "512 MB buffer written between timed steps; each step also writes 10.5 GB",
                   "parallelism": f"replicas x{world}"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clock,
    }
    if north is not None:
        line["north_star"] = north
    elif not args.no_north_star:
        line["north_star"] = {"skipped": f"{world} ranks: measured on one GPU only"}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def plain_rate(b, c, rays, t0, dt, steps, chunk, dev, stream):
    """The plain FP64 form (K1, one mr_trace_device launch per chunk of
    `chunk` steps, full trajectories) over the whole step horizon of these
    rays: a ray still running at the end of a chunk continues from its last
    state in the next one (bit-identical to one launch: dt is a power of two,
    so every chunk's start time is exact), ended rays are dropped between
    chunks.  Only the launches are timed (CUDA events).  Returns
    (ray-steps, seconds, launches)."""
    import torch

    import mantaray_gb300 as mr

    n = int(rays[0].numel())
    buf = torch.empty(5 * (chunk + 1) * n, dtype=torch.float64, device=dev)
    nr = torch.empty(n, dtype=torch.int32, device=dev)
    st = torch.empty(n, dtype=torch.uint8, device=dev)
    cur = [r.contiguous() for r in rays]
    t, left, ray_steps, seconds, launches = t0, steps, 0, 0.0, 0
    while left > 0 and cur[0].numel() > 0:
        k, m = min(chunk, left), int(cur[0].numel())
        traj = buf[: 5 * (k + 1) * m].view(5, k + 1, m)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mr.trace_device(b, c, *cur, t, t + k * dt, dt, traj, nr[:m], st[:m], math="identity",
                        stream=stream)
        e1.record(stream)
        e1.synchronize()
        seconds += e0.elapsed_time(e1) / 1e3
        launches += 1
        ray_steps += int((nr[:m].to(torch.int64) - 1).sum().item())
        alive = st[:m] == 0  # MR_RAY_COMPLETE: every step of the chunk taken
        cur = [traj[q, k][alive].contiguous() for q in range(1, 5)]
        t += k * dt
        left -= k
    del buf
    return ray_steps, seconds, launches


def fp64_trajectories(b, c, rays, t0, dt, steps, dev, stream):
    """Full plain FP64 trajectories (traj[5][steps + 1][n], rows) of these
    rays, on the device."""
    import torch

    import mantaray_gb300 as mr

    n = int(rays[0].numel())
    traj = torch.empty((5, steps + 1, n), dtype=torch.float64, device=dev)
    nr = torch.empty(n, dtype=torch.int32, device=dev)
    st = torch.empty(n, dtype=torch.uint8, device=dev)
    mr.trace_device(b, c, *rays, t0, t0 + steps * dt, dt, traj, nr, st, math="identity",
                    stream=stream)
    torch.cuda.synchronize()
    return traj, nr


def chunked_endpoint_errors(end, n_steps, traj, nr, per=512):
    """batch.endpoint_errors of end states against device trajectories,
    `per` rays at a time (small host copies).  Returns per-ray relative
    position and direction errors (NaN where not compared)."""
    from mantaray_gb300.batch import endpoint_errors

    n = int(nr.numel())
    rel, dth = [], []
    for s in range(0, n, per):
        e = slice(s, min(n, s + per))
        er = endpoint_errors(end[:, e], n_steps[e], traj[:, :, e].cpu().numpy(),
                             nr[e].cpu().numpy(), per_ray=True)
        rel.append(er["rel_position"])
        dth.append(er["direction"])
    return np.concatenate(rel), np.concatenate(dth)


def error_stats(rel, dth, mask=None):
    """p50 / p99 / max of the compared rays' errors (optionally within mask)."""
    m = np.isfinite(rel) & (True if mask is None else mask)
    if not m.any():
        return {"rays": 0}
    r, d = rel[m], dth[m]
    return {"rays": int(m.sum()), "rel_position_p50": float(np.median(r)),
            "rel_position_p99": float(np.percentile(r, 99)), "rel_position_max": float(r.max()),
            "direction_p99_rad": float(np.percentile(d, 99)), "direction_max_rad": float(d.max())}


def last_finite_states(traj, nr):
    """Each ray's last finite row of device trajectories: (states [5][n], row)."""
    import torch

    n = int(nr.numel())
    last = (nr.to(torch.int64) - 1).clamp(min=0)
    idx = torch.arange(n, device=traj.device)
    fin = torch.isfinite(traj[1:, last, idx]).all(dim=0)
    last = torch.where(fin, last, (last - 1).clamp(min=0))
    return traj[:, last, idx].cpu().numpy(), last.cpu().numpy()


def batch_kernels_per_call(cfg, max_cells: int, n_scenarios: int, decimation: int,
                           max_steps: int) -> int:
    """This project's kernels in one batched call: rk4_f32, the NaN fill of
    the decimated rows, and with ordering order_keys + 3 per 8-bit pass of the
    sort key (direction 8 bits, Morton code 2 x cell bits, scenario bits); in
    sweeps, each sweep after the first adds sweep_next, 3 per 8-bit pass of
    the running rays' key (Morton code 2 x 2-cell-block bits, scenario bits)
    and rk4_f32."""
    cbits = int(np.ceil(np.log2(max_cells))) if max_cells > 1 else 0
    sbits = int(np.ceil(np.log2(n_scenarios))) if n_scenarios > 1 else 0
    passes = (8 + 2 * min(cbits, 16) + sbits + 7) // 8
    k = 1 + (1 if decimation else 0) + ((1 + 3 * passes) if cfg.order else 0)
    if cfg.sweep_steps > 0:
        blocks = (max_cells + 1) // 2
        bbits = 0
        while bbits < 15 and (1 << bbits) < blocks:
            bbits += 1
        sweep_passes = max(1, (2 * bbits + sbits + 7) // 8)
        sweeps = max(1, -(-max_steps // cfg.sweep_steps))
        k += (sweeps - 1) * (2 + 3 * sweep_passes)
    return k


def north_star_batched(args, dev, stream, flush) -> dict:
    """The large single-scenario throughput case: rays entering an 8,192^2
    shelf-slope field at 50 m (h, u, v and their cell gradients as FP32 cell
    records: 5.4 GB, far above L2) for up to 50,000 steps of 2 s, in
    graph-replayed calls of the autotuned batched FP32 form whose ray counts
    vary +-50% about 16,777,216 (seeded).  Beside it: the plain FP64 form's
    rate on a subset of the same rays over the same horizon, and the batched
    end states' error against plain FP64 trajectories of the same rays."""
    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300 import workloads as W
    from mantaray_gb300.batch import BatchTracer, make_config

    nominal = args.ns_rays
    cap = nominal * 3 // 2
    t_gen = time.perf_counter()
    fields, rays = W.shelf_slope(n=args.ns_grid, n_rays=cap, steps=args.ns_steps)
    t_gen = time.perf_counter() - t_gen
    b = mr.Bathymetry.grid(fields[0], fields[1], fields[2])
    c = mr.Current.grid(fields[3], fields[4], fields[5], fields[6])
    del fields
    tracer = BatchTracer([(b, c)])
    ins = [torch.from_numpy(rays[k]).to(dev) for k in ("x0", "y0", "kx0", "ky0")]
    steps, dt, t0 = rays["steps"], rays["dt"], rays["t0"]
    name = (f"shelf_slope_{nominal}rays_pm50pct_{args.ns_grid}x{args.ns_grid}_dt2_"
            f"{steps}steps_graph_replay")
    probe = min(cap, 1 << 20)
    if args.launch:
        blk, bps, rpl, order, *more = (int(v) for v in args.launch.split(","))
        cfg = make_config(blk, bps, rpl, 32, order, *more[:2])
    else:
        # short probe of every shape on 2^20 rays, then the fastest six
        # (and the ordered ones in sweeps) again on 2^23 rays over a long
        # trace, where the rays have spread over the whole field (half the
        # benchmark's ray density: how well sweeps share cell records
        # depends on it), then the three fastest of those on the nominal
        # call itself (16.8 M rays over the whole horizon, one call each)
        many = min(cap, 1 << 23)
        cfg = tracer.autotune(*ins, dt, min(steps, 1000), t0=t0,
                              cache_key=f"{torch.cuda.get_device_name(dev)}:{name}:{probe}:{many}",
                              long_steps=min(steps, 10000), long_rays=many, finalists=6,
                              probe_rays=probe, final_rays=nominal, final_steps=steps)
    g = tracer.graph(*ins, dt, steps, t0=t0, config=cfg)
    out = g.out
    counts = np.random.default_rng(4004).integers(nominal // 2, cap + 1,
                                                  args.ns_warmup + args.ns_calls)
    for i in range(args.ns_warmup):
        g.launch(int(counts[i]), stream=stream)
    torch.cuda.synchronize()
    times, done = [], 0
    with ClockSampler(dev.index or 0) as clocks:
        for i in range(args.ns_calls):
            cnt = int(counts[args.ns_warmup + i])
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.launch(cnt, stream=stream)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            done += int(out.n_steps[:cnt].to(torch.int64).sum().item())
    clock = clocks.summary()
    value = done / sum(times)
    timed_counts = counts[args.ns_warmup:]

    # endpoint errors against plain FP64 trajectories: rays every call traces
    n_err = min(args.ns_error_rays, nominal // 2)
    eidx = torch.from_numpy(np.linspace(0, nominal // 2 - 1, n_err).astype(np.int64)).to(dev)
    end_b = out.end_state[:, eidx].cpu().numpy()
    nst_b = out.n_steps[eidx].cpu().numpy()
    stat_b = out.status[eidx].cpu().numpy()
    erays = [t[eidx] for t in ins]
    traj, nr = fp64_trajectories(b, c, erays, t0, dt, steps, dev, stream)
    rel, dth = chunked_endpoint_errors(end_b, nst_b, traj, nr)
    # the FP64 model's own sensitivity: its endpoint change when the start
    # moves 10 cm along x (sens), and the largest change under that, a 1e-5
    # rad turn and a 1e-5 relative change of |k| -- perturbations of the size
    # FP32 rounding accumulates to over a long trace (worst: NaN where a
    # perturbed ray ends at another step)
    th, kk = torch.atan2(erays[3], erays[2]), torch.hypot(erays[2], erays[3])
    worst = None
    for start in ([erays[0] + 0.1] + erays[1:],
                  erays[:2] + [kk * torch.cos(th + 1e-5), kk * torch.sin(th + 1e-5)],
                  erays[:2] + [erays[2] * (1.0 + 1e-5), erays[3] * (1.0 + 1e-5)]):
        traj_p, nr_p = fp64_trajectories(b, c, start, t0, dt, steps, dev, stream)
        end_p, last_p = last_finite_states(traj_p, nr_p)
        del traj_p
        e, _ = chunked_endpoint_errors(end_p, last_p, traj, nr)
        if worst is None:
            sens = e
        worst = e if worst is None else np.maximum(worst, e)
    del traj
    cond = worst <= 1e-4  # rays whose FP64 endpoint is well-conditioned

    # the plain FP64 form's rate on a subset of the same rays, same horizon
    n_plain = min(args.ns_plain_rays, nominal)
    pidx = torch.from_numpy(np.linspace(0, cap - 1, n_plain).astype(np.int64)).to(dev)
    plain_steps, plain_s, plain_launches = plain_rate(
        b, c, [t[pidx] for t in ins], t0, dt, steps, args.ns_plain_chunk, dev, stream)
    plain = plain_steps / plain_s

    L = mr._native.load()
    import ctypes

    fp32_peak = ctypes.c_double()
    mr._native.check(L.mr_measure_fma_peak(0, ctypes.byref(fp32_peak)))
    ach = value * ALG_FP32_FLOP_PER_RAY_STEP / 1e12
    roof = {"bound": "fp32", "achieved": ach, "peak": fp32_peak.value, "unit": "TFLOP/s",
            "frac": ach / fp32_peak.value,
            "peak_source": "measured: FP32 FMA-chain kernel on this GPU, this run",
            "flop_per_ray_step": ALG_FP32_FLOP_PER_RAY_STEP,
            "executed_flop_per_ray_step": FP32_FLOP_PER_RAY_STEP,
            "executed_frac": value * FP32_FLOP_PER_RAY_STEP / 1e12 / fp32_peak.value}
    per_step, note = k2_shelf_dram(cfg.sweep_steps)
    roof["traffic"] = per_step * done / args.ns_calls
    roof["traffic_note"] = note
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        src = "MEASURED_PEAKS.json hbm_gbs"
    except (OSError, ValueError, KeyError):
        hbm_peak, src = 6800.0, "fallback"
    gbs = per_step * value / 1e9
    roof["hbm"] = {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                   "peak_source": src,
                   "note": ("in sweeps the cell records mostly come from L2 (80% hits in the "
                            "capture): issue-bound, like the fields that fit in L2"
                            if cfg.sweep_steps else
                            "the DRAM reads of cell records on cell changes (40% L2 hits in "
                            "the capture): bound by their latency, neither this bandwidth "
                            "nor the FP32 pipe is saturated")}
    roof["traffic_floor"] = float(np.mean(timed_counts)) * (4 * 8 + 5 * 8 + 4 + 4 + 1)
    status = np.bincount(stat_b, minlength=4)
    return {
        "workload": name, "metric": METRIC, "value": value, "unit": METRIC, "dtype": "f32",
        "calls": args.ns_calls, "warmup_calls": args.ns_warmup,
        "ms_per_call": 1e3 * sum(times) / args.ns_calls,
        "rays_per_call": {"min": int(timed_counts.min()), "max": int(timed_counts.max()),
                          "mean": float(timed_counts.mean()), "capacity": cap},
        "ray_steps_per_call": done / args.ns_calls, "max_steps": steps, "dt": dt,
        "graph_replay": True, "launch": cfg.as_dict(), "autotuned": not args.launch,
        "field": f"{args.ns_grid}^2 f32 cell records (h, u, v, gradients), generated in "
                 f"{t_gen:.0f} s on the host",
        "l2": "512 MB buffer written between timed calls; cell records 5.4 GB > L2",
        "plain_fp64_same_rays": {"value": plain, "unit": METRIC, "rays": n_plain,
                                 "ray_steps": plain_steps, "launches": plain_launches,
                                 "chunk_steps": args.ns_plain_chunk, "math": "identity",
                                 "how": "mr_trace_device per chunk of steps over the whole "
                                        "horizon, running rays continued, launches timed"},
        "batched_over_plain": value / plain, "target_batched_over_plain": ">= 5",
        "endpoint_error_vs_fp64": {
            "of": n_err,
            "status_counts": {"complete": int(status[0]), "out_of_domain": int(status[1]),
                              "dry": int(status[2]), "bad_wavenumber": int(status[3])},
            "all_compared_rays": error_stats(rel, dth),
            "fp64_conditioned_rays": dict(
                error_stats(rel, dth, cond), share_of_rays=float(np.mean(cond)),
                which="rays whose FP64 endpoint moves by <= 1e-4 of its path under each of "
                      "three start perturbations: 10 cm along x, 1e-5 rad, 1e-5 of |k|"),
            "target_rel_position": "<= 1e-3"},
        "fp64_endpoint_change_for_10cm_start_shift": {
            "rel_position_p50": float(np.nanmedian(sens)),
            "rel_position_p99": float(np.nanpercentile(sens, 99)),
            "rel_position_max": float(np.nanmax(sens))},
        "roofline": roof, "clocks": clock,
        "gpu_launches": args.ns_calls * batch_kernels_per_call(cfg, args.ns_grid - 1, 1, 0, steps),
    }


def adjoint_times(precision, n_rays, steps, warmup, calls, dev, stream):
    """Forward (with checkpoints) and forward + gradient times of the
    differentiation case (262,144 rays x 3,000 steps on the 512^2 shelf-bump
    field, checkpoints every 55 steps, endpoint (y, theta) misfit loss against
    targets traced with the shoal raised 10%)."""
    import torch

    from mantaray_gb300.diff import endpoint_loss, grid, ray_endpoints
    from mantaray_gb300.workloads import shelf_bump

    w = shelf_bump(n_rays=n_rays, steps=steps)
    tg = shelf_bump(n_rays=n_rays, steps=steps, bump_scale=1.1)
    dtype = torch.float64 if precision == 64 else torch.float32
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev).to(dtype)  # noqa: E731
    g = grid(512, 512, 0.0, 0.0, 200.0, 200.0)
    rays = [t(a) for a in (w.x0, w.y0, w.kx0, w.ky0)]
    D, U, V = t(w.depth), t(w.u), t(w.v)
    every = 55
    tgt, tst = ray_endpoints(*rays, t(tg.depth), U, V, g, g, 1.0, steps, every)
    y_t, th_t = tgt[1], torch.atan2(tgt[3], tgt[2])

    def forward_only():
        with torch.no_grad():
            return ray_endpoints(*rays, D, U, V, g, g, 1.0, steps, every)

    def gradient():
        depth = D.clone().requires_grad_(True)
        u = U.clone().requires_grad_(True)
        v = V.clone().requires_grad_(True)
        r = [x.clone().requires_grad_(True) for x in rays]
        end, status = ray_endpoints(*r, depth, u, v, g, g, 1.0, steps, every)
        keep = (status == 0) & (tst == 0)
        loss = endpoint_loss(end, torch.where(keep, status, torch.ones_like(status)), y_t, th_t)
        loss.backward()
        return loss

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(calls):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return sum(ts) / len(ts)

    t_fwd = timed(forward_only)
    t_grad = timed(gradient)
    return w, t_fwd, t_grad


def north_star_adjoint(args, dev, stream) -> dict:
    """Gradient / forward time of the differentiation case, FP64 and FP32."""
    res = {"workload": "shelf_bump_262144rays_512x512_dt1_3000steps_checkpoints55",
           "calls": args.ns_adjoint_calls, "target_gradient_over_forward": "<= 5"}
    with ClockSampler(dev.index or 0) as clocks:
        for prec in (64, 32):
            _, t_fwd, t_grad = adjoint_times(prec, 262144, 3000, 1, args.ns_adjoint_calls, dev,
                                             stream)
            res[f"fp{prec}"] = {"forward_ms": 1e3 * t_fwd, "gradient_ms": 1e3 * t_grad,
                                "gradient_over_forward": t_grad / t_fwd}
    res["clocks"] = clocks.summary()
    return res


def batched_arm(args, rank: int, world: int, local_rank: int):
    """The batched FP32 form (rk4_f32) on one of the benchmark workloads, with
    the plain FP64 form timed beside it on a subset of the same rays and the
    endpoint error of the FP32 results against it."""
    import ctypes

    import torch

    import mantaray_gb300 as mr
    from mantaray_gb300 import workloads as W
    from mantaray_gb300.batch import BatchTracer, default_config, endpoint_errors, make_config

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811

        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if dist is not None:
            dist.barrier()

    graph_mode = False
    decimation = 0
    if args.workload in PLAIN_WORKLOADS:
        w = plain_workload(args)
        fields = [(w.bx, w.by, w.depth, w.cx, w.cy, w.u, w.v)]
        rays = {"x0": w.x0, "y0": w.y0, "kx0": w.kx0, "ky0": w.ky0, "scenario": None,
                "t0": w.t0, "dt": w.dt, "steps": mr.num_steps(w.t0, w.t_end, w.dt)}
        name = w.name
    elif args.workload == "multi_source":
        n = args.grid or 2048
        fields, rays = W.multi_source(n=n, steps=args.trace_steps if args.trace_steps != 4000
                                      else 20000)
        decimation = 100
        name = f"multi_source_{rays['x0'].size}rays_8x{n}x{n}_dt2_{rays['steps']}steps_every100"
    else:
        n = args.grid or 8192
        steps = args.trace_steps if args.trace_steps != 4000 else 2000
        fields, rays = W.shelf_slope(n=n, n_rays=args.rays if args.rays != 65536 else 16777216,
                                     steps=steps)
        fields = [fields]
        graph_mode = True
        name = (f"shelf_slope_{rays['x0'].size}rays_{n}x{n}_dt2_{steps}steps_graph_replay_"
                f"n_varied_50pct")
    handles = [(mr.Bathymetry.grid(f[0], f[1], f[2]), mr.Current.grid(f[3], f[4], f[5], f[6]))
               for f in fields]
    tracer = BatchTracer(handles)
    n_all = rays["x0"].size
    ins = [torch.from_numpy(np.ascontiguousarray(rays[k])).to(dev) for k in ("x0", "y0", "kx0", "ky0")]
    sid = (torch.from_numpy(rays["scenario"]).to(dev) if rays["scenario"] is not None else None)
    steps, dt, t0 = rays["steps"], rays["dt"], rays["t0"]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    cfg = default_config()
    tuned = None
    if args.launch:
        blk, bps, rpl, order, *more = (int(v) for v in args.launch.split(","))
        cfg = make_config(blk, bps, rpl, 32, order, *more[:2])
    elif not args.no_autotune:
        probe = min(n_all, 1 << 20)
        # long horizons: the fastest shapes (and the ordered ones in sweeps)
        # again on 2^22 rays over 10,000 steps, where the rays have spread,
        # then the three fastest of those on the call itself
        long_h = steps >= 5000
        many = min(n_all, 1 << 22) if long_h else probe
        cfg = tracer.autotune(*ins, dt, min(steps, 1000), t0=t0, scenario=sid,
                              cache_key=f"{torch.cuda.get_device_name(dev)}:{name}:{probe}:{many}",
                              long_steps=min(steps, 10000) if long_h else None,
                              long_rays=many, finalists=6, probe_rays=probe,
                              final_rays=n_all if long_h else None,
                              final_steps=steps if long_h else None)
        tuned = cfg.as_dict()

    rng = np.random.default_rng(7)
    if graph_mode:
        # capacity 1.5x the nominal count; each call traces U[0.5, 1.5] x nominal rays
        nominal = n_all * 2 // 3
        g = tracer.graph(*ins, dt, steps, t0=t0, decimation=decimation, scenario=sid, config=cfg)
        counts = rng.integers(nominal // 2, n_all + 1, args.warmup + args.steps)
        out = g.out

        def one(i):
            g.launch(int(counts[i]), stream=stream)
            return int(counts[i])
    else:
        out = tracer.alloc(n_all, steps, decimation, device=dev)

        def one(i):
            tracer.trace(*ins, dt, steps, t0=t0, decimation=decimation, scenario=sid, config=cfg,
                         out=out, stream=stream)
            return n_all

    cmax = max(max(fs[2].shape) - 1 for fs in fields)
    kernels_per_call = batch_kernels_per_call(cfg, cmax, len(handles), decimation, steps)
    for i in range(args.warmup):
        one(i)
    torch.cuda.synchronize()
    times, done_steps, launches = [], 0, 0
    with ClockSampler(local_rank) as clocks:
        barrier()
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            nrays = one(args.warmup + i)
            e1.record(stream)
            launches += kernels_per_call
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            done_steps += int(out.n_steps[:nrays].to(torch.int64).sum().item())
        torch.cuda.synchronize()
        barrier()
    clock = clocks.summary()
    local_t = sum(times)
    t_max = reduce_scalar(local_t, "max") if dist is not None else local_t
    value = done_steps * world / t_max
    kernel_rate = done_steps / local_t

    # ---- end to end: host initial states in, host end states (+ rows) out ----
    e2e = None
    if not args.no_e2e:
        hin = [torch.from_numpy(np.ascontiguousarray(rays[k])).pin_memory()
               for k in ("x0", "y0", "kx0", "ky0")]
        hend = torch.empty_like(out.end_state, device="cpu").pin_memory()
        hsaved = torch.empty_like(out.saved, device="cpu").pin_memory()
        hsteps = torch.empty_like(out.n_steps, device="cpu").pin_memory()
        hstat = torch.empty_like(out.status, device="cpu").pin_memory()
        from mantaray_gb300.batch import BatchResult

        out_h = BatchResult(hsaved if decimation else out.saved, out.end_state, out.n_steps,
                            out.n_saved, out.status)
        e2e_t, e2e_steps, h2d, d2h = [], 0, 0, 0
        for i in range(args.steps + 1):
            # graph replay: that call's ray count, the first c rays of the buffers
            c = int(counts[args.warmup + i - 1]) if graph_mode and i else n_all
            torch.cuda.synchronize()
            t_a = time.perf_counter()
            for d, h in zip(ins, hin):
                d[:c].copy_(h[:c], non_blocking=True)
            if graph_mode:
                g.launch(c, stream=stream)
            else:
                # the decimated rows go straight to the page-locked host buffer
                tracer.trace(*ins, dt, steps, t0=t0, decimation=decimation, scenario=sid,
                             config=cfg, out=out_h, stream=stream)
            hend[:, :c].copy_(out.end_state[:, :c], non_blocking=True)
            hsteps[:c].copy_(out.n_steps[:c], non_blocking=True)
            hstat[:c].copy_(out.status[:c], non_blocking=True)
            torch.cuda.synchronize()
            if i:
                e2e_t.append(time.perf_counter() - t_a)
                e2e_steps += int(hsteps[:c].to(torch.int64).sum().item())
                h2d += 4 * c * 8
                d2h += int(5 * c * 8 + c * 5 + (out.saved.numel() * 4 if decimation else 0))
        e2e = {"value": e2e_steps * world / sum(e2e_t), "unit": METRIC,
               "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
               "path": ("torch copies of page-locked host buffers around "
                        + ("mr_batch_graph_launch" if graph_mode else
                           "mr_batch_trace_device (decimated rows written by the kernel into "
                           "page-locked host memory)")),
               "ms_per_step": 1e3 * sum(e2e_t) / args.steps}

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- the plain FP64 form on a subset of the same rays, and the error ----
    # plain FP64 rate on a GPU-filling subset (one stream per scenario, all
    # launched together); errors on up to 4,096 of its rays
    sub = int(min(n_all, 65536))
    idx = np.sort(rng.choice(n_all, sub, replace=False))
    scen_of = rays["scenario"][idx] if rays["scenario"] is not None else np.zeros(sub, np.uint8)
    errs_all = {"rel_position": [], "direction": [], "compared": 0, "n": 0}
    sens = []
    ref_out = tracer.trace(*[t[torch.from_numpy(idx).to(dev)] for t in ins], dt, steps, t0=t0,
                           scenario=(torch.from_numpy(scen_of).to(dev)
                                     if rays["scenario"] is not None else None), config=cfg)
    torch.cuda.synchronize()
    end_sub = ref_out.end_state.cpu().numpy()
    nst_sub = ref_out.n_steps.cpu().numpy()
    del ref_out
    launches_plain = []
    for s_i, (b, c) in enumerate(handles):
        m = np.nonzero(scen_of == s_i)[0]
        if m.size == 0:
            continue
        sel = idx[m]
        pin = [torch.from_numpy(np.ascontiguousarray(rays[k][sel])).to(dev)
               for k in ("x0", "y0", "kx0", "ky0")]
        traj = torch.empty((5, steps + 1, sel.size), dtype=torch.float64, device=dev)
        nr = torch.empty(sel.size, dtype=torch.int32, device=dev)
        st = torch.empty(sel.size, dtype=torch.uint8, device=dev)
        launches_plain.append((s_i, m, b, c, pin, traj, nr, st, torch.cuda.Stream(dev)))
    torch.cuda.synchronize()
    e_start = torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    ends = []
    for s_i, m, b, c, pin, traj, nr, st, strm in launches_plain:
        strm.wait_event(e_start)
        mr.trace_device(b, c, *pin, t0, t0 + steps * dt, dt, traj, nr, st, math="identity",
                        stream=strm)
        e = torch.cuda.Event(enable_timing=True)
        e.record(strm)
        ends.append(e)
    torch.cuda.synchronize()
    plain_time = max(e_start.elapsed_time(e) for e in ends) / 1e3
    plain_steps = 0
    for s_i, m, b, c, pin, traj, nr, st, strm in launches_plain:
        plain_steps += int((nr.to(torch.int64) - 1).sum().item())
        k = min(m.size, max(1, 4096 // len(handles)))
        er = endpoint_errors(end_sub[:, m[:k]], nst_sub[m[:k]], traj[:, :, :k].cpu().numpy(),
                             nr[:k].cpu().numpy())
        errs_all["rel_position"].append(er["rel_position"])
        errs_all["direction"].append(er["direction"])
        errs_all["compared"] += er["compared"]
        errs_all["n"] += er["n"]
        # the FP64 model's own sensitivity: the same rays started 1 cm further in x
        pin_p = [pin[0][:k] + 0.01, pin[1][:k], pin[2][:k], pin[3][:k]]
        traj_p = torch.empty((5, steps + 1, k), dtype=torch.float64, device=dev)
        nr_p = torch.empty(k, dtype=torch.int32, device=dev)
        st_p = torch.empty(k, dtype=torch.uint8, device=dev)
        mr.trace_device(b, c, *pin_p, t0, t0 + steps * dt, dt, traj_p, nr_p, st_p,
                        math="identity", stream=stream)
        tp, np_ = traj_p.cpu().numpy(), nr_p.cpu().numpy().astype(np.int64)
        ik = np.arange(k)
        last = np_ - 1
        last = np.where(np.all(np.isfinite(tp[1:, last, ik]), axis=0), last, np.maximum(last - 1, 0))
        es = endpoint_errors(tp[:, last, ik], last, traj[:, :, :k].cpu().numpy(),
                             nr[:k].cpu().numpy())
        sens.append(es["rel_position"])
        del traj_p
    del launches_plain
    rel = np.concatenate(errs_all["rel_position"])
    dth = np.concatenate(errs_all["direction"])
    sens_all = np.concatenate(sens)
    plain_rate = plain_steps / plain_time

    L = mr._native.load()
    fp32_peak = ctypes.c_double()
    mr._native.check(L.mr_measure_fma_peak(0, ctypes.byref(fp32_peak)))
    ach = kernel_rate * ALG_FP32_FLOP_PER_RAY_STEP / 1e12
    roofline = {"bound": "fp32", "achieved": ach, "peak": fp32_peak.value, "unit": "TFLOP/s",
                "frac": ach / fp32_peak.value,
                "peak_source": "measured: FP32 FMA-chain kernel on this GPU, this run",
                "traffic": None, "flop_per_ray_step": ALG_FP32_FLOP_PER_RAY_STEP,
                "flop_note": "algorithmic: the reference's 270 FP64 add/mul/div and 440 f32 "
                             "interpolation operations per ray-step, all in FP32; executed: ncu "
                             "count with the current on the bathymetry's grid",
                "executed_flop_per_ray_step": FP32_FLOP_PER_RAY_STEP,
                "executed_frac": kernel_rate * FP32_FLOP_PER_RAY_STEP / 1e12 / fp32_peak.value}
    # DRAM bytes per ray-step of ncu captures, scaled to one call's ray-steps
    k2_dram_per_ray_step = {"seamount": (18.60e6 / (65536 * 400),
                                         "65,536-ray x 400-step seamount capture"),
                            "shelf_slope": ((452.10e6 + 36.66e6) / 330.35e6,
                                            "4,096^2-grid, 2^20-ray x 400-step shelf-slope "
                                            "capture")}
    if args.workload in k2_dram_per_ray_step:
        per, src = k2_dram_per_ray_step[args.workload]
        roofline["traffic"] = per * done_steps / args.steps
        roofline["traffic_note"] = f"DRAM bytes per call, scaled by ray-steps from the {src}"
    cpu = None
    if not args.no_cpu_baseline:
        if args.workload in PLAIN_WORKLOADS:
            cpu = cpu_baseline(w, args.cpu_seconds)
        else:
            # the first scenario's fields with a seeded sample of its rays
            f = fields[0]
            pick = np.nonzero(rays["scenario"] == 0)[0] if rays["scenario"] is not None \
                else np.arange(n_all)
            pick = np.sort(np.random.default_rng(11).choice(pick, min(pick.size, 65536),
                                                           replace=False))
            wc = W.Workload(name + "_scenario0_sample", *f, *(rays[k][pick] for k in
                                                              ("x0", "y0", "kx0", "ky0")),
                            t0, t0 + steps * dt, dt)
            cpu = cpu_baseline(wc, args.cpu_seconds)
            cpu["sample"] += "; scenario 0's fields, a seeded 65,536-ray sample of its rays"
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": name, "form": "batched FP32 (rk4_f32), persistent, work queue",
                   "rays_per_gpu": n_all, "max_steps": steps, "dt": dt, "decimation": decimation,
                   "scenarios": len(handles), "launch": (tuned or cfg.as_dict()),
                   "autotuned": tuned is not None, "graph_replay": graph_mode,
                   "plain_fp64_same_rays": {"value": plain_rate, "unit": METRIC,
                                            "rays": sub, "math": "identity"},
                   "batched_over_plain": value / world / plain_rate,
                   "endpoint_error_vs_fp64": {
                       "rays": int(errs_all["compared"]), "of": int(errs_all["n"]),
                       "rel_position_p50": float(np.median(rel)),
                       "rel_position_p99": float(np.percentile(rel, 99)),
                       "rel_position_max": float(rel.max()),
                       "direction_p99_rad": float(np.percentile(dth, 99)),
                       "direction_max_rad": float(dth.max())},
                   "fp64_endpoint_change_for_1cm_start_shift": {
                       "rel_position_p50": float(np.median(sens_all)),
                       "rel_position_p99": float(np.percentile(sens_all, 99)),
                       "rel_position_max": float(sens_all.max())},
                   "l2": "512 MB buffer written between timed steps",
                   "parallelism": f"replicas x{world}"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
        "clocks": clock,
    }
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def adjoint_arm(args, rank: int, world: int, local_rank: int):
    """The differentiation case: gradient of the endpoint loss with respect to
    the initial states and every depth / current node for 262,144 rays x
    3,000 steps (checkpoints every 55 steps), against the forward pass."""
    import torch

    import mantaray_gb300 as mr

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    n_rays = args.rays if args.rays != 65536 else 262144
    steps = args.trace_steps if args.trace_steps != 4000 else 3000
    stream = torch.cuda.current_stream(dev)
    with ClockSampler(local_rank) as clocks:
        w, t_fwd, t_grad = adjoint_times(args.precision, n_rays, steps, args.warmup, args.steps,
                                         dev, stream)
    clock = clocks.summary()
    # the plain FP64 drop-in kernel over the same rays and fields (f32-cast
    # lookups, as the reference), for scale
    b = mr.Bathymetry.grid(w.bx, w.by, w.depth)
    c = mr.Current.grid(w.cx, w.cy, w.u, w.v)
    sub = min(n_rays, 65536)
    pin = [torch.from_numpy(a[:sub]).to(dev) for a in (w.x0, w.y0, w.kx0, w.ky0)]
    traj = torch.empty((5, steps + 1, sub), dtype=torch.float64, device=dev)
    nr = torch.empty(sub, dtype=torch.int32, device=dev)
    st = torch.empty(sub, dtype=torch.uint8, device=dev)
    times = []
    for i in range(args.warmup + args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mr.trace_device(b, c, *pin, 0.0, float(steps), 1.0, traj, nr, st, math="identity",
                        stream=stream)
        e1.record(stream)
        e1.synchronize()
        if i >= args.warmup:
            times.append(e0.elapsed_time(e1) / 1e3)
    t_plain = statistics.mean(times) * n_rays / sub
    ray_steps = n_rays * steps
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": ray_steps / t_grad, "unit": METRIC, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_grad,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == 64 else "f32", "data": "synthetic",
        "config": {"workload": w.name, "form": "differentiation: forward with checkpoints + "
                                               "discrete adjoint (mr_diff_*)",
                   "rays": n_rays, "steps_per_ray": steps, "checkpoint_every": 55,
                   "gradient_ms": 1e3 * t_grad, "forward_ms": 1e3 * t_fwd,
                   "plain_fp64_forward_ms": 1e3 * t_plain,
                   "gradient_over_forward": t_grad / t_fwd,
                   "gradient_over_plain_forward": t_grad / t_plain,
                   "value_is": "ray-steps of the traced rays per second of a full gradient"},
        "roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": 2 * args.steps,
        "clocks": clock,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus if "RANK" in os.environ else 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        reference_arm(args, rank, world)
    elif args.ns_only:
        import torch

        torch.cuda.set_device(local_rank)
        dev = torch.device("cuda", local_rank)
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
        print(json.dumps(north_star_batched(args, dev, torch.cuda.current_stream(dev), flush)),
              flush=True)
    elif args.form == "batched":
        batched_arm(args, rank, world, local_rank)
    elif args.form == "adjoint":
        adjoint_arm(args, rank, world, local_rank)
    else:
        gb300_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
