"""Throughput of the WENO-FD hot path on GB300: cell-updates/s at 4096^2.

Workload: periodic shear layer on [0,1]^2 (rho = 2 for |y-0.5| < 0.25 else 1,
u = +-0.5, v = 0.01 sin(4 pi x) + seeded N(0, 1e-3), p = 2.5, gamma 1.4),
4096 x 4096 nodes, SSP-RK3, WENO-Z, CFL 0.7.  One step = one full RK3 time
step (time-step reduction + 3 stages with their boundary fills) over the
whole grid; cell-updates = nodes x steps.  The state (537 MB per array) is
larger than L2, so no flush is needed between steps.

The headline form is the fastest form that is built (FP32 flux arithmetic
with FP64 state / RK sums / dt); the plain FP64 WENO-Z path, bitwise equal to
the reference, is measured in the same run on the same GPU, and the density
L1 difference between the two after the same steps is reported.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(replicas only: the path is one whole-domain solve per GPU); value is the
sum over ranks, timed as the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fd-weno-eulerequation_gb300", "python"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

N = 4096
SEED = 2024
METRIC = "cell-updates/s at 4096^2 (learned+FP32 vs plain FP64 WENO-Z, same GB300) at stated L1 err"
# algorithmic HBM bytes per node for one SSP-RK3 step with FP64 state:
# stage 1 reads U^n, writes U1 (64 B); stages 2, 3 read U^n and U^k, write (96 B each)
BYTES_PER_CELL_RK3 = 256


def config_for(precision: int, device: int) -> dict:
    return {"TESTCASE": 5, "ELEMNUMX": N, "ELEMNUMY": N, "RKMETH": 2, "CFL": 0.7, "SCHEME": 1,
            "SEED": SEED, "PRECISION": precision, "DEVICE": device, "TEND": 1.0e9}


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict | None:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peaks() -> dict:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def committed_traffic() -> dict:
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def cpu_baseline(budget_s: float = 12.0) -> dict:
    """The oracle port (C, OpenMP over all host cores) on the same workload:
    whole 4096^2 RK3 steps until about budget_s of wall time."""
    import oracle as orc

    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    p = orc.Problem(orc.SHEAR, N, N, orc.WENOZ, 2, 0.7, seed=SEED, t_end=1e9)
    dt = p.calc_dt()
    steps, t0 = 0, time.perf_counter()
    while True:
        p.rk_step(dt)
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or steps >= 20:
            break
    return {"value": steps * N * N / el, "unit": "cell-updates/s", "cores": threads, "kind": "port",
            "sample": f"{steps} RK3 step(s) of the 4096^2 shear layer, oracle C restatement, "
                      f"{threads} OpenMP threads, {el:.1f} s"}


def run_reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cb = cpu_baseline(budget_s=max(5.0, 120.0 / max(1, args.steps + args.warmup)))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"shear layer {N}x{N}, RK3, WENO-Z, CFL 0.7, seed {SEED}",
                       "reference": "oracle/ C restatement of the reference's per-step path (the "
                                    "reference sources are not on this host); OpenMP over host cores"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def time_form(wenofd, torch, precision: int, device: int, steps: int, warmup: int, stream):
    s = wenofd.Solver(config_for(precision, device))
    s.set_stream(stream.cuda_stream)
    s.initialize()
    s.advance(max_steps=warmup)
    l0 = s.info().launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(device)
    ev0.record(stream)
    n = s.advance(max_steps=steps)
    ev1.record(stream)
    torch.cuda.synchronize(device)
    assert n == steps
    ms = ev0.elapsed_time(ev1)
    launches = s.info().launches - l0
    return s, ms, launches


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=None, help="timed steps of the plain FP64 leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-headline", action="store_true",
                    help="time the headline form only (no FP64 leg, error, e2e or CPU leg): for profiling")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import numpy as np
    import torch

    import wenofd

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream(device=local)
    cells = N * N

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if dist is None:
            return x
        t = torch.tensor([x], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # ---- headline form (FP32 flux arithmetic), device-timed
    barrier()
    with ClockSampler(local) as clk:
        s32, ms32, launches = time_form(wenofd, torch, wenofd.FP32, local, args.steps, args.warmup, stream)
    ms32 = max_over_ranks(ms32)
    value = world * args.steps * cells / (ms32 / 1e3)
    if args.only_headline:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "cell-updates/s", "steps": args.steps,
                              "ms_per_step": ms32 / args.steps, "gpu_launches": launches,
                              "note": "headline form only (profiling run)"}))
        s32.close()
        return

    # ---- plain FP64 WENO-Z (bitwise the reference) on the same GPU
    k64 = args.fp64_steps if args.fp64_steps is not None else max(2, min(args.steps, 5))
    barrier()
    s64, ms64, _ = time_form(wenofd, torch, wenofd.FP64, local, k64, args.warmup, stream)
    ms64 = max_over_ranks(ms64)
    value64 = world * k64 * cells / (ms64 / 1e3)

    # density difference after the same number of steps from the same state
    rho32 = s32.get_state()[0]
    s64b = wenofd.Solver(config_for(wenofd.FP64, local))
    s64b.set_stream(stream.cuda_stream)
    s64b.initialize()
    s64b.advance(max_steps=args.warmup + args.steps)
    rho64 = s64b.get_state()[0]
    l1 = float(np.mean(np.abs(rho32 - rho64)))
    linf = float(np.max(np.abs(rho32 - rho64)))
    s64b.close()
    s64.close()

    # ---- stage kernel alone (roofline): mean launch duration, CUDA events on its stream
    ms_stage = s32.time_stages(reps=3)
    bytes_per_launch = BYTES_PER_CELL_RK3 / 3.0 * cells
    achieved = bytes_per_launch / (ms_stage / 1e3) / 1e9
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic = committed_traffic().get("stage_fp32_wenoz_4096", {}).get("dram_bytes_per_launch")

    # ---- end to end through the C ABI with pinned host buffers
    host = torch.empty((4, N, N), dtype=torch.float64, pin_memory=True)
    s32.initialize()
    s32.get_state_ptr(host.data_ptr())
    s32.advance(max_steps=1)
    k_e2e = max(3, min(args.steps, 10))
    barrier()
    torch.cuda.synchronize(local)
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        s32.set_state_ptr(host.data_ptr())
        s32.advance(max_steps=1)
        s32.get_state_ptr(host.data_ptr())
    torch.cuda.synchronize(local)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = world * k_e2e * cells / e2e_s
    s32.close()

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline()

    if rank == 0:
        clocks = clk.summary()
        line = {
            "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"shear layer {N}x{N}, SSP-RK3, WENO-Z, CFL 0.7, seed {SEED}",
                       "form": "FP32 flux/reconstruction, FP64 state, RK sums and dt",
                       "l2": "inputs larger than L2 (537 MB per state array)",
                       "parallelism": f"replicas x{world}"},
            "plain_fp64": {"value": value64, "unit": "cell-updates/s", "steps": k64,
                           "ms_per_step": ms64 / k64, "dtype": "f64", "parity": "bitwise vs reference"},
            "speedup_vs_plain_fp64": value / value64,
            "l1_rho_vs_fp64": l1, "linf_rho_vs_fp64": linf,
            "err_note": f"FP32 form vs plain FP64 GPU path (= FP64 oracle bitwise) after "
                        f"{args.warmup + args.steps} steps from the same state",
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_stage<float, WENO-Z> (one RK stage)",
                         "ms_per_launch": ms_stage,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks
                         else "fallback 6800 GB/s"},
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "steps": k_e2e,
                    "h2d_bytes_per_step": 4 * cells * 8, "d2h_bytes_per_step": 4 * cells * 8,
                    "path": "C ABI wenofd_set_state + wenofd_advance(1) + wenofd_get_state, pinned host"},
            "clocks": clocks,
        }
        if cb is not None:
            line["cpu_baseline"] = cb
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
