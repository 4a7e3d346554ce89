#!/usr/bin/env python
"""Benchmark of the split-operator propagation step on GB300.

Workload (default): the 2-D radial x angular problem -- 4096 radial points on
r in [0.5, 60] x 128 Gauss-Legendre angular points (Legendre transform to
l_max = 127), Morse + beta e^{-r/2} P2(cos th), mass 1000, dt = 0.5, border
damping with a loss checker, stack [Damp, V/2, Legendre, Rot/2, FFT, K].
One bench step = one split-operator time step of that problem, timed with CUDA
events on the library's stream; the L2 is flushed (256 MiB write) before every
timed step, so each step reads its state and tables from HBM.

Prints ONE JSON line (rank 0).  ``--impl reference`` times the reference's CPU
algorithm instead (the C++ FP64 restatement in oracle/, all host threads).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt·steps/s at rel-L2≤1e-6 vs FP64 plain; time-to-ground-state"
UNIT = "grid-pt·steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32_simt", choices=["fp64", "fp32_tf32x3", "fp32_bf16x3", "fp32_simt"])
    ap.add_argument("--nr", type=int, default=4096)
    ap.add_argument("--nth", type=int, default=128)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="timed region only (no e2e, accuracy or CPU legs): the case profiled under ncu")
    return ap.parse_args()


def workload_name(a):
    return (f"radial_angular_2d Nr={a.nr} x Ntheta={a.nth} (GL), Morse D=0.1 a=1 re=3 + 0.02 e^(-r/2) P2, "
            f"mass 1000, dt=0.5, damping+loss, stack [Damp,V/2,L,Rot/2,F,K]")


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        mx = max(float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs"), d.get("bf16_tflops"), "measured"
    return 6800.0, 1900.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of each pass kind from the committed ncu summary (or {})."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_per_launch.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            if line.strip() and not line.startswith("#"):
                k, v = line.rstrip("\n").split("\t")[:2]
                out[k] = float(v)
    return out


def cpu_baseline(a, seconds):
    """The C++ FP64 restatement of the reference algorithm on all host threads, bounded sample."""
    from oracle import cpu_port as P
    port = P.RadialAngular(a.nr, a.nth)
    threads = os.cpu_count() or 1
    port.run(1, threads=threads)  # warm-up (also builds the library)
    t0 = time.perf_counter()
    port.run(1, threads=threads)
    one = time.perf_counter() - t0
    n = max(1, min(200, int(seconds / max(one, 1e-6))))
    t0 = time.perf_counter()
    port.run(n, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": a.nr * a.nth * n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} steps of the {a.nr}x{a.nth} problem, FP64, C++ restatement of the reference passes"}


def dist_setup(n):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("SO_BENCH_GLOO") is None else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(a):
    world, rank, _ = dist_setup(a.gpus)
    if rank != 0:
        return
    from oracle import cpu_port as P
    port = P.RadialAngular(a.nr, a.nth)
    threads = os.cpu_count() or 1
    port.run(a.warmup, threads=threads)
    t0 = time.perf_counter()
    port.run(a.steps, threads=threads)
    dt = time.perf_counter() - t0
    v = a.nr * a.nth * a.steps / dt
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": dt / a.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_name(a), "precision": "fp64 (reference algorithm, CPU)"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{a.steps} timed steps of the {a.nr}x{a.nth} problem (C++ FP64 restatement "
                                       "of the reference's passes; the Rust crate cannot be built here)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def rel_l2(x, y):
    import numpy as np
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


def run_ours(a):
    import numpy as np
    import torch

    world, rank, local = dist_setup(a.gpus)
    torch.cuda.set_device(local)
    import split_operator_gb300 as so
    from split_operator_gb300 import workloads as W

    stream = torch.cuda.Stream()
    prop, h = W.radial_angular_2d(nr=a.nr, nth=a.nth, step_no=10 ** 6, precision=a.precision)
    prop.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    points = a.nr * a.nth

    def step_timed(ev0, ev1):
        with torch.cuda.stream(stream):
            flush.zero_()
        ev0.record(stream)
        prop.steps(1)
        ev1.record(stream)

    for _ in range(a.warmup):
        step_timed(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    prop.synchronize()

    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    prop.set_timing(True)
    n0 = so.launch_count()
    barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for e0, e1 in evs:
        step_timed(e0, e1)
    prop.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier(world)
    launches = so.launch_count() - n0
    kt = prop.kernel_times()
    prop.set_timing(False)
    clocks.stop()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    ms_max = allmax(world, ms)
    value = points * a.steps * world / (ms_max / 1e3)

    # roofline of the dominant pass kind (live CUDA events on the library's stream)
    hbm, _, peak_kind = measured_peaks()
    dom = max(kt, key=lambda t: t[2]) if kt else None
    roof = None
    if dom:
        name, n, tms, b = dom
        ach = (b / n) / (tms / n / 1e3) / 1e9
        traffic = ncu_traffic().get(name)
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": traffic, "kernel": name, "launches": n, "avg_us": tms / n * 1e3,
                "algorithmic_bytes_per_launch": b / n, "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
                "share_of_step": tms / ms if ms > 0 else None}

    if a.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms_max / a.steps,
                              "quick": True, "passes": [list(t) for t in kt]}), flush=True)
        return
    # end to end through the C ABI: pinned host input -> device, one step, device -> pinned host
    host_in = torch.empty(points * 2, dtype=torch.float64).pin_memory()
    host_out = torch.empty(points * 2, dtype=torch.float64).pin_memory()
    host_in.numpy()[:] = prop.get_array().view(np.float64).ravel()
    e2e_steps = max(3, min(a.steps, 20))
    prop.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        prop.set_array_ptr(host_in.data_ptr())
        prop.steps(1)
        prop.get_array_ptr(host_out.data_ptr())
    e2e_s = allmax(world, time.perf_counter() - t0)
    e2e = {"value": points * e2e_steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": points * 16,
           "d2h_bytes_per_step": points * 16, "steps": e2e_steps,
           "note": "so_propagation_set_array (pinned FP64 host) + so_propagation_steps(1) + so_propagation_get_array"}

    # accuracy of this precision against the plain FP64 GPU path on the same inputs
    acc = {}
    if rank == 0:
        nchk = 100
        p64, _ = W.radial_angular_2d(nr=a.nr, nth=a.nth, step_no=nchk, precision="fp64")
        pfx, hf = W.radial_angular_2d(nr=a.nr, nth=a.nth, step_no=nchk, precision=a.precision)
        p64.steps(nchk)
        pfx.steps(nchk)
        acc = {"steps": nchk, "rel_l2": rel_l2(pfx.get_array(), p64.get_array()),
               "norm_drift": abs(pfx.norm() - p64.norm()),
               "loss_diff": abs(pfx.all_losses()[0] - p64.all_losses()[0])}
        # plain FP64 GPU path throughput on the same workload (the 20x denominator)
        p64.set_stream(stream.cuda_stream)
        fe = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
        for e0, e1 in fe:
            with torch.cuda.stream(stream):
                flush.zero_()
            e0.record(stream)
            p64.steps(1)
            e1.record(stream)
        p64.synchronize()
        torch.cuda.synchronize()
        f64_ms = sum(e0.elapsed_time(e1) for e0, e1 in fe) / len(fe)
        acc["fp64_gpu_value"] = points / (f64_ms / 1e3)
        acc["speedup_vs_fp64_gpu"] = value / world / acc["fp64_gpu_value"]

    if rank != 0:
        return
    cpu = None
    if not a.no_cpu_baseline:
        cpu = cpu_baseline(a, a.cpu_seconds)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if a.precision == "fp64" else "f32", "data": "synthetic",
            "config": {"workload": workload_name(a), "precision": a.precision,
                       "l2": "flushed before every timed step (256 MiB write, untimed)",
                       "parallelism": "replicas" if world > 1 else "single instance",
                       "global_batch": world, "wall_s_timed_region": wall},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clocks.summary(), "accuracy_vs_fp64": acc, "passes": [list(t) for t in kt]}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
