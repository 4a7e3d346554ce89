#!/usr/bin/env python
"""Benchmark of the split-operator propagation step on GB300.

Default workload (``--workload batch``): 512 independent 2-D radial x angular
propagations of uneven sizes -- Nr drawn from {512..8192}, Ntheta from
{32, 64, 128, 256} (Gauss-Legendre, Legendre transform to l_max = Ntheta - 1),
Morse D(1-e^{-a(r-re)})^2 + beta e^{-r/2} P2(cos th) with D, a, re, beta seeded per
instance, mass 1000, dt = 0.5, border damping with a loss checker, stack
[Damp, V/2, Legendre, Rot/2, FFT, K] -- stepped together by the batched executor
(FP32 state, split-BF16x6 tensor-core Legendre transforms -- three fixed-point bf16 slices
per operand, exact FP32 sums -- FP64 norm folds and loss).  The
states and tables (~4.2 GB) are far larger than L2, so no flush is needed.
One bench step = one split-operator time step of all 512 instances.

``--workload single`` is the single 4096 x 128 problem (L2 flushed before every
timed step).  ``--impl reference`` times the reference's CPU algorithm instead (the
C++ FP64 restatement in oracle/, all host threads) on the same workload.
Prints ONE JSON line (rank 0).
"""
import argparse
import json
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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "single"])
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--precision", default="fp32_bf16x6",
                    choices=["fp64", "fp32_tf32x3", "fp32_bf16x3", "fp32_bf16x6", "fp32_simt", "float_float"])
    ap.add_argument("--nr", type=int, default=4096)
    ap.add_argument("--nth", type=int, default=128)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true",
                    help="timed region only (no e2e, accuracy or CPU legs): the case profiled under ncu")
    ap.add_argument("--no-ground-state", action="store_true", help="skip the time-to-ground-state leg")
    ap.add_argument("--ground-state-sets", type=int, default=16,
                    help="held-out parameter sets of the time-to-ground-state leg")
    ap.add_argument("--no-tune", action="store_true",
                    help="built-in launch schedules (the autotuner is skipped)")
    ap.add_argument("--tune-cache", default=None,
                    help="autotuner schedule cache: loaded instead of tuning when it exists, else written")
    return ap.parse_args()


def workload_name(a):
    if a.workload == "batch":
        return (f"batched radial x angular: {a.instances} instances, Nr in {{512..8192}}, Ntheta in {{32,64,128,256}} "
                "(GL), Morse D~U[0.05,0.2] a~U[0.6,1.4] re~U[2,4] + beta~U[0,0.05] e^(-r/2) P2, mass 1000, dt=0.5, "
                "damping+loss, stack [Damp,V/2,L,Rot/2,F,K], seeds default_rng(1000+i)")
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
    """Measured DRAM bytes per algorithmic byte of each kernel (dram__bytes_read.sum +
    dram__bytes_write.sum over the captured launches, divided by those launches'
    algorithmic bytes), from the committed ncu summary; {} when absent."""
    p = os.path.join(ROOT, "profiles", "dram_traffic_ratio.txt")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            if line.strip() and not line.startswith("#"):
                k, v = line.split()[:2]
                out[k] = float(v)
    return out


def kernel_of(group_name):
    """The CUDA kernel a batched group runs: its name carries the pass family."""
    if "tc3xtf32" in group_name or "tcbf16x3" in group_name or "tcbf16x6" in group_name:
        return "angular_tc_kernel_batched"
    if "fftpair" in group_name:
        # float-float pairs run their own instantiation
        return "fft_pair_kernel_batched_ff" if " ff " in f" {group_name} " else "fft_pair_kernel_batched"
    if "scalar" in group_name:
        return "scalar_program_kernel"
    return "pass_kernel_batched"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo" if os.environ.get("SO_BENCH_GLOO") else "nccl")
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
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rel_l2(x, y):
    import numpy as np
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


# ------------------------------------------------------------------ CPU legs
def cpu_sample(a):
    """Instances the CPU legs time: the single problem, or a size-stratified sample of the batch."""
    if a.workload == "single":
        return [dict(nr=a.nr, nth=a.nth, seed=2026, d=0.1, a=1.0, re=3.0, beta=0.02)]
    from split_operator_gb300 import workloads as W
    params = W.batched_instance_params(a.instances)
    # two instances of every (Nr, Ntheta) class present, in instance order
    seen, out = {}, []
    for p in params:
        k = (p["nr"], p["nth"])
        if seen.get(k, 0) < 2:
            seen[k] = seen.get(k, 0) + 1
            out.append(p)
    return out


def cpu_rate(a, seconds, steps=None):
    """pt*steps/s of the C++ FP64 restatement of the reference passes on all host threads."""
    from oracle import cpu_port as P
    threads = os.cpu_count() or 1
    sample = cpu_sample(a)
    ports = [P.RadialAngular(s["nr"], s["nth"], seed=s["seed"], d=s["d"], a=s["a"], re=s["re"], beta=s["beta"])
             for s in sample]
    for pt in ports:
        pt.run(1, threads=threads)  # warm-up
    if steps is None:
        t0 = time.perf_counter()
        for pt in ports:
            pt.run(1, threads=threads)
        one = time.perf_counter() - t0
        steps = max(1, min(200, int(seconds / max(one, 1e-6))))
    t0 = time.perf_counter()
    for pt in ports:
        pt.run(steps, threads=threads)
    dt = time.perf_counter() - t0
    pts = sum(s["nr"] * s["nth"] for s in sample)
    desc = (f"{steps} steps of {len(sample)} instances ({pts} grid points: two of every Nr x Ntheta class of the "
            "batch)" if a.workload == "batch" else f"{steps} steps of the {a.nr}x{a.nth} problem")
    return pts * steps / dt, threads, desc + ", FP64, C++ restatement of the reference passes (oracle/cpu_port.cpp)"


def run_reference(a):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    v, threads, desc = cpu_rate(a, a.cpu_seconds, steps=max(1, a.steps // 10))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_name(a), "precision": "fp64 (reference algorithm, CPU)",
                       "note": "the Rust crate cannot be built here; its algorithm runs as a C++ restatement"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU leg
def build_props(a, precision, count=None, world=1, rank=0):
    """This rank's propagations.  Batched workload on N > 1 GPUs: the instance list holds N x
    `instances` seeded instances and each rank takes its shard (longest processing time first
    by Nr x Ntheta): per-GPU work stays fixed as N grows, with no exchange between ranks."""
    from split_operator_gb300 import workloads as W
    if a.workload == "single":
        return [W.radial_angular_2d(nr=a.nr, nth=a.nth, step_no=10 ** 6, precision=precision)[0]]
    n = count or a.instances
    if world > 1:
        from split_operator_gb300 import shards
        mine, _ = shards.shard(W.batched_instance_params(n * world), world, rank)
        return W.batched_radial_angular(len(mine), precision=precision, step_no=10 ** 6, params=mine)
    return W.batched_radial_angular(n, precision=precision, step_no=10 ** 6)


def global_points(a, world, points):
    """Grid points of the whole job: the full instance list (N > 1, batched), else N replicas."""
    if world == 1 or a.workload == "single":
        return points * world
    from split_operator_gb300 import workloads as W
    return sum(p["nr"] * p["nth"] for p in W.batched_instance_params(a.instances * world))


def roofline_from(times, total_ms):
    """Roofline of the kernel with the largest share of the timed step: its algorithmic
    bytes over all its launches divided by its summed CUDA-event launch times."""
    hbm, _, peak_kind = measured_peaks()
    if not times:
        return None
    agg = {}
    for name, n, tms, b in times:
        k = agg.setdefault(kernel_of(name), [0, 0.0, 0.0, []])
        k[0] += n
        k[1] += tms
        k[2] += b
        k[3].append(name)
    kern, (n, tms, b, groups) = max(agg.items(), key=lambda kv: kv[1][1])
    ach = b / (tms / 1e3) / 1e9
    ratio = ncu_traffic().get(kern)
    return {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "traffic": ratio * b / n if ratio else None, "kernel": kern, "launches": n,
            "avg_us": tms / n * 1e3, "algorithmic_bytes_per_launch": b / n,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per algorithmic byte on a "
                              "96-instance batch, scaled to this launch's algorithmic bytes" if ratio else None,
            "peak_source": f"{peak_kind} hbm_gbs (burst copy)",
            "share_of_timed": tms / total_ms if total_ms > 0 else None, "groups": len(groups)}


def run_ours(a):
    import numpy as np
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    import split_operator_gb300 as so

    stream = torch.cuda.Stream()
    props = build_props(a, a.precision, world=world, rank=rank)
    for p in props:
        p.set_stream(stream.cuda_stream)
    points = sum(int(np.prod(p.wave_function_shape())) for p in props)  # this rank's
    job_points = global_points(a, world, points)
    single = a.workload == "single"
    batch = None if single else so.Batch(props)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if single else None

    def run_steps(k, timing):
        if single:
            props[0].set_timing(timing)
            evs = []
            for _ in range(k):
                with torch.cuda.stream(stream):
                    flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                props[0].steps(1)
                e1.record(stream)
                evs.append((e0, e1))
            props[0].synchronize()
            torch.cuda.synchronize()
            kt = props[0].kernel_times() if timing else []
            props[0].set_timing(False)
            return sum(x.elapsed_time(y) for x, y in evs), kt
        batch.set_timing(timing)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.steps(k)
        e1.record(stream)
        torch.cuda.synchronize()
        kt = batch.kernel_times() if timing else []
        batch.set_timing(False)
        return e0.elapsed_time(e1), kt

    # launch schedules: the built-in ones are timed first (for the record), then the autotuner
    # picks per lane extent on this workload (states restored) unless a cache file is given
    tune = None
    if not single and not a.no_tune:
        import tempfile
        so.reset_schedules()
        run_steps(a.warmup, False)
        ms_default, _ = run_steps(a.steps, False)
        cache = a.tune_cache or os.path.join(tempfile.gettempdir(), f"split_operator_gb300_schedules_{os.getpid()}.json")
        if a.tune_cache and os.path.exists(a.tune_cache):
            so.load_schedules(a.tune_cache)
            rep = {"loaded_from": a.tune_cache}
        else:
            t0 = time.perf_counter()
            rep = batch.tune(cache, trial_steps=3)
            rep["tune_wall_s"] = time.perf_counter() - t0
        tune = {"default_schedule_ms_per_step": ms_default / a.steps, "report": rep}
    run_steps(a.warmup, False)
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    n0 = so.launch_count()
    barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    ms, kt = run_steps(a.steps, single)  # batch: production path (CUDA graph); single: per-pass events
    wall = time.perf_counter() - wall0
    barrier(world)
    launches = so.launch_count() - n0
    clocks.stop()
    ms_max = allmax(world, ms)
    value = job_points * a.steps / (ms_max / 1e3)
    if not single:
        # per-launch breakdown of the same K steps with CUDA events on every batched launch
        ms_t, kt = run_steps(a.steps, True)
    roof = roofline_from(kt, ms if single else ms_t)
    if tune is not None:
        tune["tuned_ms_per_step"] = ms_max / a.steps
        tune["gain"] = tune["default_schedule_ms_per_step"] / tune["tuned_ms_per_step"]

    if a.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms_max / a.steps,
                              "quick": True, "passes": [list(t) for t in kt], "roofline": roof, "autotune": tune}),
                  flush=True)
        return

    # end to end through the C ABI: pinned FP64 host state in, one step, state out
    e2e_steps = 5
    # every instance's state back to back in one pinned array (in and out), in member order:
    # the library then moves each pipeline chunk with one copy per direction
    sizes = [int(np.prod(p.wave_function_shape())) * 2 for p in props]
    host_in = torch.empty(sum(sizes), dtype=torch.float64).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    hosts = [host_in[int(offs[k]):int(offs[k + 1])] for k in range(len(props))]
    outs = [host_out[int(offs[k]):int(offs[k + 1])] for k in range(len(props))]
    for p, h in zip(props, hosts):
        h.numpy()[:] = p.get_array().view(np.float64).ravel()
    in_ptrs, out_ptrs = [h.data_ptr() for h in hosts], [o.data_ptr() for o in outs]

    def e2e_step():
        if single:
            props[0].set_array_ptr(in_ptrs[0])
            props[0].steps(1)
            props[0].get_array_ptr(out_ptrs[0])
        else:
            batch.steps_host_ptr(in_ptrs, out_ptrs, 1)

    for _ in range(3):  # warm-up (the first calls set up the chunk pipeline's streams and launch groups)
        e2e_step()
    torch.cuda.synchronize()
    # three timed runs of e2e_steps steps each; the median run is the figure (the host link
    # of a shared machine shows occasional stalls of a whole run)
    reps = []
    for _ in range(3):
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            e2e_step()
        reps.append(allmax(world, time.perf_counter() - t0))
    e2e_s = sorted(reps)[1]
    # one more step as three separate calls (each waited on), for the breakdown only
    ph = []
    t = time.perf_counter()
    if single:
        props[0].set_array_ptr(in_ptrs[0])
    else:
        batch.set_arrays_ptr(in_ptrs)
    torch.cuda.synchronize()
    ph.append(time.perf_counter() - t)
    t = time.perf_counter()
    props[0].steps(1) if single else batch.steps(1)
    torch.cuda.synchronize()
    ph.append(time.perf_counter() - t)
    t = time.perf_counter()
    if single:
        props[0].get_array_ptr(out_ptrs[0])
    else:
        batch.get_arrays_ptr(out_ptrs)
    ph.append(time.perf_counter() - t)
    e2e = {"value": job_points * e2e_steps / e2e_s, "unit": UNIT, "runs_ms_per_step": [r / e2e_steps * 1e3 for r in reps], "h2d_bytes_per_step": points * 16,
           "d2h_bytes_per_step": points * 16, "steps": e2e_steps,
           "unpipelined_phase_ms": {"set_arrays": ph[0] * 1e3, "steps": ph[1] * 1e3, "get_arrays": ph[2] * 1e3},
           "host_link_gbs": {"h2d": 211, "d2h": 193, "source": "cudaMemcpyAsync of 1 GiB pinned, measured on this "
                                                               "GPU model"},
           "note": ("every step: one so_batch_steps_host call: pinned FP64 host states of all instances in, one "
                    "step, states out to pinned host buffers, pipelined over 16 instance chunks on their own "
                    "streams (copy engines both ways); the instances' states lie back to back in one pinned "
                    "array per direction, so each chunk moves with one copy per direction") if not single else
                   "every step: so_propagation_set_array from a pinned FP64 host buffer, one step, "
                   "so_propagation_get_array into a pinned host buffer"}

    acc = {}
    if rank == 0:
        # accuracy against the plain FP64 GPU path on identical inputs
        from split_operator_gb300 import workloads as W
        nchk = 100
        if single:
            chk = [dict(nr=a.nr, nth=a.nth, seed=2026, d=0.1, a=1.0, re=3.0, beta=0.02)]
            classes = chk
        else:
            params = W.batched_instance_params(a.instances)
            chk = [next(p for p in params if p["nth"] == t and p["nr"] == r)
                   for t, r in ((32, 8192), (64, 4096), (128, 2048), (256, 4096))
                   if any(p["nth"] == t and p["nr"] == r for p in params)]
            # the first instance of every (Nr, Ntheta) size class of the batch
            first = {}
            for p in params:
                first.setdefault((p["nr"], p["nth"]), p)
            classes = [first[k] for k in sorted(first)]
        # one step from the same state (the metric's bound: rel-L2 <= 1e-6 against FP64): the FP32
        # mode's own rounded state is copied into an FP64 propagation, and both take one step
        one = []
        for c in classes:
            kw = dict(nr=c["nr"], nth=c["nth"], step_no=2, seed=c["seed"], d=c["d"], a=c["a"], re=c["re"],
                      beta=c["beta"])
            pfx = W.radial_angular_2d(precision=a.precision, **kw)[0]
            p64 = W.radial_angular_2d(precision="fp64", **kw)[0]
            p64.set_array(pfx.get_array())
            pfx.steps(1)
            p64.steps(1)
            one.append({"nr": c["nr"], "nth": c["nth"], "rel_l2": rel_l2(pfx.get_array(), p64.get_array())})
            del pfx, p64
        acc["one_step"] = {"classes": one, "max_rel_l2": max(e["rel_l2"] for e in one), "bound": 1e-6,
                           "within_bound": all(e["rel_l2"] <= 1e-6 for e in one)}
        errs = []
        for c in chk:
            kw = dict(nr=c["nr"], nth=c["nth"], step_no=nchk, seed=c["seed"], d=c["d"], a=c["a"], re=c["re"],
                      beta=c["beta"])
            p64 = W.radial_angular_2d(precision="fp64", **kw)[0]
            pfx = W.radial_angular_2d(precision=a.precision, **kw)[0]
            pff = W.radial_angular_2d(precision="float_float", **kw)[0]
            p64.steps(nchk)
            pfx.steps(nchk)
            pff.steps(nchk)
            x64 = p64.get_array()
            errs.append({"nr": c["nr"], "nth": c["nth"], "rel_l2": rel_l2(pfx.get_array(), x64),
                         "norm_diff": abs(pfx.norm() - p64.norm()),
                         "loss_diff": abs(pfx.all_losses()[0] - p64.all_losses()[0]),
                         "float_float_rel_l2": rel_l2(pff.get_array(), x64)})
            del p64, pfx, pff
        acc.update({"steps": nchk, "instances": errs, "max_rel_l2": max(e["rel_l2"] for e in errs)})
        # plain FP64 GPU path throughput on the same workload (the 20x denominator): every instance
        del batch
        if single:
            props64 = build_props(a, "fp64")
            points64 = points
        else:
            props64 = build_props(a, "fp64")
            points64 = points
            acc["fp64_gpu_instances"] = len(props64)
        f64_steps = 10
        if single:
            p64 = props64[0]
            evs = []
            for _ in range(f64_steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                p64.steps(1)
                e1.record()
                evs.append((e0, e1))
            p64.synchronize()
            torch.cuda.synchronize()
            f64_ms = sum(x.elapsed_time(y) for x, y in evs)
        else:
            b64 = so.Batch(props64)
            b64.steps(3)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            b64.steps(f64_steps)
            e1.record()
            torch.cuda.synchronize()
            f64_ms = e0.elapsed_time(e1)
        acc["fp64_gpu_value"] = points64 * f64_steps / (f64_ms / 1e3)
        acc["speedup_vs_fp64_gpu"] = value / world / acc["fp64_gpu_value"]
        del props64
        if not single:
            b64 = None
        # the float-float state (FP64-like accuracy on the FP32 pipes) on the same instances
        propsff = build_props(a, "float_float")
        if single:
            evs = []
            for _ in range(f64_steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                propsff[0].steps(1)
                e1.record()
                evs.append((e0, e1))
            propsff[0].synchronize()
            torch.cuda.synchronize()
            ff_ms = sum(x.elapsed_time(y) for x, y in evs)
        else:
            bff = so.Batch(propsff)
            bff.steps(3)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            bff.steps(f64_steps)
            e1.record()
            torch.cuda.synchronize()
            ff_ms = e0.elapsed_time(e1)
            bff = None
        acc["float_float_gpu_value"] = points64 * f64_steps / (ff_ms / 1e3)
        acc["float_float_vs_fp64_gpu"] = acc["float_float_gpu_value"] / acc["fp64_gpu_value"]
        acc["float_float_max_rel_l2"] = max(e["float_float_rel_l2"] for e in errs)
        del propsff

    tgs = None
    if rank == 0 and not single and not a.no_ground_state:
        # the metric's second half: time to the ground state, learned start vs Gaussian start
        from split_operator_gb300 import learned_start as LS
        if os.path.exists(LS.MODEL_2048x64):
            tgs = LS.time_to_ground_state(count=a.ground_state_sets)
        else:
            tgs = {"unavailable": "trained model file missing"}

    if rank != 0:
        return
    cpu = None
    if not a.no_cpu_baseline:
        v, threads, desc = cpu_rate(a, a.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms_max / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "float_float": "f32x2 (float-float)"}.get(a.precision, "f32"), "data": "synthetic",
            "config": {"workload": workload_name(a), "precision": a.precision, "grid_points": points,
                       "l2": ("inputs larger than L2 (states + tables ~" + f"{points * 24 / 1e9:.1f} GB)")
                       if not single else "flushed before every timed step (256 MiB write, untimed)",
                       "parallelism": ("single GPU" if world == 1 else "replicas" if single else
                                       "instance shards (longest processing time first by Nr x Ntheta)"),
                       "global_batch": len(props) * world if single or world == 1 else a.instances * world,
                       "job_grid_points": job_points, "wall_s_timed_region": wall},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clocks.summary(), "accuracy_vs_fp64": acc, "autotune": tune, "time_to_ground_state": tgs,
            "passes": [list(t) for t in kt]}
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
