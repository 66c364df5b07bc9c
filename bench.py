#!/usr/bin/env python3
"""Benchmark of the cuda compute methods (one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

A step is one pass of the hot path over one batch of synthetic input (see
WORKLOADS). `value` is whole-job throughput with inputs resident in HBM; `e2e`
is the same metric through the C-ABI call on pinned HOST buffers with the
host<->device copies inside the timed region. Steps are timed with CUDA events on
the stream the kernels run on; L2 is flushed (a 256 MiB write) between timed
steps, outside the timed spans. `--impl reference` times the CPU restatement of
particular's rayon method (the oracle, all host threads) on the same workload.
Multi-GPU runs are independent replicas (the path has no exchange step).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


# --------------------------------------------------------------------------- utils
def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="bf_plummer_131072")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[4:]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        pmax = max(r[2] for r in rows)
        loaded = [r for r in rows if r[2] >= 0.5 * pmax] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in loaded:
            for nm, v in zip(names, r[3][1:]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": loaded[0][1],
                "power_w_max": pmax, "samples": len(loaded), "reasons": sorted(reasons)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return json.load(open(path))
    except (OSError, ValueError):
        return {}


# --------------------------------------------------------------------------- workloads
class BruteForceWorkload:
    """All-pairs accelerations of an N=131072 Plummer sphere (a=1, M=1, equal masses),
    softening 0.01, compensated FP32: one acceleration evaluation per step."""

    name = "bf_plummer_131072"
    metric = "bodies/s"
    unit = "bodies/s"

    def __init__(self, n=131072, softening=0.01):
        from particular_gb300 import ics
        self.n = n
        self.softening = softening
        self.bodies = ics.plummer(n)["bodies"]

    def config(self):
        return {"workload": self.name, "n_bodies": self.n, "softening": self.softening,
                "ic": "Plummer a=1 M=1 equal masses, seeded SplitMix64",
                "interaction": "AccelerationSoftened checked", "method": "cuda::BruteForce",
                "l2": "flushed between timed steps (256 MiB write)"}

    # ---- GPU arm
    def setup_gpu(self, res, torch, stream):
        self.torch = torch
        self.res = res
        self.d_b = torch.from_numpy(self.bodies).to("cuda")
        self.d_out = torch.empty((self.n, 3), dtype=torch.float32, device="cuda")
        self.h_b = torch.from_numpy(self.bodies).pin_memory()
        self.h_out = torch.empty((self.n, 3), dtype=torch.float32).pin_memory()

    def step_device(self):
        from particular_gb300 import _native as N
        N.check(N.lib().pt_bf_accel_f32_device(self.res.handle, self.d_b.data_ptr(), self.n,
                                               self.d_b.data_ptr(), self.n, self.softening, 1, 0,
                                               self.d_out.data_ptr()))

    def step_e2e(self):
        from particular_gb300 import _native as N
        N.check(N.lib().pt_bf_accel_f32(self.res.handle, self.h_b.data_ptr(), self.n,
                                        self.h_b.data_ptr(), self.n, self.softening, 1, 0,
                                        self.h_out.data_ptr()))

    def h2d_d2h_bytes(self):
        return 16 * self.n, 12 * self.n

    def roofline(self, res, step_ms):
        from particular_gb300 import _native as N
        import ctypes
        peak = ctypes.c_double(0)
        N.check(N.lib().pt_measure_fp32_peak(res.handle, ctypes.byref(peak)))
        achieved = 20.0 * self.n * self.n / (step_ms * 1e-3) / 1e12
        return {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                "frac": achieved / peak.value, "traffic": None,
                "kernel": "bf_fast (+ bf_fixup)",
                "algorithmic": "20 flop per pair interaction x N^2 pairs per launch",
                "peak_source": "measured FFMA-chain kernel over all SMs (pt_measure_fp32_peak)"}

    # ---- CPU arm (oracle: parallel::BruteForce restated, all host threads)
    def cpu_step(self, threads, sample):
        from oracle import oracle as O
        idx = np.linspace(0, self.n - 1, sample).astype(np.int64)
        t0 = time.perf_counter()
        O.bf_f32(self.bodies[idx], self.bodies, self.softening, True, threads=threads)
        dt = time.perf_counter() - t0
        return sample / dt  # full-evaluation bodies/s: every target costs N pairs

    def cpu_sample(self):
        return 8192


WORKLOADS = {BruteForceWorkload.name: BruteForceWorkload}


# --------------------------------------------------------------------------- arms
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import build as obuild, oracle as O
    obuild.build()
    wl = WORKLOADS[args.workload]()
    threads = O.max_threads()
    sample = wl.cpu_sample()
    for _ in range(max(0, min(args.warmup, 1))):
        wl.cpu_step(threads, max(256, sample // 8))
    rates = [wl.cpu_step(threads, sample) for _ in range(args.steps)]
    value = statistics.mean(rates)
    line = {"metric": wl.metric, "value": value, "unit": wl.unit, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wl.n / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": wl.config(), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": wl.unit, "cores": threads, "kind": "port",
                             "sample": f"{sample} targets of the full source set per step"},
            "e2e": {"value": value, "unit": wl.unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    torch.cuda.set_device(local)
    from particular_gb300 import CudaResources, build_native
    build_native.build()
    wl = WORKLOADS[args.workload]()
    res = CudaResources(local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    res.set_stream(stream.cuda_stream)
    wl.setup_gpu(res, torch, stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def timed(step, k):
        spans = []
        for _ in range(k):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            spans.append((e0, e1))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in spans)

    for _ in range(max(3, args.warmup)):
        wl.step_device()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = res.launch_count
    barrier()
    t_ms = timed(wl.step_device, args.steps)
    barrier()
    launches = res.launch_count - launches0
    clk = clocks.stop()
    for _ in range(2):
        wl.step_e2e()
    barrier()
    t_e2e = timed(wl.step_e2e, args.steps)
    barrier()
    if dist:
        tt = torch.tensor([t_ms, t_e2e], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms, t_e2e = tt.tolist()
    step_ms = t_ms / args.steps
    value = world * wl.n / (step_ms * 1e-3)
    e2e_value = world * wl.n / (t_e2e / args.steps * 1e-3)
    h2d, d2h = wl.h2d_d2h_bytes()
    roof = wl.roofline(res, step_ms)
    if rank != 0:
        return 0
    line = {"metric": wl.metric, "value": value, "unit": wl.unit, "n_gpus": world,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": wl.config(),
            "roofline": roof,
            "e2e": {"value": e2e_value, "unit": wl.unit, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": t_e2e / args.steps},
            "gpu_launches": int(launches), "clocks": clk}
    if not args.no_cpu_baseline:
        from oracle import build as obuild, oracle as O
        obuild.build()
        threads = O.max_threads()
        rate = wl.cpu_step(threads, wl.cpu_sample())
        line["cpu_baseline"] = {"value": rate, "unit": wl.unit, "cores": threads, "kind": "port",
                                "sample": f"{wl.cpu_sample()} targets against all sources"}
    print(json.dumps(line), flush=True)
    res.close()
    return 0


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
