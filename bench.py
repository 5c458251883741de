"""Benchmark: batched FP32 C2C FFT, N=4096 x batch 65536 (2 GiB in, 2 GiB out).

One step = one forward transform of the whole batch (one kernel launch),
inputs resident in HBM, output to a separate buffer.  The working set (4 GiB)
is far larger than L2 (129 MB), so no flush is needed between steps.

metric = GFLOP/s = 5*N*log2(N)*batch / t (the reference harness's convention,
test/gfft_performance.h:67-78); the roofline object reports the same launch
as algorithmic HBM bytes (one read + one write of the data) per second.

`--impl reference` times the reference's algorithm on the host cores: the
compiled reference cannot run here (it needs the reference tree), so its CPU
restatement (oracle/gfft_restate.cpp, bit-exact with the compiled reference)
runs with OpenMP over the batch, all host threads.

Multi-GPU (torchrun, --gpus N): transforms are independent, so every rank
runs the same per-GPU batch with no collective on the data path ("weak"
scaling); a barrier brackets the timed region and the time is the max over
ranks.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 4096
BATCH = 65536
WORKLOAD = "fp32 c2c fft N=4096 x batch 65536, out of place"

# DRAM bytes (read + write) of one launch on this workload: the ncu capture
# summarised in profiles/spec_kernel_fp32_n4096.md measured 1.0248e9 bytes
# for batch 16384; traffic scales with the transforms processed (x4).
NCU_TRAFFIC_BYTES = {(4096, 65536): 4 * 1.0248e9}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=400)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--batch", type=int, default=BATCH)
    p.add_argument("--n", type=int, default=N)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    return p.parse_args()


def flops(n, batch):
    return 5.0 * n * math.log2(n) * batch


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(n, batch_sample, reps=3):
    """The reference's algorithm (CPU restatement) on all host threads over a
    bounded sample of the workload; min of `reps` runs after one warm-up."""
    import numpy as np

    from gfft_gb300 import inputs
    from oracle import pyoracle
    x = inputs.uniform(0x5EED0003, 2 * n * batch_sample).astype(np.float32)
    y = np.empty_like(x)
    pyoracle.gfft_batch(n, batch_sample, 1, 0, 1, x, y)
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        pyoracle.gfft_batch(n, batch_sample, 1, 0, 1, x, y)
        best = min(best, time.perf_counter() - t0)
    return {"value": flops(n, batch_sample) / best / 1e9, "unit": "GFLOP/s", "cores": pyoracle.num_threads(),
            "kind": "port",
            "sample": "%d transforms of N=%d fp32 (%.0f MiB), restatement of the reference's serial objects, "
                      "OpenMP over the batch, min of %d runs" % (batch_sample, n, 8 * n * batch_sample / 2 ** 20,
                                                                  reps)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    from oracle import pyoracle
    n = args.n
    # a bounded sample per step: about a second of CPU work
    sample = 4096
    import numpy as np

    from gfft_gb300 import inputs
    x = inputs.uniform(0x5EED0003, 2 * n * sample).astype(np.float32)
    y = np.empty_like(x)
    for _ in range(args.warmup):
        pyoracle.gfft_batch(n, sample, 1, 0, 1, x, y)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pyoracle.gfft_batch(n, sample, 1, 0, 1, x, y)
    dt = (time.perf_counter() - t0) / args.steps
    v = flops(n, sample) / dt / 1e9
    cores = pyoracle.num_threads()
    line = {"metric": "C2C FFT GFLOP/s (5Nlog2N/t)", "value": v, "unit": "GFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform[-1,1))",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "n": n, "batch": args.batch, "sample_batch": sample,
                       "l2": "inputs larger than L2 not applicable (host)"},
            "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": cores, "kind": "port",
                             "sample": "%d of the %d transforms per step; the reference's algorithm restated "
                                       "(bit-exact with the compiled reference), OpenMP over the batch"
                                       % (sample, args.batch)},
            "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    import gfft_gb300
    from gfft_gb300 import gfft as G
    world, rank, local = dist_setup(args)
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    gfft_gb300.build()
    n, batch = args.n, args.batch
    nel = 2 * n * batch
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    x = torch.rand(nel, device=dev, dtype=torch.float32, generator=g).mul_(2).sub_(1)
    y = torch.empty_like(x)
    obj = G.TransformObject(n, G.FLOAT, G.DFT, 1, G.Serial, G.OUT_OF_PLACE, batch)
    info = obj.info()
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(max(3, args.warmup)):
        obj.fft(x, y)
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for i in range(args.steps):
        obj.fft(x, y)
        ev[i + 1].record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    clk = clocks.stop()
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = t.item()
    ms = total_ms / args.steps
    value = flops(n, batch) * world / (ms * 1e-3) / 1e9

    # roofline of the engine kernel: one launch per step
    launch_ms = statistics.mean(per) / info["kernels_per_exec"]
    alg_bytes = 2 * nel * 4  # read + write
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": NCU_TRAFFIC_BYTES.get((n, batch)), "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": launch_ms}

    # end to end through the C ABI host entry point, pinned host buffers
    e2e = None
    if not args.no_e2e:
        hx = x.cpu().pin_memory()
        hy = torch.empty_like(hx).pin_memory()
        obj.fft(hx, hy)  # allocates the staging buffer once
        e2e_steps = max(3, min(args.steps, 10))
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            obj.fft(hx, hy)
        e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
        e2e = {"value": flops(n, batch) * world / (e_ms * 1e-3) / 1e9, "unit": "GFLOP/s",
               "h2d_bytes_per_step": nel * 4, "d2h_bytes_per_step": nel * 4, "ms_per_step": e_ms,
               "path": "gfft_exec_host (C ABI): pinned H2D + transform + D2H + stream sync"}
        del hx, hy

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(n, 4096)
        except Exception as e:  # reported, never fatal
            cpu = {"value": None, "error": str(e)[:200]}
    if rank == 0:
        line = {"metric": "C2C FFT GFLOP/s (5Nlog2N/t)", "value": value, "unit": "GFLOP/s", "n_gpus": world,
                "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (uniform[-1,1), torch rng)",
                "config": {"workload": WORKLOAD, "n": n, "batch": batch, "bytes_in": nel * 4,
                           "l2": "inputs larger than L2 (4 GiB working set), no flush",
                           "plan": {"passes": info["n_global_passes"], "radices": info["radices"],
                                    "threads": info["threads"], "units": info["units"],
                                    "variant": info["kernel_variant"]}},
                "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": args.steps * info["kernels_per_exec"]}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
