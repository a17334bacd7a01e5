"""Benchmark: fused FREQ_OFFSET_REAL convolution on GB300.

Workload (one step): fftset_fft_conv over 16384 independent blocks of 1536
complex bins (3072 real floats each), Gaussian input sigma = 1, kernel of 3072
taps = seeded Gaussian x exp(-t/400) prepared once with
fftset_fft_conv_get_kernel; one batched launch. Algorithmic bytes per step:
one read of every input block, one write of every output block, one read of
the kernel spectrum: 16384 * 24576 + 12288 = 402,665,472 B. Inputs (201 MB)
exceed L2 (129 MB), so no flush is needed between steps.

value     GB/s on device-resident buffers (CUDA events on the launching stream)
e2e       same metric through the C ABI with pinned HOST buffers, so each step
          includes the host->device copy of the input and the device->host copy
          of the output
roofline  the conv kernel against the measured HBM copy bandwidth
cpu_baseline  the oracle's C restatement of the reference, all host cores

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "conv/FFT GB/s vs 8 TB/s HBM; ragged-batch vs per-call speedup at relL2≤2e-6·logN"
L = 1536
BLOCKS = 16384
TAPS = 2 * L
BYTES_PER_STEP = BLOCKS * (2 * L * 4) * 2 + 2 * L * 4
WORKLOAD = "freqoffsetreal_conv_L1536_x16384"


def make_inputs(rank: int = 0):
    rng = np.random.default_rng(2 + 1000 * rank)
    x = rng.standard_normal((BLOCKS, 2 * L), dtype=np.float32)
    t = np.arange(TAPS)
    h = (np.random.default_rng(3).standard_normal(TAPS) * np.exp(-t / 400.0)).astype(np.float32)
    return x, h


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of the conv kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get(WORKLOAD)
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled while the GPU works."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def cpu_baseline(x, h, nthreads=None, reps=3):
    """Oracle C restatement of the reference on all host cores (bounded sample:
    the full 16384-block workload, best of `reps`)."""
    from oracle import oracle as O
    nthreads = nthreads or os.cpu_count() or 1
    kind = "port"
    P = O.PortPlan(O.MOD_FREQ_OFFSET_REAL, L, 4)
    K = P.get_kernel(h)
    out = np.empty_like(x)
    best = None
    for _ in range(reps):
        s = P.run_batch("conv", out, x, K, nthreads=nthreads)
        best = s if best is None else min(best, s)
    return {"value": BYTES_PER_STEP / best / 1e9, "unit": "GB/s", "cores": nthreads, "kind": kind,
            "sample": f"{BLOCKS} blocks x {L} bins, {nthreads} threads, best of {reps}",
            "seconds_per_step": best}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return world, rank, local


def run_reference(args):
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return
    from oracle import oracle as O
    x, h = make_inputs(0)
    nthreads = os.cpu_count() or 1
    P = O.PortPlan(O.MOD_FREQ_OFFSET_REAL, L, 4)
    K = P.get_kernel(h)
    out = np.empty_like(x)
    for _ in range(args.warmup):
        P.run_batch("conv", out, x, K, nthreads=nthreads)
    secs = [P.run_batch("conv", out, x, K, nthreads=nthreads) for _ in range(args.steps)]
    t = sum(secs) / len(secs)
    value = BYTES_PER_STEP / t / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "complex_bins": L, "blocks": BLOCKS, "bytes_per_step": BYTES_PER_STEP,
                   "note": "oracle C restatement of the reference (the reference sources are not on this host)"},
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": nthreads, "kind": "port",
                         "sample": f"{BLOCKS} blocks x {L} bins per step, {nthreads} threads"},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gb300(args):
    import torch
    world, rank, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    import fftset_gb300 as fs

    S = fs.FftSet()
    f = S.create_fft(fs.FREQ_OFFSET_REAL, L)
    x_np, h_np = make_inputs(rank)
    x = torch.from_numpy(x_np).cuda()
    h = torch.from_numpy(h_np).cuda()
    K = torch.empty_like(h)
    f.conv_get_kernel(K, h)
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    S.set_stream(stream)
    S.set_blocking(False)

    def step():
        f.conv_batch(y, x, K)

    # autotune: every compiled kernel for this size, plus the generic one
    # (--variant V pins one kernel instead)
    sweep = {}
    for v in (range(-1, f.variants) if args.variant is None else []):
        try:
            f.set_variant(fs.OP_CONV, v)
        except fs.FftsetError:
            continue
        for _ in range(3):
            step()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(10):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        sweep[str(v)] = ev0.elapsed_time(ev1) / 10
    if args.variant is None:
        tuned_ms = f.autotune(fs.OP_CONV, BLOCKS)
    else:
        f.set_variant(fs.OP_CONV, args.variant)
        tuned_ms = None
    variant = f.variant(fs.OP_CONV)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    # parity of the benchmarked output (first blocks) against the oracle
    from oracle import oracle as O
    nchk = 64
    P = O.PortPlan(O.MOD_FREQ_OFFSET_REAL, L, 4)
    y_ref = P.conv(x_np[:nchk], P.get_kernel(h_np))
    rel = O.rel_l2(y[:nchk].cpu().numpy(), y_ref)
    rel64 = O.rel_l2(y[:nchk].cpu().numpy(), O.negacyclic_conv64(x_np[:nchk], h_np))

    sampler = ClockSampler(local)
    sampler.start()
    t_soak = time.perf_counter()
    while time.perf_counter() - t_soak < 1.0:  # keep the GPU loaded while the sampler spins up
        for _ in range(50):
            step()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * BYTES_PER_STEP / (ms * 1e-3) / 1e9

    # end to end through the C ABI with pinned host buffers
    S.set_blocking(True)
    xh = torch.from_numpy(x_np).pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    f.conv_batch(yh, xh, K)
    e2e_steps = max(3, min(args.steps, 20))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        f.conv_batch(yh, xh, K)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_ok = O.rel_l2(yh[:nchk].numpy(), y_ref) <= O.tolerance(2 * L)

    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_STEP / (ms * 1e-3) / 1e9
    if rank == 0:
        cb = cpu_baseline(x_np, h_np) if world == 1 else None
        line = {
            "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "complex_bins": L, "blocks_per_gpu": BLOCKS, "taps": TAPS,
                       "bytes_per_step_per_gpu": BYTES_PER_STEP, "l2": "inputs larger than L2 (201 MB > 129 MB)",
                       "parity_relL2_vs_port": rel, "parity_relL2_vs_fp64": rel64,
                       "kernel_variant": variant, "variant_ms": sweep, "autotune_ms": tuned_ms,
                       "tolerance": O.tolerance(2 * L)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": ncu_traffic()},
            "cpu_baseline": cb,
            "e2e": {"value": world * BYTES_PER_STEP / e2e_s / 1e9, "unit": "GB/s",
                    "h2d_bytes_per_step": int(x_np.nbytes), "d2h_bytes_per_step": int(x_np.nbytes),
                    "parity_ok": bool(e2e_ok)},
            "gpu_launches": args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line))
    S.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--variant", type=int, default=None,
                    help="pin the conv kernel variant (-1 generic) instead of autotuning")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
