#!/usr/bin/env python3
"""Benchmark of the C2C FFT execute path on one GB300 (or N replicas).

Default workload: 1D complex FP64 C2C, N = 2^24, forward + inverse (the
single-transform case of the benchmark configuration "1D complex FP64 C2C
forward+inverse: single N=2^24 and batched 256x2^16").  One step = one
forward and one inverse transform of the device-resident array.

  value     GFLOP/s (5 N log2 N per direction), whole job, device-resident
            data (inputs in HBM when the timed region starts)
  e2e       the same metric through the C interface with host buffers:
            every step uploads the input from pinned memory (tope1DUpload)
            and runs tope1DExec FORWARD and INVERSE, each of which reads the
            result back into the host buffer (the reference's Exec contract)
  roofline  the dominant kernel (the pass kernel): algorithmic bytes per
            launch (2 * 16 B * points: one read and one write of the array)
            over its average launch time, from CUDA events around every
            launch inside the timed region, against the measured HBM copy
            bandwidth
  cpu_baseline  the reference's own kernels (oracle/_ref) or, where they
            were not built, the oracle's restatement, on this host's cores,
            on a bounded sample of the same workload

--impl reference times only that CPU implementation (rank 0).
Multi-GPU (torchrun): independent replicas, one per GPU, no collective on
the data path; value = units of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes
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

WORKLOADS = {
    "1d_2p24": {"dims": (1 << 24, 1, 1), "batch": 1,
                "desc": "1D C2C FP64, N=2^24, forward+inverse, uniform[-1,1) re/im"},
    "1d_256x2p16": {"dims": (1 << 16, 1, 1), "batch": 256,
                    "desc": "1D C2C FP64, batched 256 x 2^16, forward+inverse, uniform[-1,1) re/im"},
    "2d_4096": {"dims": (4096, 4096, 1), "batch": 1,
                "desc": "2D C2C FP64 4096x4096, forward+inverse, N(0,1) re/im"},
    "3d_256": {"dims": (256, 256, 256), "batch": 1,
               "desc": "3D C2C FP64 256^3, forward+inverse, N(0,1) re/im"},
    "1d_4096": {"dims": (4096, 1, 1), "batch": 1,
                "desc": "1D C2C FP64, N=4096, batch 1, forward+inverse, uniform[-1,1) re/im"},
    "3d_512": {"dims": (512, 512, 512), "batch": 1,
               "desc": "3D C2C FP64 512^3, forward+inverse, N(0,1) re/im (the FP64 comparison "
                       "point of the split-precision 512^3 configuration)"},
    "1d_4096x2p14": {"dims": (1 << 14, 1, 1), "batch": 4096,
                     "desc": "1D C2C FP64 batched 4096 x 2^14, forward+inverse, uniform re/im "
                             "(the FP64 comparison point of the split-precision configuration)"},
    "f32_3d_512": {"dims": (512, 512, 512), "batch": 1, "f32": True,
                   "desc": "split precision: 3D C2C 512^3, FP32 data, uniform[-1,1) field + "
                           "Gaussian pulse 1e6 (sigma 4) on the real part, forward+inverse"},
    "f32_1d_4096x2p14": {"dims": (1 << 14, 1, 1), "batch": 4096, "f32": True,
                         "desc": "split precision: 1D C2C batched 4096 x 2^14, FP32 data, "
                                 "uniform field + Gaussian pulse 1e6 (sigma 4) per row, "
                                 "forward+inverse"},
    "r2c_f32_1d_2p24": {"dims": (1 << 24, 1, 1), "batch": 1, "real": True, "f32": True,
                        "desc": "1D real-to-complex, split precision (FP32 data), N=2^24 "
                                "uniform[-1,1) reals, forward (R2C) + inverse (C2R); GFLOP/s "
                                "counts 2.5 N log2 N per direction"},
    "1d_97x2p20": {"dims": (97, 1, 1), "batch": 1 << 20,
                   "desc": "1D C2C FP64, batched 2^20 x 97 (a prime below 128: the exact "
                           "O(N^2) DFT kernel), forward+inverse, uniform[-1,1) re/im; GFLOP/s "
                           "counts the nominal 5 N log2 N per direction"},
    "r2c_1d_2p24": {"dims": (1 << 24, 1, 1), "batch": 1, "real": True,
                    "desc": "1D real-to-complex FP64, N=2^24 uniform[-1,1) reals, forward (R2C) "
                            "+ inverse (C2R); GFLOP/s counts 2.5 N log2 N per direction"},
    "1d_1e6": {"dims": (1000000, 1, 1), "batch": 1,
               "desc": "1D C2C FP64, N=10^6 = 2^6 5^6 (not a power of two: two mixed-radix "
                       "passes of 1000-point lines), forward+inverse, uniform[-1,1) re/im"},
    "1d_prime": {"dims": (999983, 1, 1), "batch": 1,
                 "desc": "1D C2C FP64, N=999983 (prime: Bluestein over 2^a 3^b 5^c 7^d-point "
                         "sub-transforms), forward+inverse, uniform[-1,1) re/im"},
    "batch_uneven": {"uneven": True, "f32": False,
                     "desc": "uneven batch: 20,000 1D transforms N=2^k, k~U{6..16}, plus 500 2D "
                             "transforms with sides from {64..1024}, uniform re/im, FP64, "
                             "forward+inverse; one persistent launch per direction from a "
                             "captured CUDA graph"},
    "batch_uneven_f32": {"uneven": True, "f32": True,
                         "desc": "uneven batch as batch_uneven, split precision (FP32 data)"},
    "batch_uneven_small": {"uneven": True, "f32": False, "n1d": 2000, "n2d": 50,
                           "desc": "uneven batch drawn like batch_uneven with 2,000 1D and 50 2D "
                                   "transforms (a profiling-size case, ~0.5 GB), FP64"},
}


def uneven_shapes(seed=None, n1d=20000, n2d=500):
    """The uneven batch: 1D lengths 2^k, k uniform on 6..16, then 2D shapes
    with NX, NY drawn independently from {64,...,1024}; SplitMix64-seeded."""
    u = splitmix_uniform((n1d + 2 * n2d + 1) // 2 + 1, SEED0 + 5 if seed is None else seed)
    u01 = (u + 1.0) / 2.0
    k = 6 + np.minimum((u01[:n1d] * 11).astype(int), 10)
    sides = np.array([64, 128, 256, 512, 1024])
    s = sides[np.minimum((u01[n1d:n1d + 2 * n2d] * 5).astype(int), 4)]
    nx = [int(1 << int(v)) for v in k] + [int(v) for v in s[0::2]]
    ny = [1] * n1d + [int(v) for v in s[1::2]]
    return nx, ny
# split-precision modes: library constant name, and the arithmetic name of its profiles
SPLIT_MODES = {"accurate": 0, "fast": 1, "tensor": 2}
SPLIT_ARITH = {"accurate": "df32", "fast": "f32", "tensor": "tc"}
METRIC = "C2C GFLOP/s & HBM GB/s vs roofline, FP64 plain vs split-precision at stated rel-L2"
SEED0 = 0x70E0F0F7
L2_BYTES = 129 * 10 ** 6
FALLBACK_HBM_GBS = 6800.0
# measured on a GB300 (profiles/fp_pipe_rates_gb300.md): DFMA 0.50 Tinstr/s (1.0 TFLOP/s)
FP64_PIPE_TFLOPS = 1.0


# ------------------------------------------------------------------ inputs
def splitmix_uniform(n_complex: int, seed: int) -> np.ndarray:
    """uniform[-1,1): value e = 2*u(seed, e) - 1, u from SplitMix64 >> 11."""
    out = np.empty(2 * n_complex)
    chunk = 1 << 22
    with np.errstate(over="ignore"):
        for s in range(0, 2 * n_complex, chunk):
            idx = np.arange(s, min(s + chunk, 2 * n_complex), dtype=np.uint64)
            z = np.uint64(seed) + (idx + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
            out[s:s + len(idx)] = 2.0 * ((z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53) - 1.0
    return out


def splitmix_normal(n_complex: int, seed: int) -> np.ndarray:
    u = splitmix_uniform(n_complex, seed)  # in [-1, 1)
    u1 = (u[0::2] + 1.0) / 2.0
    u2 = (u[1::2] + 1.0) / 2.0
    r = np.sqrt(-2.0 * np.log1p(-u1))
    out = np.empty(2 * n_complex)
    out[0::2] = r * np.cos(2 * np.pi * u2)
    out[1::2] = r * np.sin(2 * np.pi * u2)
    return out


def pulse_field(dims, batch, seed=SEED0 + 4, amp=1e6, sigma=4.0) -> np.ndarray:
    """uniform[-1,1) field plus amp*exp(-r^2/(2 sigma^2)) on the real part,
    centred on the grid (on each row for batched 1D)."""
    nx, ny, nz = dims
    x = splitmix_uniform(nx * ny * nz * batch, seed)
    g = [np.arange(n, dtype=np.float64) - n // 2 for n in (nz, ny, nx)]
    p = amp * np.exp(-(g[0][:, None, None] ** 2 + g[1][None, :, None] ** 2 +
                       g[2][None, None, :] ** 2) / (2 * sigma * sigma)).ravel()
    x[0::2] += np.tile(p, batch)
    return x


def make_input(wl: dict) -> np.ndarray:
    nx, ny, nz = wl["dims"]
    n = nx * ny * nz * wl["batch"]
    if wl.get("real"):
        return splitmix_uniform(n // 2, SEED0 + 2)  # n reals
    if wl.get("f32"):
        return pulse_field(wl["dims"], wl["batch"])
    if ny * nz > 1:
        return splitmix_normal(n, SEED0 + 3)
    return splitmix_uniform(n, SEED0 + 2)


def flops_per_step(wl: dict) -> float:
    nx, ny, nz = wl["dims"]
    n = nx * ny * nz
    per_dir = (2.5 if wl.get("real") else 5.0) * n * np.log2(n)
    return 2 * per_dir * wl["batch"]


def pass_points(wl: dict) -> int:
    """Complex points one pass launch of the dominant kernel moves: the array,
    its packed half for real data, or, for a 1D length with a prime factor
    above 13, the sub-transform of its Bluestein plan."""
    nx, ny, nz = wl["dims"]
    n = nx * ny * nz
    if wl.get("real"):
        return n // 2 * wl["batch"]
    if ny * nz == 1 and n >= 128 and not smooth(n, (2, 3, 5, 7, 11, 13)):
        # the library's choice: the next power of two >= 2n - 1, or the
        # smallest 2^a 3^b 5^c 7^d >= 2n - 1 when that is at most 0.6 of it
        mp = 1
        while mp < 2 * n - 1:
            mp *= 2
        m = 2 * n - 1
        while not smooth(m, (2, 3, 5, 7)):
            m += 1
        return (m if 10 * m <= 6 * mp else mp) * wl["batch"]
    return n * wl["batch"]


def sig(v: float, digits: int = 5) -> float:
    """v to `digits` significant digits (CPU rates of the O(N^2) reference
    path are far below 1e-4 GFLOP/s)."""
    return float(f"{v:.{digits}g}")


def smooth(n: int, primes) -> bool:
    for p in primes:
        while n % p == 0:
            n //= p
    return n == 1


def p_min(n: int, fp32: bool = False) -> int:
    return int(np.ceil(np.log2(n) / (14 if fp32 else 13)))


# ------------------------------------------------------------------ helpers
def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the
    platform string)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":", 1)[0].strip() == "Model name":
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def workload_config(args, wl: dict) -> dict:
    """The `config` object of a bench line: the workload alone, identical in
    both arms (what computes it is described outside `config`)."""
    if wl.get("uneven"):
        nx, ny = uneven_shapes(n1d=wl.get("n1d", 20000), n2d=wl.get("n2d", 500))
        total = sum(a * b for a, b in zip(nx, ny))
        es = 8 if wl.get("f32") else 16
        extra = {"transforms": len(nx)}
    else:
        nx_, ny_, nz_ = wl["dims"]
        total = nx_ * ny_ * nz_ * wl["batch"]
        es = 8 if wl.get("f32") else 16
        extra = {}
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return dict({"workload": args.workload, "description": wl["desc"], "points": total},
                **extra,
                l2=(f"inputs larger than L2 ({total * es >> 20} MiB array vs 129 MB L2)"
                    if total * es > L2_BYTES else "array fits in L2 (latency-bound size)"),
                parallelism=f"replicas x{ws}")


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(workload: str, arith: str):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu
    summary for this workload (profiles/*.txt line 'traffic_bytes_per_launch:')."""
    for p in sorted((ROOT / "profiles").glob(f"*_kernel_{arith}_{workload}.txt")):
        for line in p.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                try:
                    return int(float(line.split(":", 1)[1].split()[0]))
                except ValueError:
                    return None
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.6)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws: int, use_cuda: bool):
    if ws <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("nccl" if use_cuda else "gloo")
    return dist


def max_over_ranks(dist, value: float, device=None) -> float:
    """Max of a float over all ranks (identity without a process group)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(dist, local_ms_per_step: float, units_per_rank: float, device=None):
    """Whole-job rate: all ranks' units over the slowest rank's time."""
    ws = dist.get_world_size() if dist is not None else 1
    ms = max_over_ranks(dist, local_ms_per_step, device)
    return ms, units_per_rank * ws / (ms * 1e-3)


# ------------------------------------------------------------------ CPU leg
def cpu_reference_rate(wl: dict, budget_s: float = 30.0, steps: int = 1, warmup: int = 0):
    """Time the reference's kernels (oracle/_ref) or the oracle's restatement
    on the host cores; returns (GFLOP/s, dict).  The sample shrinks (1D: a
    shorter length, others: fewer steps) when a full step would not fit."""
    import oracle
    kind = "reference" if oracle.REF_SO.exists() else "port"
    emu = oracle.RefEmu() if kind == "reference" else oracle.Oracle()
    cores = os.cpu_count() or 1
    emu.set_threads(cores)
    nx, ny, nz = wl["dims"]
    batch = wl["batch"]
    x = make_input(wl)
    n_all = nx * ny * nz
    if ny * nz == 1 and n_all & (n_all - 1) and n_all >= 128:
        # the reference's non-power-of-two path is its O(n^2) DFT kernel
        # (kernels1D.cl:549-573): time it on a shorter length and scale by n^2
        n_s = 20000
        xs = x[: 2 * n_s]
        dft = emu.dft if hasattr(emu, "dft") else emu.dft_ref
        dft(xs, n_s)
        t0 = time.perf_counter()
        dft(xs, n_s)
        t_s = time.perf_counter() - t0
        t = 2 * t_s * (n_all / n_s) ** 2  # forward + inverse
        gflops = flops_per_step(wl) / t / 1e9
        sample = (f"the reference DFT (O(n^2)) at n={n_s}, forward, {t_s:.3f} s on {cores} threads, "
                  f"scaled by (n/{n_s})^2 to n={n_all} and doubled for the inverse")
        return gflops, {"value": sig(gflops), "unit": "GFLOP/s", "cores": cores,
                        "cpu_model": cpu_model(), "kind": kind, "sample": sample,
                        "ms_per_step": t * 1e3}
    if wl.get("real"):
        # the reference has no real-data path: its complex transform of the
        # reals with zero imaginary parts
        z = np.zeros(2 * n_all * batch)
        z[0::2] = x
        x = z

    def one(xs, dims, b):
        t0 = time.perf_counter()
        if b == 1:
            y = emu.exec(xs, *dims, 1)
            emu.exec(y, *dims, 0)
        else:  # the reference has no batched 1D: rows one by one
            n = dims[0]
            for i in range(b):
                row = xs[2 * n * i: 2 * n * (i + 1)]
                y = emu.exec(row, n, 1, 1, 1)
                emu.exec(y, n, 1, 1, 0)
        return time.perf_counter() - t0

    sample_dims, sample_batch, xs = (nx, ny, nz), batch, x
    if batch > 1:  # time a bounded number of rows
        sample_batch = min(batch, 16)
        xs = x[: 2 * nx * sample_batch]
    for _ in range(warmup):
        one(xs, sample_dims, sample_batch)
    times = []
    t_start = time.perf_counter()
    for _ in range(max(1, steps)):
        times.append(one(xs, sample_dims, sample_batch))
        if time.perf_counter() - t_start > budget_s:
            break
    t = statistics.median(times)
    n_s = sample_dims[0] * sample_dims[1] * sample_dims[2]
    flops = flops_per_step(dict(wl, dims=sample_dims, batch=sample_batch))
    gflops = flops / t / 1e9
    sample = (f"{'x'.join(map(str, sample_dims))} x batch {sample_batch}, forward+inverse, "
              f"{len(times)} timed step(s), median {t:.3f} s, {cores} threads")
    return gflops, {"value": sig(gflops), "unit": "GFLOP/s", "cores": cores,
                    "cpu_model": cpu_model(), "kind": kind, "sample": sample,
                    "ms_per_step": t * 1e3}


# ------------------------------------------------------------------ GPU leg
def run_gpu(args, wl: dict) -> dict:
    import torch
    import __graft_entry__ as g
    T = g.load_package()
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    os.environ["TOPEFFT_DEVICE"] = str(local)
    dist = dist_init(ws, True)
    nx, ny, nz = wl["dims"]
    batch = wl["batch"]
    n = nx * ny * nz
    total = n * batch
    f32 = bool(wl.get("f32"))
    real = bool(wl.get("real"))
    es = 8 if f32 else 16
    x = make_input(wl)
    xs = x.astype(np.float32) if f32 else x  # what the plan stores

    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    T.topeSetArith(f, T.TOPE_ARITH_DF64 if args.arith == "df64" else T.TOPE_ARITH_FP64)
    T.topeSetSplitMode(f, SPLIT_MODES[args.split])

    def make_plan(data, single):
        if ny * nz == 1:
            p = T.TopePlan1D()
            if single:
                T.tope1DBatchPlanInitF32(f, p, nx, batch, T.R2C if real else T.C2C, data)
            elif batch == 1:
                T.tope1DPlanInit(f, p, nx, T.R2C if real else T.C2C, data)
            else:
                T.tope1DBatchPlanInit(f, p, nx, batch, T.R2C if real else T.C2C, data)
        elif nz == 1:
            p = T.TopePlan2D()
            (T.tope2DPlanInitF32 if single else T.tope2DPlanInit)(f, p, nx, ny, T.C2C, data)
        else:
            p = T.TopePlan3D()
            (T.tope3DPlanInitF32 if single else T.tope3DPlanInit)(f, p, nx, ny, nz, T.C2C, data)
        T.check(f)
        return p

    def destroy(p):
        {T.TopePlan1D: T.tope1DDestroy, T.TopePlan2D: T.tope2DDestroy,
         T.TopePlan3D: T.tope3DDestroy}[type(p)](f, p)

    t = make_plan(xs.copy(), f32)
    stream = torch.cuda.ExternalStream(f.command_queue)

    def step():
        T.execDevice(f, t, T.FORWARD)
        T.execDevice(f, t, T.INVERSE)

    for _ in range(args.warmup):
        step()
    T.topeSync(f)
    sampler = ClockSampler(local)
    sampler.start()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    T.topeSync(f)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = sampler.stop()
    T.check(f)
    ms_local = e0.elapsed_time(e1) / args.steps
    ms, value = aggregate(dist, ms_local, flops_per_step(wl), device=torch.device("cuda", local))
    value_gflops = value / 1e9

    # per-launch kernel times for the roofline, in a separate loop: the event
    # pair around every launch would otherwise add to small steps' time
    pt_steps = max(1, min(args.steps, 10))
    T.topeSetPassTiming(f, 1)
    T.topeResetPassTimes(f, t)
    for _ in range(pt_steps):
        step()
    T.topeSync(f)
    T.check(f)
    passes = T.pass_times(f, t)
    T.topeSetPassTiming(f, 0)
    launches = sum(p["launches"] for p in passes) * args.steps // pt_steps

    # accuracy after all the round trips above (forward then inverse each step)
    back = np.empty_like(xs)
    (T.downloadF32 if f32 else T.download)(f, t, back)
    xs64 = xs.astype(np.float64)
    rt = float(np.sqrt(np.sum((back.astype(np.float64) - xs64) ** 2) / np.sum(xs64 * xs64)))
    accuracy = None
    if (f32 or args.arith == "df64") and not real:
        # one forward transform against the library's own native-FP64 path on
        # the FP64 input (before FP32 rounding for FP32 data); that path is
        # parity-tested against the oracle by the GPU tests
        if f32:
            T.uploadF32(f, t, xs)
            T.execF32(f, t, back, T.FORWARD)
        else:
            T.upload(f, t, xs)
            {T.TopePlan1D: T.tope1DExec, T.TopePlan2D: T.tope2DExec,
             T.TopePlan3D: T.tope3DExec}[type(t)](f, t, back, T.FORWARD)
        T.check(f)
        saved = f.arith
        T.topeSetArith(f, T.TOPE_ARITH_FP64)
        ref = x.copy()
        p64 = make_plan(ref, False)
        (T.tope1DExec if ny * nz == 1 else T.tope2DExec if nz == 1 else T.tope3DExec)(
            f, p64, ref, T.FORWARD)
        T.check(f)
        destroy(p64)
        T.topeSetArith(f, saved)
        got = back.astype(np.float64)
        accuracy = {"rel_l2_vs_fp64": float(np.sqrt(np.sum((got - ref) ** 2) / np.sum(ref * ref))),
                    "max_abs_vs_fp64": float(np.max(np.abs(got - ref))),
                    "max_abs_ref": float(np.max(np.abs(ref))),
                    "reference": ("the library's native-FP64 path on the same FP64 input, one "
                                  "forward transform (that path is checked against the oracle "
                                  "by the GPU tests)"),
                    "gate": 1e-7 if f32 else 1e-13 * float(np.log2(total))}
        del ref, got

    # dominant kernel: the pass with the largest total time
    dom = max(passes, key=lambda p: p["ns"]) if passes else None
    bytes_per_launch = 2 * es * pass_points(wl)
    peak, peak_kind = measured_peaks()
    roof = None
    if dom and dom["launches"]:
        avg_ns = dom["ns"] / dom["launches"]
        ach = bytes_per_launch / avg_ns  # bytes/ns == GB/s
        roof = {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "peak_source": peak_kind,
                "traffic": ncu_traffic(args.workload, SPLIT_ARITH[args.split] if f32 else args.arith),
                "kernel": ((f"tc_pass_kernel L=2^{dom['log_l']}" if f32 and args.split == "tensor"
                            and dom["log_l"] >= 4 else f"pass_kernel L=2^{dom['log_l']}")
                           if dom["log_l"] >= 0 else f"mixed_kernel L={dom['len']}") +
                          f" B={dom['b_tile']} ({dom['ctas']} CTAs x {dom['threads']} threads)",
                "launch_us": round(avg_ns / 1e3, 2),
                "bytes_per_launch": bytes_per_launch,
                "fp64_pipe_tflops_measured": FP64_PIPE_TFLOPS}
        if not f32 and args.arith == "fp64":
            # native FP64 is bound by the FP64 pipe: the whole step's
            # algorithmic flops against the measured DFMA rate (2 flops each)
            roof["fp64_pipe"] = {"achieved_gflops": round(value_gflops, 1),
                                 "peak_gflops": FP64_PIPE_TFLOPS * 1e3,
                                 "frac": round(value_gflops / (FP64_PIPE_TFLOPS * 1e3), 4),
                                 "basis": "5 N log2 N per direction over the step time, "
                                          "against the measured DFMA rate x 2"}

    # e2e through the C interface with pinned host buffers
    nbytes = xs.nbytes
    # a real plan's forward writes n + 2 doubles per row
    host_vals = (n + 2) * batch if real else 2 * total
    hp = T.lib.topeHostAlloc(host_vals * (4 if f32 else 8))
    ctype = ctypes.c_float if f32 else ctypes.c_double
    host = np.ctypeslib.as_array((ctype * host_vals).from_address(hp))
    host[:xs.size] = xs
    if f32:
        exec_fn, up_fn = T.execF32, T.uploadF32
    else:
        exec_fn = {T.TopePlan1D: T.tope1DExec, T.TopePlan2D: T.tope2DExec,
                   T.TopePlan3D: T.tope3DExec}[type(t)]
        up_fn = T.upload

    def e2e_step():
        up_fn(f, t, hp)
        exec_fn(f, t, hp, T.FORWARD)
        exec_fn(f, t, hp, T.INVERSE)

    e2e_steps = max(3, min(args.steps, 20))
    e2e_step()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    t1 = time.perf_counter()
    T.check(f)
    e2e_ms, e2e_val = aggregate(dist, (t1 - t0) * 1e3 / e2e_steps, flops_per_step(wl),
                                device=torch.device("cuda", local))
    T.lib.topeHostFree(hp)

    destroy(t)

    if f32 and args.split == "fast":
        arith_desc = "split precision, fast: FP32 data and butterflies, FP64-accurate hi/lo twiddles"
    elif f32 and args.split == "tensor":
        arith_desc = ("split precision, tensor: FP32 data, radix-16 stages as tcgen05 GEMMs on "
                      "three-piece FP16 splits (an exact leading FP32 accumulator and a "
                      "cross-product one), double-float twiddles and exchange, FP64-accurate "
                      "hi/lo twiddle tables")
    elif f32:
        arith_desc = ("split precision, accurate: FP32 data, double-float butterflies on chip, "
                      "FP64-accurate hi/lo twiddles")
    elif args.arith == "df64":
        arith_desc = "double-float (FP32 pairs) on FP64 storage"
    else:
        arith_desc = "native FP64"
    res = {
        "metric": METRIC, "value": round(value_gflops, 3), "unit": "GFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if f32 else "f64",
        "data": "synthetic (SplitMix64-seeded)",
        "config": workload_config(args, wl),
        "arith": arith_desc,
        "hbm_gbs_effective": round((launches / args.steps) * bytes_per_launch / (ms * 1e-3) / 1e9, 1),
        "rel_l2_roundtrip": rt,
        "accuracy": accuracy,
        "roofline": roof,
        "passes": passes,
        "e2e": {"value": round(e2e_val / 1e9, 3), "unit": "GFLOP/s",
                "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": (2 * nbytes + 16 * batch) if real else 2 * nbytes,
                "ms_per_step": round(e2e_ms, 3)},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        _, cpu = cpu_reference_rate(wl, budget_s=30.0, steps=5, warmup=1)
        res["cpu_baseline"] = cpu
    if dist is not None:
        dist.destroy_process_group()
    return res if rank == 0 else None


def batch_flops(nx, ny) -> float:
    return float(sum(2 * 5.0 * a * b * np.log2(a * b) for a, b in zip(nx, ny)))


def batch_bytes_per_launch(nx, ny, es) -> int:
    """algorithmic bytes of one direction: each pass reads and writes its
    class once (1D up to 2^12 and ... one pass, longer 1D and 2D two)"""
    tot = 0
    for a, b in zip(nx, ny):
        passes = 1 if (b == 1 and a <= 4096) else 2
        tot += passes * 2 * es * a * b
    return tot


def run_batch(args, wl: dict) -> dict:
    import torch
    import __graft_entry__ as g
    T = g.load_package()
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    os.environ["TOPEFFT_DEVICE"] = str(local)
    dist = dist_init(ws, True)
    f32 = wl["f32"]
    es = 8 if f32 else 16
    nx, ny = uneven_shapes(n1d=wl.get("n1d", 20000), n2d=wl.get("n2d", 500))
    total = sum(a * b for a, b in zip(nx, ny))
    x = splitmix_uniform(total, SEED0 + 6)
    xs = x.astype(np.float32) if f32 else x
    del x
    f = T.TopeFFT()
    T.topeFFTInit(f)
    T.check(f)
    T.topeSetArith(f, T.TOPE_ARITH_DF64 if args.arith == "df64" else T.TOPE_ARITH_FP64)
    T.topeSetSplitMode(f, SPLIT_MODES[args.split])
    b = T.TopeBatch()
    t_plan = time.perf_counter()
    T.topeBatchPlanInit(f, b, nx, ny, T.C2C, xs)
    t_plan = time.perf_counter() - t_plan
    T.check(f)
    stream = torch.cuda.ExternalStream(f.command_queue)
    flops = batch_flops(nx, ny)

    def timed(mode, steps, warm):
        T.topeBatchSetMode(f, b, mode)
        for _ in range(warm):
            T.topeBatchExecDevice(f, b, T.FORWARD)
            T.topeBatchExecDevice(f, b, T.INVERSE)
        T.topeSync(f)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            T.topeBatchExecDevice(f, b, T.FORWARD)
            T.topeBatchExecDevice(f, b, T.INVERSE)
        e1.record(stream)
        T.topeSync(f)
        T.check(f)
        return e0.elapsed_time(e1) / steps

    auto_mode = b.mode  # chosen by the plan-time autotuner
    sampler = ClockSampler(local)
    sampler.start()
    ms_local = timed(auto_mode, args.steps, args.warmup)
    clocks = sampler.stop()
    ms, value = aggregate(dist, ms_local, flops, device=torch.device("cuda", local))
    ms_persistent = (ms_local if auto_mode == T.TOPE_BATCH_PERSISTENT
                     else timed(T.TOPE_BATCH_PERSISTENT, max(2, args.steps // 4), 1))
    ms_launches = (ms_local if auto_mode == T.TOPE_BATCH_LAUNCHES
                   else timed(T.TOPE_BATCH_LAUNCHES, max(2, args.steps // 4), 1))
    ms_loop = timed(T.TOPE_BATCH_LOOP, 2, 1)
    T.topeBatchSetMode(f, b, auto_mode)
    # accuracy: round trip of the last steps
    back = np.empty_like(xs)
    T.topeBatchDownload(f, b, back)
    T.check(f)
    x64 = xs.astype(np.float64)
    rt = float(np.sqrt(np.sum((back.astype(np.float64) - x64) ** 2) / np.sum(x64 * x64)))
    # e2e: upload from pinned memory, Exec forward and inverse with read-back
    nbytes = xs.nbytes
    hp = T.lib.topeHostAlloc(nbytes)
    ctype = ctypes.c_float if f32 else ctypes.c_double
    host = np.ctypeslib.as_array((ctype * xs.size).from_address(hp))
    host[:] = xs
    hbuf = host  # typed view for the Exec read-back
    e2e_steps = max(2, min(args.steps, 5))
    T.topeBatchUpload(f, b, hp)
    T.topeBatchExec(f, b, hbuf, T.FORWARD)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        T.topeBatchUpload(f, b, hp)
        T.topeBatchExec(f, b, hbuf, T.FORWARD)
        T.topeBatchExec(f, b, hbuf, T.INVERSE)
    t1 = time.perf_counter()
    T.check(f)
    e2e_ms, e2e_val = aggregate(dist, (t1 - t0) * 1e3 / e2e_steps, flops,
                                device=torch.device("cuda", local))
    T.lib.topeHostFree(hp)
    classes, ctas, items = b.classes, b.ctas, b.work_items
    T.topeBatchDestroy(f, b)
    bytes_launch = batch_bytes_per_launch(nx, ny, es)
    peak, peak_kind = measured_peaks()
    ach = bytes_launch / (ms / 2 * 1e-3) / 1e9
    res = {
        "metric": METRIC, "value": round(value / 1e9, 3), "unit": "GFLOP/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if f32 else "f64", "data": "synthetic (SplitMix64-seeded)",
        "config": workload_config(args, wl),
        "arith": ("split " + args.split) if f32 else args.arith,
        "batch_plan": {"classes": classes, "work_items": items, "persistent_ctas": ctas},
        "mode": {0: "persistent_graph", 1: "per_class_launch_graph"}.get(auto_mode, "loop"),
        "modes_ms_per_step": {"persistent_graph": round(ms_persistent, 3),
                              "per_class_launch_graph": round(ms_launches, 3),
                              "per_transform_loop": round(ms_loop, 3)},
        "speedup_vs_per_transform_loop": round(ms_loop / ms_local, 2),
        "plan_seconds_incl_autotune": round(t_plan, 2),
        "rel_l2_roundtrip": rt,
        "roofline": {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(ach / peak, 4), "peak_source": peak_kind, "traffic": None,
                     "kernel": ("batch_kernel (one persistent launch per direction)"
                                if auto_mode == 0 else "pass_kernel launches (graph per direction)"),
                     "bytes_per_launch": bytes_launch,
                     "launch_us": round(ms / 2 * 1e3, 1)},
        "e2e": {"value": round(e2e_val / 1e9, 3), "unit": "GFLOP/s",
                "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": 2 * nbytes,
                "ms_per_step": round(e2e_ms, 3)},
        "gpu_launches": 2 * args.steps,
        "clocks": clocks,
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        res["cpu_baseline"] = cpu_batch_rate(nx, ny)
    if dist is not None:
        dist.destroy_process_group()
    return res if rank == 0 else None


def cpu_batch_rate(nx, ny, budget_s=20.0):
    """The reference's kernels on host cores over the first transforms of the
    batch, one plan per transform (as the reference would run them)."""
    import oracle
    kind = "reference" if oracle.REF_SO.exists() else "port"
    emu = oracle.RefEmu() if kind == "reference" else oracle.Oracle()
    cores = os.cpu_count() or 1
    emu.set_threads(cores)
    flops, t, i = 0.0, 0.0, 0
    while i < len(nx) and t < budget_s:
        a, b = nx[i], ny[i]
        xs = splitmix_uniform(a * b, SEED0 + i)
        t0 = time.perf_counter()
        y = emu.exec(xs, a, b, 1, 1)
        emu.exec(y, a, b, 1, 0)
        t += time.perf_counter() - t0
        flops += 2 * 5.0 * a * b * np.log2(a * b)
        i += 1
    return {"value": round(flops / t / 1e9, 4), "unit": "GFLOP/s", "cores": cores,
            "cpu_model": cpu_model(), "kind": kind,
            "sample": f"first {i} transforms of the batch, forward+inverse each, {t:.1f} s"}


def run_reference(args, wl: dict):
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    if wl.get("uneven"):
        nx, ny = uneven_shapes(n1d=wl.get("n1d", 20000), n2d=wl.get("n2d", 500))
        cpu = cpu_batch_rate(nx, ny, budget_s=60.0)
        gflops = cpu["value"]
        cpu["ms_per_step"] = batch_flops(nx, ny) / (gflops * 1e9) * 1e3
    else:
        gflops, cpu = cpu_reference_rate(
            wl, budget_s=150.0 / max(1, args.steps + args.warmup) * args.steps,
            steps=args.steps, warmup=min(args.warmup, 1))
    return {"impl": "reference", "metric": METRIC, "value": sig(gflops), "unit": "GFLOP/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(cpu["ms_per_step"], 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (SplitMix64-seeded)",
            "config": workload_config(args, wl),
            "arith": "the reference's FP64 kernels on the host cores of rank 0",
            "cpu_baseline": cpu,
            "e2e": {"value": sig(gflops), "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def companion(args, wl: dict, res64: dict, label: str, *, workload=None, arith=None,
              split=None) -> dict:
    """One extra measurement on the default line: the same (or a named)
    workload with another arithmetic, with its own roofline, accuracy and
    speed-up over the line's plain FP64 value."""
    a = argparse.Namespace(**vars(args))
    a.no_cpu_baseline, a.steps = True, min(args.steps, 20)
    if workload is not None:
        a.workload = workload
        wl = WORKLOADS[workload]
    if arith is not None:
        a.arith = arith
    if split is not None:
        a.split = split
        wl = dict(wl, f32=True)
    r = run_gpu(a, wl)
    out = {"mode": label, "workload": a.workload, "value": r["value"], "unit": r["unit"],
           "ms_per_step": r["ms_per_step"], "steps": a.steps,
           "rel_l2_roundtrip": r["rel_l2_roundtrip"],
           "speedup_vs_fp64_line": round(r["value"] / res64["value"], 3),
           "roofline": r.get("roofline"), "e2e": (r.get("e2e") or {}).get("value"),
           "gpu_launches": r.get("gpu_launches"), "clocks": r.get("clocks")}
    if r.get("accuracy"):
        out["accuracy"] = r["accuracy"]
    return out


def split_companion(args, wl: dict, res64: dict) -> dict:
    """The metric sets the plain FP64 path against the split-precision form at
    its stated error: the same workload with FP32 storage (input with the 1e6
    Gaussian pulse), its rel-L2 against the library's FP64 path (itself
    parity-tested against the oracle), and its speed-up over the FP64 line."""
    r = companion(args, wl, res64, "split precision, " + args.split_companion_mode,
                  split=args.split_companion_mode)
    acc = r.get("accuracy") or {}
    r.update({"rel_l2_vs_fp64": acc.get("rel_l2_vs_fp64"),
              "max_abs_vs_fp64": acc.get("max_abs_vs_fp64"), "gate": 1e-7,
              "speedup_vs_fp64": r["speedup_vs_fp64_line"],
              "roofline_frac": (r.get("roofline") or {}).get("frac"),
              "input": "the same workload's uniform field plus a 1e6 Gaussian pulse, stored as FP32"})
    return r


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="1d_2p24")
    ap.add_argument("--arith", choices=["fp64", "df64"], default="fp64")
    ap.add_argument("--split", choices=sorted(SPLIT_MODES), default="accurate",
                    help="arithmetic of the FP32 (split-precision) workloads")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-split-companion", action="store_true",
                    help="skip the split-precision run added to FP64 complex workloads")
    ap.add_argument("--split-companion-mode", choices=sorted(SPLIT_MODES), default="accurate",
                    help="split-precision mode of that run")
    ap.add_argument("--no-companions", action="store_true",
                    help="skip the double-float and 3D 256^3 runs added to the default line")
    args = ap.parse_args(argv)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        res = run_reference(args, wl)
    elif wl.get("uneven"):
        res = run_batch(args, wl)
    else:
        res = run_gpu(args, wl)
        npts = wl["dims"][0] * wl["dims"][1] * wl["dims"][2]
        if (res is not None and not args.no_split_companion and not wl.get("f32")
                and not wl.get("real") and npts & (npts - 1) == 0
                and int(os.environ.get("WORLD_SIZE", "1")) == 1):
            res["split_precision"] = split_companion(args, wl, res)
            if args.split_companion_mode != "tensor":
                # the tensor form (tcgen05 stages) on the same workload
                res["split_precision_tensor"] = split_companion(
                    argparse.Namespace(**dict(vars(args), split_companion_mode="tensor")), wl, res)
        if (res is not None and not args.no_companions and args.workload == "1d_2p24"
                and args.arith == "fp64" and int(os.environ.get("WORLD_SIZE", "1")) == 1):
            # the double-float arithmetic on FP64 data (same gate as FP64)
            # and the second workload of the FP64 target, 3D 256^3
            res["df64"] = companion(args, wl, res, "double-float FP64 (FP32 pairs)",
                                    arith="df64")
            res["fp64_3d_256"] = companion(args, wl, res, "native FP64", workload="3d_256")
            res["df64_3d_256"] = companion(args, wl, res, "double-float FP64 (FP32 pairs)",
                                           workload="3d_256", arith="df64")
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
