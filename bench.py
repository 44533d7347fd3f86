#!/usr/bin/env python
"""Benchmark of the GB300 Givens hot path: the bulk application of k x (n-1) rotations to an
m x n matrix (bulk_wave_order_2x2_rmul!, src/wave.jl:36-162; benchmark/benchmark.jl:4-30),
on the microbenchmark workload Q 16384 x 16384 column-major FP64 ~ U[-1,1), k = 64 layers of
n-1 rotations (c,s) = (cos t, sin t), t ~ U[0, 2 pi).  Reported metric: Givens GFLOP/s with
6 flops per rotation per row (benchmark/benchmark.jl:10-11).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--dtype f64|f32]

One JSON line on rank 0.  `value` is device-timed with Q resident in HBM (Q is 2.1 GB, far
larger than the 129 MB L2, so no flush is needed between steps); `e2e` goes through the C ABI
entry point with pinned host buffers, copies included.  Under torchrun every rank runs its own
replica on its own GPU (the path does not shard; the reference's row slabs would need only a
broadcast of (c,s)), and `value` sums the replicas' work over the slowest rank's time.
`--impl reference` times the CPU restatement of the reference's wave kernel
(oracle/symeig_oracle.c, row-slab threaded like src/wave.jl:36-60) on all host cores.

The default line also carries, untimed by `value`, the other items of the metric:
  solve_n16384          qr_algorithm! at n = 16384 (case A) on the device, multishift chase,
                        with its errors, beside cpu_reference_solve_n16384, the reference's own
                        solve path (its chase, then every flush's grid by the row-slab threaded
                        wave kernel) timed on the host cores on a row sample of Q;
  solve_n2000[_multishift]  the README example (README.md:65-77);
  batched               4096 tridiagonals n ~ U{32..1024}: batched call vs a loop of single
                        solves on the batch's own matrices vs the host;
  adjoint               n = 4096 forward + backward / forward, with the gradient's error;
  f32_apply, scaled_form    the FP32 apply and the scaled FP64 form on the apply workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD = "bulk Givens apply: Q 16384x16384 column-major, k=64 layers of 16383 rotations (cos t, sin t)"
METRIC = "Givens GFLOP/s (6 flops per rotation per row), bulk apply 16384x16384 k=64"
TRAFFIC_FILE = ROOT / "profiles" / "wave_apply_f64_16384_k64.md"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--dtype", choices=["f64", "f32"], default="f64")
    p.add_argument("--m", type=int, default=16384)
    p.add_argument("--n", type=int, default=16384)
    p.add_argument("--k", type=int, default=64)
    p.add_argument("--no-extras", action="store_true", help="skip every side measurement of the default line")
    p.add_argument("--no-solve-extras", action="store_true",
                   help="skip the n=16384 solve, batched and adjoint keys of the default line")
    p.add_argument("--workload", choices=["apply", "solve", "batched", "adjoint", "dense"], default="apply",
                   help="apply: the bulk-apply microbenchmark (default); solve: one full qr_algorithm!")
    p.add_argument("--case", choices=["A", "B"], default="A",
                   help="solve workload: A d_i = i, e ~ U[0,1) (seed 1); B d ~ N(0,1), e ~ 0.5 N(0,1) (seed 2)")
    p.add_argument("--q", choices=["f64", "f32"], default="f64", help="solve workload: Q precision")
    p.add_argument("--oracle-check", action="store_true",
                   help="solve workload: also run the CPU oracle's chase (eigenvalues only) and compare bits")
    p.add_argument("--form", choices=["canonical", "scaled"], default="canonical",
                   help="FP64 apply form: canonical rotations (4 FP64 ops per rotation-row) or the "
                        "scaled form (2 FMAs per rotation-row; a few ulps from canonical)")
    p.add_argument("--chase-mode", type=int, choices=[0, 1, 2, 3], default=None,
                   help="solve/dense workloads (default 0) and the adjoint's forward (default 3): 0 Newton-form "
                        "two-warp chase, 1 reference form, 2 Newton + redo, 3 multishift batches")
    p.add_argument("--ms-bulges", type=int, default=64, help="solve workload, chase mode 3: bulge cap of a batch")
    p.add_argument("--ms-rows", type=int, default=16, help="solve workload, chase mode 3: block rows per bulge")
    p.add_argument("--ms-release", type=int, default=4, help="solve workload, chase mode 3: steps between progress releases")
    p.add_argument("--count", type=int, default=4096, help="batched workload: number of tridiagonals")
    p.add_argument("--loop-sample", type=int, default=16,
                   help="batched workload: matrices timed one launch per matrix (extrapolated by sum n^2)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def flops_per_step(m, n, k):
    return 6.0 * k * (n - 1) * m


def make_inputs(m, n, k, dtype, seed, device):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    tdt = torch.float64 if dtype == "f64" else torch.float32
    # column-major Q: a row-major (n, m) tensor viewed transposed
    Qt = (torch.rand(n, m, generator=g, dtype=torch.float64) * 2 - 1).to(tdt)
    th = torch.rand(k, n - 1, generator=g, dtype=torch.float64) * (2 * np.pi)
    cs = torch.stack([torch.cos(th), torch.sin(th)], -1).to(tdt).contiguous()  # Julia layout
    if device is not None:
        return Qt.to(device).T, cs.to(device)
    return Qt.T, cs


# ---- clocks -------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        self.device_index = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- CPU side (the oracle's port of the reference's wave kernel) ---------------------------
def cpu_wave_gflops(m, n, k, dtype, threads, target_s=8.0, max_rows=None):
    """Time the reference's wave-order kernel (C port, row slabs on `threads` threads, the
    timing build: contraction allowed and tuned for the host's cores) on a bounded row sample of
    the workload; GFLOP/s scales with rows, so the sample is representative.  Returns
    (gflops, rows, seconds, shape)."""
    from oracle import oracle as orc
    orc.build()
    rng = np.random.default_rng(1)
    npdt = np.float64 if dtype == "f64" else np.float32
    th = rng.random((n - 1, k)) * 2 * np.pi
    cs = np.empty((n - 1, k, 2), dtype=npdt)
    cs[..., 0] = np.cos(th)
    cs[..., 1] = np.sin(th)
    kk = k if k % 2 == 0 else k - 1          # the reference kernel needs even k and odd n-1
    nn = n if (n - 1) % 2 == 1 else n - 1
    cs = np.asfortranarray(cs[: nn - 1, :kk])
    rows = min(m, max(threads * 64, 256))
    while True:
        Q = np.asfortranarray(rng.random((rows, nn)).astype(npdt) * 2 - 1)
        t0 = time.perf_counter()
        orc.apply_wave(Q, cs, nthreads=threads, fast=True)
        dt = time.perf_counter() - t0
        cap = max_rows or m
        if dt >= target_s * 0.5 or rows >= cap:
            return flops_per_step(rows, nn, kk) / dt / 1e9, rows, dt, (rows, nn, kk)
        rows = int(min(cap, rows * max(2.0, min(16.0, target_s / max(dt, 1e-3)))))


_HOST_PEAK_SCRIPT = """
import json, time, numpy as np
n = 4096
a = np.random.default_rng(0).random((n, n)); b = np.random.default_rng(1).random((n, n))
a @ b
best = 1e30
for _ in range(3):
    t0 = time.perf_counter(); a @ b; best = min(best, time.perf_counter() - t0)
print(json.dumps(2.0 * n ** 3 / best / 1e9))
"""


def host_peak(threads):
    """DGEMM rate of the host (numpy's BLAS, n = 4096, best of 3) on one thread -- the
    analogue of the reference's single-threaded LinearAlgebra.peakflops() (README.md:28-34) --
    and on `threads` threads.  Each in a subprocess with the BLAS thread count fixed at start."""
    out = {"n": 4096, "kind": "numpy BLAS dgemm, best of 3"}
    for key, t in (("one_thread_gflops", 1), ("all_threads_gflops", threads)):
        env = dict(os.environ, OPENBLAS_NUM_THREADS=str(t), OMP_NUM_THREADS=str(t), MKL_NUM_THREADS=str(t))
        try:
            r = subprocess.run([sys.executable, "-c", _HOST_PEAK_SCRIPT], env=env, capture_output=True,
                               text=True, timeout=300)
            out[key] = round(float(r.stdout.strip().splitlines()[-1]), 2)
        except Exception as exc:  # reported, not fatal: the baseline stands without it
            out[key] = None
            out["error"] = f"{type(exc).__name__}"
    return out


def cpu_baseline_apply(m, n, k, dtype, threads):
    """The cpu_baseline object of the apply workload: the C port of the reference's wave
    kernel on all host cores and on one, with the host's DGEMM rates beside it."""
    gf, rows, dt, shape = cpu_wave_gflops(m, n, k, dtype, threads, target_s=8.0)
    cpu = {"value": round(gf, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
           "sample": (f"C port of the reference wave kernel (timing build), {threads} threads, {shape[0]} of {m} "
                      f"rows x {shape[1]} cols, k={shape[2]}, {dt:.1f} s")}
    gf1, _, dt1, shape1 = cpu_wave_gflops(m, n, k, dtype, 1, target_s=3.0, max_rows=1024)
    cpu["one_thread"] = {"value": round(gf1, 3), "unit": "GFLOP/s", "cores": 1,
                         "sample": f"{shape1[0]} of {m} rows x {shape1[1]} cols, k={shape1[2]}, {dt1:.1f} s"}
    hp = host_peak(threads)
    cpu["host_peak"] = hp
    if dtype == "f64" and hp.get("one_thread_gflops"):
        # the reference reports its kernel at 75% of single-thread dgemm (README.md:34)
        cpu["frac_of_host_peak"] = {"one_thread": round(gf1 / hp["one_thread_gflops"], 4)}
        if hp.get("all_threads_gflops"):
            cpu["frac_of_host_peak"]["all_threads"] = round(gf / hp["all_threads_gflops"], 4)
    return cpu


def replica_reduce(ms: float, world: int, device=None) -> float:
    """The job time of N independent replicas: the slowest rank's (all_reduce MAX); every
    rank returns it.  With world == 1 it is the rank's own time."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(work_per_rank: float, world: int, ms: float) -> float:
    """Whole-job throughput: the work of all replicas over the slowest replica's time (the
    path does not shard, so every rank does the same work on its own GPU)."""
    return work_per_rank * world / (ms * 1e-3)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals = []
    sample = None
    for i in range(args.warmup + args.steps):
        gf, rows, dt, shape = cpu_wave_gflops(args.m, args.n, args.k, args.dtype, threads, target_s=4.0)
        sample = shape
        if i >= args.warmup:
            vals.append((gf, dt))
    v = statistics.median([x[0] for x in vals])
    ms = statistics.median([x[1] for x in vals]) * 1e3
    desc = (f"C port of the reference's wave kernel (oracle/symeig_oracle.c, timing build), {threads} threads, "
            f"row sample {sample[0]} of {args.m} rows x {sample[1]} cols, k={sample[2]}")
    line = {
        "metric": METRIC, "value": round(v, 3), "unit": "GFLOP/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded U[-1,1) Q, (cos t, sin t) rotations)",
        "config": {"workload": WORKLOAD, "m": args.m, "n": args.n, "k": args.k, "parallelism": "cpu threads",
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": round(v, 3), "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": desc, "host_peak": host_peak(threads)},
        "e2e": {"value": round(v, 3), "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def hbm_side(algo_bytes: float, flops_per_launch: float, kernel_ms: float, peak_tflops: float) -> dict:
    """The other side of the roofline min(FMA peak, HBM bandwidth x intensity), with the HBM
    copy bandwidth measured on this machine (MEASURED_PEAKS.json)."""
    try:
        bw = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
        src = "MEASURED_PEAKS.json"
    except Exception:
        bw, src = 6800.0, "fallback 6.8 TB/s"
    intensity = flops_per_launch / algo_bytes
    achieved = algo_bytes / (kernel_ms * 1e-3) / 1e9
    return {"bandwidth_gbs": bw, "bandwidth_source": src, "intensity_flop_per_byte": round(intensity, 2),
            "bw_x_intensity_tflops": round(bw * intensity / 1e3, 1),
            "roofline_tflops": round(min(peak_tflops, bw * intensity / 1e3), 4),
            "achieved_gbs": round(achieved, 1), "frac_of_bandwidth": round(achieved / bw, 4)}


def read_traffic():
    """DRAM bytes per launch of the wave kernel from the committed ncu summary, if present."""
    try:
        for ln in TRAFFIC_FILE.read_text().splitlines():
            if ln.startswith("traffic_bytes_per_launch:"):
                return float(ln.split(":", 1)[1].strip())
    except Exception:
        pass
    return None


def run_ours(args):
    import torch
    import torch.distributed as dist
    import __graft_entry__ as ge

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pkg = ge.load_package()
    lib = pkg.load_library()
    h = pkg.Handle(local)
    stream = torch.cuda.Stream(dev)
    h.set_stream(stream.cuda_stream)
    h.set_kernel_timing(True)
    form = 1 if (args.form == "scaled" and args.dtype == "f64") else 0
    h.set_apply_form(form)

    m, n, k = args.m, args.n, args.k
    import ctypes
    fn = getattr(lib, f"symeig_apply_givens_{args.dtype}_dev")
    Q, cs = make_inputs(m, n, k, args.dtype, seed=1234 + rank, device=dev)
    ld = Q.stride(1)

    def step():
        rc = fn(h.ptr, ctypes.c_void_p(Q.data_ptr()), ld, m, n, ctypes.c_void_p(cs.data_ptr()), k)
        if rc != 0:
            raise RuntimeError(f"symeig_apply_givens_{args.dtype}_dev -> {rc}")

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    kernel_ms, launches = [], 0
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step()
            st = h.stats()   # waits for the step's last wave kernel; per-kernel device time
            kernel_ms.append(st["wave_kernel_ms"] / max(st["wave_launches"], 1))
            # per pass: table build + wave kernel (the scaled form adds the scale recurrence)
            launches += (3 if form else 2) * st["wave_launches"]
        e1.record(stream)
        torch.cuda.synchronize()
    clocks = clk.summary()
    ms = replica_reduce(e0.elapsed_time(e1), world, dev)
    if world > 1:
        dist.barrier()
    ms_per_step = ms / args.steps
    fl = flops_per_step(m, n, k)
    value = replica_value(fl, world, ms_per_step) / 1e9

    # roofline of the dominant kernel: the FP64 (FP32) FMA pipe.  The canonical FP64 form
    # computes its products on the integer pipes from 3072 rows on (csrc/apply.cu)
    peak = pkg._lib.measure_fma_peak(local, fp64=(args.dtype == "f64"))
    int_mul = args.dtype == "f64" and form == 0 and m >= 3072
    pipe_ops = 2 if (form == 1 or int_mul) else 4
    per_launch_ms = statistics.median(kernel_ms)
    passes = max(1, -(-k // 64))
    achieved = fl / passes / (per_launch_ms * 1e-3) / 1e12
    algo_bytes = (2.0 * m * n + 2.0 * (n - 1) * k) * (8 if args.dtype == "f64" else 4)

    # e2e through the host-pointer C ABI entry point, pinned buffers, copies in the timed region
    hq = torch.empty((n, m), dtype=Q.dtype, pin_memory=True)
    hq.copy_(Q.T)
    hcs = torch.empty_like(cs, device="cpu").pin_memory()
    hcs.copy_(cs)
    hfn = getattr(lib, f"symeig_apply_givens_{args.dtype}")
    h2 = pkg.Handle(local)
    h2.set_apply_form(form)

    def e2e_step():
        rc = hfn(h2.ptr, ctypes.c_void_p(hq.data_ptr()), m, m, n, ctypes.c_void_p(hcs.data_ptr()), k)
        if rc != 0:
            raise RuntimeError(f"symeig_apply_givens_{args.dtype} -> {rc}")
    e2e_step()
    if world > 1:
        dist.barrier()
    # each call is synchronous (the copies back are complete when it returns), so each step is
    # timed on its own; the median of 5 is the value, because a call now and then stalls for
    # tens of ms on the host side (measured: 105-109 ms against 72.6 ms, in builds with and
    # without any change to the path), and the mean is reported beside it
    e2e_steps = max(5, min(args.steps, 9))
    times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        e2e_step()
        times.append(time.perf_counter() - t0)
    med = sorted(times)[len(times) // 2]
    e2e_s = replica_reduce(med * 1e3, world, dev) * 1e-3
    mean_s = replica_reduce(sum(times) / len(times) * 1e3, world, dev) * 1e-3
    esz = 8 if args.dtype == "f64" else 4
    e2e = {"value": round(fl * world / e2e_s / 1e9, 3), "unit": "GFLOP/s",
           "h2d_bytes_per_step": int(m * n * esz + (n - 1) * k * 2 * esz),
           "d2h_bytes_per_step": int(m * n * esz), "ms_per_step": round(e2e_s * 1e3, 3),
           "statistic": f"median of {e2e_steps} steps, each timed alone",
           "mean_ms_per_step": round(mean_s * 1e3, 3), "mean_value": round(fl * world / mean_s / 1e9, 3),
           "entry_point": f"symeig_apply_givens_{args.dtype} (host pointers, pinned)"}
    del hq, hcs
    h2.close()

    extras = {}
    if rank == 0 and not args.no_extras:
        extras = side_measurements(pkg, lib, h, dev, stream, args)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_apply(m, n, k, args.dtype, os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_per_step, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.dtype,
            "data": "synthetic (seeded U[-1,1) Q, (cos t, sin t) rotations, t ~ U[0, 2pi))",
            "config": {"workload": WORKLOAD, "m": m, "n": n, "k": k,
                       "form": "scaled" if form else "canonical",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (Q = %.2f GB)" % (m * n * esz / 1e9)},
            "roofline": {"bound": "fp64" if args.dtype == "f64" else "fp32", "achieved": round(achieved, 4),
                         "peak": round(peak, 4), "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
                         "frac_of_givens_ceiling": round(achieved / peak / (6.0 / (2.0 * pipe_ops)), 4),
                         "peak_source": "measured now by symeig_measure_fma_peak (FMA = 2 flops). " + (
                             "A rotation-row is 6 counted flops: its two products run on the integer pipes "
                             "(exact IEEE products, int_mul.cuh) and its two FMAs on the FP64 pipe, so the "
                             "FP64-pipe ceiling is 6 / (2 x 2) = 1.5 of the FMA peak; fp64_pipe_frac is the "
                             "pipe's use" if int_mul else
                             "The scaled form spends 2 FMAs per rotation-row, so its ceiling is 1.5 and "
                             "fp64_pipe_frac is the measure of pipe use" if form == 1 else
                             "A Givens rotation-row is 4 FMA-pipe ops for 6 counted flops, so 0.75 is the ceiling"),
                         "hbm": hbm_side(algo_bytes, fl / passes, per_launch_ms, peak),
                         "fp64_instr_per_rotation_row": pipe_ops,
                         "products_on_integer_pipes": int_mul,
                         "fp64_pipe_frac": round(pipe_ops * (fl / 6.0 / passes) / (per_launch_ms * 1e-3)
                                                 / (peak * 1e12 / 2.0), 4),
                         "traffic": read_traffic(), "algorithmic_bytes": algo_bytes,
                         "kernel_ms": round(per_launch_ms, 3)},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        dist.destroy_process_group()


def side_measurements(pkg, lib, h, dev, stream, args):
    """FP32 apply on the same workload and the n=2000 solve (README example) for context."""
    import ctypes
    import torch
    out = {}
    m, n, k = args.m, args.n, args.k
    if args.dtype == "f64":
        Q, cs = make_inputs(m, n, k, "f32", seed=99, device=dev)
        fn = lib.symeig_apply_givens_f32_dev
        for _ in range(3):
            fn(h.ptr, ctypes.c_void_p(Q.data_ptr()), Q.stride(1), m, n, ctypes.c_void_p(cs.data_ptr()), k)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(5):
            fn(h.ptr, ctypes.c_void_p(Q.data_ptr()), Q.stride(1), m, n, ctypes.c_void_p(cs.data_ptr()), k)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 5
        peak32 = pkg._lib.measure_fma_peak(dev.index, fp64=False)
        gf = flops_per_step(m, n, k) / (ms * 1e-3) / 1e9
        out["f32_apply"] = {"value": round(gf, 1), "unit": "GFLOP/s", "ms_per_step": round(ms, 3),
                            "frac_of_fp32_peak": round(gf / 1e3 / peak32, 4), "fp32_peak_tflops": round(peak32, 2)}
        del Q, cs
    # the scaled (fast-Givens) form of the FP64 apply on the same workload
    if args.dtype == "f64" and args.form != "scaled":
        Q, cs = make_inputs(m, n, k, "f64", seed=77, device=dev)
        fn = lib.symeig_apply_givens_f64_dev
        h.set_apply_form(1)
        step = lambda: fn(h.ptr, ctypes.c_void_p(Q.data_ptr()), Q.stride(1), m, n, ctypes.c_void_p(cs.data_ptr()), k)
        for _ in range(3):
            step()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(5):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        st = h.stats()
        h.set_apply_form(0)
        ms = e0.elapsed_time(e1) / 5
        gf = flops_per_step(m, n, k) / (ms * 1e-3) / 1e9
        peak64 = pkg._lib.measure_fma_peak(dev.index, fp64=True)
        out["scaled_form"] = {"value": round(gf, 1), "unit": "GFLOP/s", "ms_per_step": round(ms, 3),
                              "kernel_ms": round(st["wave_kernel_ms"] / max(st["wave_launches"], 1), 3),
                              "frac_of_fp64_peak": round(gf / 1e3 / peak64, 4),
                              "note": "two FMAs per rotation-row with per-column scales (symeig_set_apply_form 1); "
                                      "a few ulps from the canonical form, not bit-equal to it"}
        del Q, cs
    # qr_algorithm! at n = 2000, d = 1:n, e ~ U[0,1) seed 0 (README.md:65-77)
    nn = 2000
    rng = np.random.default_rng(0)
    d, e = np.arange(1, nn + 1, dtype=np.float64), rng.random(nn - 1)
    H = pkg.SymTridiagonal(d.copy(), e.copy())
    Qh = np.asfortranarray(np.eye(nn))
    h.set_stream(None)
    t0 = time.perf_counter()
    _, conv, it = pkg.qr_algorithm_(H, Qh, handle=h)
    dt = time.perf_counter() - t0
    st = h.stats()
    h.set_stream(stream.cuda_stream)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    resid = float(np.linalg.norm(T @ Qh - Qh * H.dv) / np.linalg.norm(T))
    orth = float(np.linalg.norm(Qh.T @ Qh - np.eye(nn)))
    out["solve_n2000"] = {"seconds": round(dt, 3), "converged": conv, "iter": it,
                          "chase_ms": round(st["chase_ms"], 1), "apply_ms": round(st["apply_ms"], 1),
                          "rotations": st["rotations"], "resid_rel": resid, "orth": orth}
    # the same solve with the multishift chase (chase mode 3: the reference's error bounds,
    # another sweep sequence)
    H = pkg.SymTridiagonal(d.copy(), e.copy())
    Qh = np.asfortranarray(np.eye(nn))
    h.set_stream(None)
    t0 = time.perf_counter()
    _, conv, it = pkg.qr_algorithm_(H, Qh, handle=h, chase_mode=3)
    dt = time.perf_counter() - t0
    st = h.stats()
    h.set_stream(stream.cuda_stream)
    resid = float(np.linalg.norm(T @ Qh - Qh * H.dv) / np.linalg.norm(T))
    orth = float(np.linalg.norm(Qh.T @ Qh - np.eye(nn)))
    out["solve_n2000_multishift"] = {"seconds": round(dt, 3), "converged": conv, "iter": it,
                                     "chase_ms": round(st["chase_ms"], 1), "apply_ms": round(st["apply_ms"], 1),
                                     "rotations": st["rotations"], "bulge_batches": st["bulge_batches"],
                                     "resid_rel": resid, "orth": orth, "bound_10n_eps": 10 * nn * 2.220446049250313e-16}
    if args.no_solve_extras:
        return out
    # the full eigensolve at n = 16384 (case A) with the multishift chase, beside the
    # reference's own solve path timed on the host cores
    torch.cuda.synchronize()
    out["solve_n16384"] = measure_solve(pkg, 16384, "A", "f64", 3, "canonical", with_clocks=False)
    if not args.no_cpu_baseline:
        out["cpu_reference_solve_n16384"] = cpu_reference_solve(16384, "A", os.cpu_count() or 1)
        out["solve_n16384"]["speedup_vs_cpu_reference"] = round(
            out["cpu_reference_solve_n16384"]["value"] / out["solve_n16384"]["seconds"], 2)
    out["batched"] = measure_batched(pkg, with_cpu=not args.no_cpu_baseline)
    out["adjoint"] = measure_adjoint(pkg, with_cpu=not args.no_cpu_baseline)
    return out


def solve_inputs(n, case):
    if case == "A":
        rng = np.random.default_rng(1)
        return np.arange(1, n + 1, dtype=np.float64), rng.random(n - 1)
    rng = np.random.default_rng(2)
    return rng.standard_normal(n), 0.5 * rng.standard_normal(n - 1)


def _tq_errors(torch, d, e, lam, Q):
    """||TQ - Q diag(lam)||_F / ||T||_F and ||Q^T Q - I||_F in FP64 on the GPU (d, e: device
    FP64 vectors; Q: device matrix, any float dtype)."""
    Q = Q.to(torch.float64)
    TQ = d[:, None] * Q
    TQ[:-1] += e[:, None] * Q[1:]
    TQ[1:] += e[:, None] * Q[:-1]
    normT = math.sqrt(float((d * d).sum() + 2 * (e * e).sum()))
    resid = float(torch.linalg.norm(TQ - Q * lam[None, :])) / normT
    del TQ
    G = Q.T @ Q
    G.diagonal().sub_(1.0)
    return resid, float(torch.linalg.norm(G))


def measure_solve(pkg, n, case, q="f64", chase_mode=3, form="canonical", ms=(64, 16, 4), with_clocks=True):
    """One full qr_algorithm!(SymTridiagonal(d, e), Q = I) on the device, with its errors:
    eigenvalues against LAPACK (scipy stemr, host), ||TQ - QD||_F / ||T||_F and ||Q^T Q - I||_F
    on the GPU in FP64."""
    import torch
    from scipy.linalg import eigh_tridiagonal
    d, e = solve_inputs(n, case)
    dev = torch.device("cuda", 0)
    qdt = torch.float64 if q == "f64" else torch.float32
    h = pkg.Handle(0)
    h.set_multishift(*ms)
    td, te = torch.from_numpy(d.copy()).to(dev), torch.from_numpy(e.copy()).to(dev)
    Q = torch.eye(n, dtype=qdt, device=dev).T
    torch.cuda.synchronize()
    clk = ClockSampler(0) if with_clocks else None
    if clk:
        clk.__enter__()
    t0 = time.perf_counter()
    _, conv, it = pkg.qr_algorithm_(pkg.SymTridiagonal(td, te), Q, handle=h, chase_mode=chase_mode,
                                    apply_form=1 if (form == "scaled" and q == "f64") else 0)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    if clk:
        clk.__exit__(None, None, None)
    st = h.stats()
    h.close()
    lam = td.cpu().numpy()
    resid, orth = _tq_errors(torch, torch.from_numpy(d).to(dev), torch.from_numpy(e).to(dev), td, Q)
    del Q
    t_lapack = time.perf_counter()
    ref = eigh_tridiagonal(d, e, eigvals_only=True)
    t_lapack = time.perf_counter() - t_lapack
    normT = float(np.max(np.abs(ref)))
    eig_err = float(np.max(np.abs(np.sort(lam) - ref)))
    eps = float(np.finfo(np.float64).eps)
    out = {"seconds": round(secs, 3), "n": n, "case": case, "q": q, "chase_mode": chase_mode, "form": form,
           "converged": bool(conv), "iterations": it, "rotations": st["rotations"], "flushes": st["flushes"],
           "chase_ms": round(st["chase_ms"], 1), "apply_ms": round(st["apply_ms"], 1),
           "givens_gflops_apply": round(6.0 * n * st["rotations"] / max(st["apply_ms"] * 1e-3, 1e-9) / 1e9, 1),
           "applied_rotation_rows": st["applied_rotation_rows"], "bulge_batches": st["bulge_batches"],
           "early_flushes": st["early_flushes"], "redone_sweeps": st["redone_sweeps"],
           "errors": {"eig_max_abs_vs_lapack": eig_err, "eig_bound_10n_eps_normT": 10 * n * eps * normT,
                      "resid_rel": resid, "orth": orth, "bound_10n_eps": 10 * n * eps,
                      "eig_over_bound": eig_err / (10 * n * eps * normT), "resid_over_bound": resid / (10 * n * eps),
                      "orth_over_bound": orth / (10 * n * eps)},
           "lapack_eigvals": {"seconds": round(t_lapack, 3), "cores": os.cpu_count(),
                              "kind": "scipy eigh_tridiagonal, eigenvalues only (no vectors), host"}}
    if q == "f32":
        # the FP32-Q variant's Q is held to the FP32 bound 10 n eps32 (its eigenvalues come from
        # the FP64 chase and keep the FP64 bound)
        eps32 = float(np.finfo(np.float32).eps)
        out["errors"].update({"bound_10n_eps32": 10 * n * eps32, "resid_over_bound_eps32": resid / (10 * n * eps32),
                              "orth_over_bound_eps32": orth / (10 * n * eps32)})
    if clk:
        out["clocks"] = clk.summary()
    return out


def cpu_reference_solve(n, case, threads, apply_every=4):
    """The reference's solve path timed on the host (oracle.qr_reference_path, timing build):
    its chase on one core and its grid placement; after every flush, the whole (n-1) x 128 grid
    applied to all n rows of Q by the row-slab threaded wave kernel on `threads` threads
    (src/bulge_chasing.jl:146-288 -> src/wave.jl:36-60).  To bound the run, only every
    apply_every-th flush is applied (the chase never reads Q, and the kernel's cost follows the
    grid's rotations), and the apply time scales by rotations of all flushes / rotations of the
    applied ones.  Even n only, as the reference."""
    from oracle import oracle as orc
    d, e = solve_inputs(n, case)
    Q = np.asfortranarray(np.eye(n))
    t0 = time.perf_counter()
    conv, it, fl, tc, ta, ra, rt = orc.qr_reference_path(d, e, Q, max_layers=128, nthreads=threads, fast=True,
                                                         apply_every=apply_every)
    wall = time.perf_counter() - t0
    scale = rt / max(ra, 1)
    return {"value": round(tc + ta * scale, 2), "unit": "s", "cores": threads, "kind": "port",
            "chase_s_1_core": round(tc, 3), "apply_s_sampled_flushes": round(ta, 3),
            "apply_s_scaled": round(ta * scale, 2), "converged": conv, "iterations": it, "flushes": fl,
            "rotations": rt, "rotations_of_applied_flushes": ra, "wall_s": round(wall, 2),
            "sample": (f"the reference's solve path (oracle/symeig_oracle.c oracle_qr_reference_path, timing "
                       f"build): chase on 1 core; every {apply_every}th flush's whole grid applied to all {n} "
                       f"rows of Q by the row-slab wave kernel on {threads} threads; apply time scaled by "
                       f"rotations, x{scale:.2f}")}


def run_solve(args):
    """One full qr_algorithm! on the device (the full-eigensolve workload: n = 16384, case A or
    B, FP64 or FP32 Q), with its errors stated; --oracle-check adds the CPU oracle's chase
    (bit-equal eigenvalues in chase modes 0-2) and the timed CPU baseline of the reference's
    solve path."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    torch.cuda.set_device(0)
    n = args.n
    if args.chase_mode is None:
        args.chase_mode = 0
    r = measure_solve(pkg, n, args.case, args.q, args.chase_mode, args.form,
                      (args.ms_bulges, args.ms_rows, args.ms_release))
    out = {
        "metric": f"qr_algorithm! full solve seconds, n={n} case {args.case}, Q {args.q}",
        "value": r["seconds"], "unit": "s", "higher_is_better": False, "n_gpus": 1,
        "dtype": "f64" if args.q == "f64" else "f64 chase, f32 Q",
        "data": "synthetic (seeded, as in the full-eigensolve configuration)",
        "config": {"workload": "qr_algorithm!(SymTridiagonal(d, e), Q = I)", "n": n, "case": args.case,
                   "q": args.q, "max_layers": 128, "chase_mode": args.chase_mode, "form": args.form,
                   **({"ms_bulges": args.ms_bulges, "ms_rows": args.ms_rows, "ms_release": args.ms_release}
                      if args.chase_mode == 3 else {})},
        **{k: v for k, v in r.items() if k not in ("seconds",)},
    }
    if args.oracle_check:
        from oracle import oracle as orc
        d, e = solve_inputs(n, args.case)
        od, oe = d.copy(), e.copy()
        t0 = time.perf_counter()
        c_o, it_o, fl_o, rot_o = orc.qr_algorithm(od, oe, None)
        chase_s = time.perf_counter() - t0
        out["oracle_chase"] = {"seconds_1_core": round(chase_s, 2), "iterations": it_o, "rotations": rot_o}
        if n % 2 == 0 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_reference_solve(n, args.case, os.cpu_count() or 1, apply_every=1)
    print(json.dumps(out), flush=True)


def measure_batched(pkg, count=4096, loop_sample=8, check=256, cpu_sample=64, with_cpu=True):
    """Batched eigensolves (qr_algorithm_batched_, one call): `count` tridiagonals with
    n ~ U{32..1024}, d ~ N(0,1), e ~ U[0.1,1) (seed 3), FP64 Q (and, as `q32`, the same batch
    with FP32 Q), against (a) one
    qr_algorithm! call per matrix on the same GPU, timed on a sample of the batch's own
    matrices in the reference's sweep sequence (chase mode 0) and with the multishift chase
    (mode 3), extrapolated by sum n^2 (the apply's work per sweep is n^2 per matrix; the loop
    over all 4096 would take about half an hour); (b) the host: the oracle's solves (timing
    build) of a sample on all cores, extrapolated by sum n^3.  Errors: eigenvalues of `check`
    matrices against LAPACK, residual and orthogonality of a few."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    from scipy.linalg import eigh_tridiagonal
    dev = torch.device("cuda", 0)
    h = pkg.Handle(0)
    rng = np.random.default_rng(3)
    sizes = rng.integers(32, 1025, size=count)
    t_tune = time.perf_counter()
    tuning = pkg.batched_autotune(sizes=sizes, handle=h)   # timed on the batch's own orders
    t_tune = time.perf_counter() - t_tune
    d = rng.standard_normal(int(sizes.sum()))
    e = rng.random(int((sizes - 1).sum())) * 0.9 + 0.1
    doff = np.concatenate([[0], np.cumsum(sizes)])
    eoff = np.concatenate([[0], np.cumsum(sizes - 1)])
    qoff = np.concatenate([[0], np.cumsum(sizes * sizes)])
    td, te = torch.from_numpy(d.copy()).to(dev), torch.from_numpy(e.copy()).to(dev)
    tQ = torch.zeros(int(qoff[-1]), dtype=torch.float64, device=dev)
    for j, n in enumerate(sizes):
        tQ[qoff[j]:qoff[j + 1]].view(n, n).fill_diagonal_(1.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    conv, iters = pkg.qr_algorithm_batched_(td, te, sizes, tQ, handle=h)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    st = h.stats()
    lam_all = td.cpu().numpy()
    eps = float(np.finfo(np.float64).eps)
    eig_ratio = resid_max = orth_max = 0.0
    chk = rng.choice(count, min(check, count), replace=False)
    for j in chk:
        n = int(sizes[j])
        dj, ej = d[doff[j]:doff[j + 1]], e[eoff[j]:eoff[j + 1]]
        ref = eigh_tridiagonal(dj, ej, eigvals_only=True)
        err = float(np.max(np.abs(np.sort(lam_all[doff[j]:doff[j + 1]]) - ref)))
        eig_ratio = max(eig_ratio, err / (10 * n * eps * float(np.max(np.abs(ref)))))
    for j in chk[:16]:
        n = int(sizes[j])
        Qj = tQ[qoff[j]:qoff[j + 1]].view(n, n).T
        r, o = _tq_errors(torch, torch.from_numpy(d[doff[j]:doff[j + 1]]).to(dev),
                          torch.from_numpy(e[eoff[j]:eoff[j + 1]]).to(dev), td[doff[j]:doff[j + 1]], Qj)
        resid_max, orth_max = max(resid_max, r / (10 * n * eps)), max(orth_max, o / (10 * n * eps))
    del tQ
    # the same batch with FP32 Q (the FP32-Q variant: FP64 chase, (c,s) rounded to float)
    td32, te32 = torch.from_numpy(d.copy()).to(dev), torch.from_numpy(e.copy()).to(dev)
    tQ32 = torch.zeros(int(qoff[-1]), dtype=torch.float32, device=dev)
    for j, n in enumerate(sizes):
        tQ32[qoff[j]:qoff[j + 1]].view(n, n).fill_diagonal_(1.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    conv32, _ = pkg.qr_algorithm_batched_(td32, te32, sizes, tQ32, handle=h)
    torch.cuda.synchronize()
    secs32 = time.perf_counter() - t0
    eps32 = float(np.finfo(np.float32).eps)
    r32 = o32 = 0.0
    for j in chk[:16]:
        n = int(sizes[j])
        Qj = tQ32[qoff[j]:qoff[j + 1]].view(n, n).T
        r, o = _tq_errors(torch, torch.from_numpy(d[doff[j]:doff[j + 1]]).to(dev),
                          torch.from_numpy(e[eoff[j]:eoff[j + 1]]).to(dev), td32[doff[j]:doff[j + 1]], Qj)
        r32, o32 = max(r32, r / (10 * n * eps32)), max(o32, o / (10 * n * eps32))
    q32 = {"value": round(count / secs32, 2), "unit": "solves/s", "seconds": round(secs32, 3),
           "all_converged": bool(conv32.all()),
           "same_eigenvalues_as_f64": bool(torch.equal(td32, torch.from_numpy(lam_all).to(dev))),
           "resid_over_10n_eps32_max": r32, "orth_over_10n_eps32_max": o32, "vectors_checked": 16}
    del tQ32, td32, te32
    # (a) one call per matrix, on the batch's own matrices
    sample = rng.choice(count, min(loop_sample, count), replace=False)
    w_all = float((sizes.astype(np.float64) ** 2).sum())
    loop = {}
    for mode in (0, 3):
        loop_s, work = 0.0, 0.0
        for j in sample:
            n = int(sizes[j])
            dd = torch.from_numpy(d[doff[j]:doff[j + 1]].copy()).to(dev)
            ee = torch.from_numpy(e[eoff[j]:eoff[j + 1]].copy()).to(dev)
            Q = torch.eye(n, dtype=torch.float64, device=dev).T
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pkg.qr_algorithm_(pkg.SymTridiagonal(dd, ee), Q, handle=h, chase_mode=mode)
            torch.cuda.synchronize()
            loop_s += time.perf_counter() - t0
            work += n * n
        est = loop_s * w_all / work
        loop[f"mode{mode}"] = {"solves_per_s": round(count / est, 3), "sample": int(len(sample)),
                               "sample_seconds": round(loop_s, 2), "extrapolated_seconds": round(est, 1)}
    h.close()
    best_loop = min(loop["mode0"]["extrapolated_seconds"], loop["mode3"]["extrapolated_seconds"])
    out = {"value": round(count / secs, 2), "unit": "solves/s", "count": count, "seconds": round(secs, 3),
           "all_converged": bool(conv.all()), "iterations": int(iters.sum()), "rounds": st["flushes"],
           "tuning": tuning[0], "autotune_ms": tuning[1], "autotune_seconds": round(t_tune, 2), "q32": q32, "loop": loop,
           "speedup_vs_loop_mode0": round(loop["mode0"]["extrapolated_seconds"] / secs, 1),
           "speedup_vs_best_loop": round(best_loop / secs, 1),
           "errors": {"eig_err_over_10n_eps_normT_max": eig_ratio, "eig_checked": int(len(chk)),
                      "resid_over_10n_eps_max": resid_max, "orth_over_10n_eps_max": orth_max,
                      "vectors_checked": 16}}
    if with_cpu:
        from oracle import oracle as orc
        threads = os.cpu_count() or 1
        cs = rng.choice(count, min(cpu_sample, count), replace=False)

        def one(j):
            n = int(sizes[j])
            Qj = np.asfortranarray(np.eye(n))
            orc.qr_algorithm(d[doff[j]:doff[j + 1]].copy(), e[eoff[j]:eoff[j + 1]].copy(), Qj, fast=True)

        t0 = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(one, cs))
        cpu_s = time.perf_counter() - t0
        w3 = float((sizes.astype(np.float64) ** 3).sum())
        est = cpu_s * w3 / float((sizes[cs].astype(np.float64) ** 3).sum())
        out["cpu_baseline"] = {"value": round(count / est, 3), "unit": "solves/s", "cores": threads, "kind": "port",
                               "sample": (f"{len(cs)} of the matrices solved by the oracle (timing build, "
                                          f"chase + layer-major apply per flush) on {threads} threads, "
                                          f"{cpu_s:.1f} s, extrapolated by sum n^3")}
        out["speedup_vs_cpu"] = round(est / secs, 1)
    return out


def run_batched(args):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    torch.cuda.set_device(0)
    with ClockSampler(0) as clk:
        r = measure_batched(pkg, args.count, args.loop_sample, with_cpu=not args.no_cpu_baseline)
    out = {"metric": f"batched eigensolves per second, {args.count} tridiagonals n~U{{32..1024}}",
           "higher_is_better": True, "n_gpus": 1, "dtype": "f64",
           "data": "synthetic (seed 3: n ~ U{32..1024}, d ~ N(0,1), e ~ U[0.1,1))",
           "config": {"workload": "qr_algorithm_batched_ (persistent work queue, CUDA-graph rounds)",
                      "count": args.count, "max_layers": 128}, **r, "clocks": clk.summary()}
    print(json.dumps(out), flush=True)


def measure_adjoint(pkg, n=4096, K=64, chase_mode=3, batched=True, with_cpu=True):
    """Adjoint of the eigensolve (TridiagEigh: forward qr_algorithm!, backward
    symeig_eig_adjoint_f64_dev): n = 4096, d ~ N(0,1), e ~ U[0.1,1) (seed 4), loss
    L = sum_i w_i lam_(i) + sum_{i<=64} q_(i)^T B q_(i), w ~ N(0,1), B symmetric ~ N(0,1/n),
    eigenpairs sorted ascending.  (forward + backward) / forward time, the gradient against an
    FP64 reference (LAPACK eigenpairs and the closed-form pullback in numpy), the adjoint GEMMs
    against the measured FP64 MMA peak; optionally the batched variant (256 x n = 512) and the
    host's forward + backward (the reference's solve path, then the pullback by numpy BLAS)."""
    import torch
    from scipy.linalg import eigh_tridiagonal
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(4)
    d = rng.standard_normal(n)
    e = rng.random(n - 1) * 0.9 + 0.1
    w = rng.standard_normal(n)
    Bm = rng.standard_normal((n, n)) / np.sqrt(n)
    Bm = (Bm + Bm.T) / 2
    tw, tB = torch.tensor(w, device=dev), torch.tensor(Bm, device=dev)

    def loss(lam, Q):
        order = torch.argsort(lam)
        QK = Q[:, order][:, :K]
        return (tw * lam[order]).sum() + (QK * (tB @ QK)).sum()

    # one untimed pass of the whole path at n = 256 (library and kernel loading)
    wd = torch.tensor(d[:256], device=dev, requires_grad=True)
    we = torch.tensor(e[:255], device=dev, requires_grad=True)
    wl, wQ = pkg.TridiagEigh.apply(wd, we, chase_mode)
    wo = torch.argsort(wl)
    wK = wQ[:, wo][:, :K]
    ((tw[:256] * wl[wo]).sum() + (wK * (tB[:256, :256] @ wK)).sum()).backward()
    torch.cuda.synchronize()
    td = torch.tensor(d, device=dev, requires_grad=True)
    te = torch.tensor(e, device=dev, requires_grad=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lam, Q = pkg.TridiagEigh.apply(td, te, chase_mode)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    L = loss(lam, Q)
    torch.cuda.synchronize()
    tl = time.perf_counter()
    L.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    fwd, loss_s, bwd = t1 - t0, tl - t1, t2 - tl
    # FP64 reference gradient
    tr0 = time.perf_counter()
    lam_r, V = eigh_tridiagonal(d, e)
    gV = np.zeros((n, n))
    gV[:, :K] = 2 * Bm @ V[:, :K]
    F = lam_r[None, :] - lam_r[:, None]
    np.fill_diagonal(F, 1.0)
    F = 1.0 / F
    np.fill_diagonal(F, 0.0)
    A = V @ (np.diag(w) + F * (V.T @ gV)) @ V.T
    g_ref = np.concatenate([np.diag(A), np.diag(A, 1) + np.diag(A, -1)])
    ref_s = time.perf_counter() - tr0
    g = np.concatenate([td.grad.cpu().numpy(), te.grad.cpu().numpy()])
    rel = float(np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref))
    # the adjoint kernels alone (two FP64 tensor-core GEMMs with fused epilogues)
    glam = torch.randn(n, device=dev, dtype=torch.float64)
    gQ = torch.randn(n, n, device=dev, dtype=torch.float64)
    lam_d, Q_d = lam.detach(), Q.detach()
    pkg.eig_adjoint(lam_d, Q_d, glam, gQ)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    pkg.eig_adjoint(lam_d, Q_d, glam, gQ)
    e1.record()
    torch.cuda.synchronize()
    adj_ms = e0.elapsed_time(e1)
    dmma_peak = pkg._lib.measure_dmma_peak(0)
    del gQ, Q, Q_d
    out = {"value": round((fwd + loss_s + bwd) / fwd, 4), "unit": "ratio", "n": n, "K": K,
           "forward_chase_mode": chase_mode,
           "forward_s": round(fwd, 3), "loss_s": round(loss_s, 3), "backward_s": round(bwd, 3),
           "grad_rel_err_vs_fp64_reference": rel, "fp64_reference_host_s": round(ref_s, 2),
           "adjoint_kernels_ms": round(adj_ms, 2),
           "roofline": {"bound": "fp64 tensor (mma.sync .f64)", "achieved": round(4.0 * n ** 3 / (adj_ms * 1e-3) / 1e12, 3),
                        "peak": round(dmma_peak, 3), "unit": "TFLOP/s",
                        "frac": round(4.0 * n ** 3 / (adj_ms * 1e-3) / 1e12 / dmma_peak, 4),
                        "peak_source": "measured now by symeig_measure_dmma_peak"}}
    if batched:
        B, nb = 256, 512
        db = torch.tensor(rng.standard_normal((B, nb)), device=dev, requires_grad=True)
        eb = torch.tensor(rng.random((B, nb - 1)) * 0.9 + 0.1, device=dev, requires_grad=True)
        wb = torch.tensor(rng.standard_normal((B, nb)), device=dev)
        Bb = torch.tensor(rng.standard_normal((nb, nb)) / np.sqrt(nb), device=dev)
        Bb = (Bb + Bb.T) / 2
        w4d, w4e = db[:4].detach().clone().requires_grad_(True), eb[:4].detach().clone().requires_grad_(True)
        l4, Q4 = pkg.TridiagEighBatched.apply(w4d, w4e)
        o4 = torch.argsort(l4, dim=1)
        K4 = torch.gather(Q4, 2, o4[:, None, :8].expand(4, nb, 8))
        ((wb[:4] * torch.gather(l4, 1, o4)).sum() + (K4 * (Bb @ K4)).sum()).backward()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lamb, Qb = pkg.TridiagEighBatched.apply(db, eb)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ob = torch.argsort(lamb, dim=1)
        QKb = torch.gather(Qb, 2, ob[:, None, :8].expand(B, nb, 8))
        Lb = (wb * torch.gather(lamb, 1, ob)).sum() + (QKb * (Bb @ QKb)).sum()
        Lb.backward()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        out["batched"] = {"B": B, "n": nb, "forward_s": round(t1 - t0, 3), "backward_s": round(t2 - t1, 3),
                          "ratio": round((t2 - t0) / (t1 - t0), 4)}
    if with_cpu and n % 2 == 0:
        # the host's forward (the reference's solve path) and backward (numpy BLAS pullback)
        from oracle import oracle as orc
        threads = os.cpu_count() or 1
        dd, ee = d.copy(), e.copy()
        Qh = np.asfortranarray(np.eye(n))
        t0 = time.perf_counter()
        orc.qr_reference_path(dd, ee, Qh, nthreads=threads, fast=True)  # every flush applied
        t1 = time.perf_counter()
        order = np.argsort(dd)
        Vh = Qh[:, order]
        gVh = np.zeros((n, n))
        gVh[:, :K] = 2 * Bm @ Vh[:, :K]
        lh = dd[order]
        Fh = lh[None, :] - lh[:, None]
        np.fill_diagonal(Fh, 1.0)
        Fh = 1.0 / Fh
        np.fill_diagonal(Fh, 0.0)
        Ah = Vh @ (np.diag(w) + Fh * (Vh.T @ gVh)) @ Vh.T
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"value": round(t2 - t0, 3), "unit": "s (forward + backward)", "cores": threads,
                               "kind": "port", "forward_s": round(t1 - t0, 3), "backward_s": round(t2 - t1, 3),
                               "sample": ("the whole workload: the reference's solve path (oracle timing build, "
                                          f"{threads} threads) and the closed-form pullback in numpy BLAS")}
        out["speedup_vs_cpu"] = round((t2 - t0) / (fwd + loss_s + bwd), 1)
    return out


def run_adjoint(args):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    torch.cuda.set_device(0)
    n = args.n if args.n != 16384 else 4096
    with ClockSampler(0) as clk:
        r = measure_adjoint(pkg, n, 64, 3 if args.chase_mode is None else args.chase_mode,
                            with_cpu=not args.no_cpu_baseline)
    out = {"metric": f"adjoint (forward + backward) / forward time, n={n}", "higher_is_better": False,
           "n_gpus": 1, "dtype": "f64",
           "data": "synthetic (seed 4: d ~ N(0,1), e ~ U[0.1,1), w ~ N(0,1), B ~ N(0,1/n) symmetric)",
           "config": {"workload": "TridiagEigh forward + backward, loss on the 64 lowest eigenpairs", "n": n, "K": 64},
           **r, "clocks": clk.summary()}
    print(json.dumps(out), flush=True)


def run_dense(args):
    """Dense symmetric eigensolve on the device (syev: sytrd -> orgtr -> qr_algorithm!), the
    step before the reference's path: A symmetric with N(0,1) entries (seed 5), n = --n
    (default 4096).  Reports each phase's time, the reduction's throughput ((4/3) n^3 flops
    for sytrd and as many for orgtr) and the errors; the CPU baseline is LAPACK dsytrd + dorgtr
    (scipy, all host cores) on the same matrix."""
    import torch
    import __graft_entry__ as ge
    from scipy.linalg import lapack
    pkg = ge.load_package()
    if args.chase_mode is None:
        args.chase_mode = 0
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    n = args.n if args.n != 16384 else 4096
    rng = np.random.default_rng(5)
    A = rng.standard_normal((n, n))
    A = np.asfortranarray((A + A.T) / 2)
    h = pkg.Handle(0)
    # warm-up at a small order
    w = np.asfortranarray(A[:96, :96])
    pkg.syev(torch.from_numpy(w.T.copy()).to(dev).T, handle=h)
    tA = torch.from_numpy(A.T.copy()).to(dev).T
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        d, e, tau = pkg.sytrd_(tA, handle=h)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        V = pkg.orgtr(tA, tau, handle=h)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        _, conv, it = pkg.qr_algorithm_(pkg.SymTridiagonal(d, e), V, handle=h, chase_mode=args.chase_mode,
                                        apply_form=1 if args.form == "scaled" else 0)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
    lam = d
    tA0 = torch.from_numpy(A.T.copy()).to(dev).T
    resid = float(torch.linalg.norm(tA0 @ V - V * lam[None, :]) / torch.linalg.norm(tA0))
    G = V.T @ V
    G.diagonal().sub_(1.0)
    orth = float(torch.linalg.norm(G))
    ref = np.linalg.eigvalsh(A)
    eig_err = float(np.max(np.abs(np.sort(lam.cpu().numpy()) - ref)))
    eps = float(np.finfo(np.float64).eps)
    flops = 4.0 / 3.0 * n ** 3
    out = {
        "metric": f"dense symmetric eigensolve seconds, n={n}",
        "value": round(t3 - t0, 3), "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": "f64",
        "data": "synthetic (seed 5: symmetric, N(0,1) entries)",
        "config": {"workload": "syev: sytrd -> orgtr -> qr_algorithm!", "n": n, "chase_mode": args.chase_mode,
                   "form": args.form},
        "sytrd_s": round(t1 - t0, 3), "orgtr_s": round(t2 - t1, 3), "qr_s": round(t3 - t2, 3),
        "sytrd_gflops": round(flops / (t1 - t0) / 1e9, 1), "orgtr_gflops": round(flops / (t2 - t1) / 1e9, 1),
        "dmma_peak_tflops": round(pkg._lib.measure_dmma_peak(0), 3),
        "converged": bool(conv), "iterations": it,
        "errors": {"eig_max_abs_vs_lapack": eig_err, "eig_bound_10n_eps_normA": 10 * n * eps * float(np.max(np.abs(ref))),
                   "resid_rel": resid, "orth": orth, "bound_10n_eps": 10 * n * eps},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        c, dl, el, taul, info = lapack.dsytrd(A, lower=1)
        t1 = time.perf_counter()
        ql, _, info2 = lapack.dorgqr(np.asfortranarray(c[1:, : n - 1]), taul)   # dorgtr (lower)
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"value": round(t2 - t0, 3), "unit": "s (sytrd + orgtr)", "cores": os.cpu_count(),
                               "kind": "LAPACK (scipy dsytrd + dorgtr)", "sytrd_s": round(t1 - t0, 3),
                               "orgtr_s": round(t2 - t1, 3),
                               "sample": f"the same n={n} matrix, scipy's LAPACK on all host cores"}
        # the whole dense eigensolve on the host: LAPACK dsyevd (eigenvalues and vectors)
        from scipy.linalg import eigh
        t0 = time.perf_counter()
        eigh(A, driver="evd", check_finite=False)
        out["cpu_eigh"] = {"value": round(time.perf_counter() - t0, 3), "unit": "s", "cores": os.cpu_count(),
                           "kind": "LAPACK dsyevd (scipy.linalg.eigh, driver evd)",
                           "sample": f"the same n={n} matrix, all host cores"}
    print(json.dumps(out), flush=True)
    h.close()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "solve":
        run_solve(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "dense":
        run_dense(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
