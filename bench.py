#!/usr/bin/env python3
"""Benchmark: DGEMM TFLOP/s at FP64 accuracy on one GB300 -- emulated FP64
(Ozaki 7-bit slices on the bf16 tensor cores) against native FP64.

A step is one DGEMM NN, M=N=K=8192, alpha=1, beta=0 on seeded uniform(-1,1)
operands resident in HBM (3 x 512 MiB, larger than the 129 MB L2, so no
flush is needed between steps).  `value` is the emulated-FP64 throughput;
the line also carries the native FP64 rate on the same operands, the error of
the emulated result against the native one, an end-to-end figure through
cblas_dgemm with pinned host buffers, the roofline of the dominant kernel
(the tcgen05 slice GEMM) and the CPU baseline (the oracle port on the host
cores).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With N > 1 (torchrun) every rank runs an independent replica (the path does
not shard across GPUs here) and the slowest rank's time is reported.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DGEMM & DGESV TFLOP/s at FP64 accuracy: emulated/mixed vs native FP64, 1 GB300"
UNIT = "TFLOP/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--slices", type=int, default=8)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the DGESV and batched legs (profiling runs)")
    return ap.parse_args()


def workload_config(n, slices):
    return {
        "workload": f"DGEMM NN M=N=K={n}, alpha=1, beta=0, A,B,C uniform(-1,1) seeded; "
                    f"FP64-accuracy emulation with {slices} 7-bit slices vs native FP64",
        "m": n, "n": n, "k": n, "transa": "N", "transb": "N", "slices": slices,
        "l2": "inputs larger than L2 (3 x 512 MiB), no flush",
        "parallelism": "replicas",
    }


# --------------------------------------------------------------------------
# distributed helpers (replicas; one process per GPU under torchrun)
# --------------------------------------------------------------------------
def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        mhz, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": mx,
                "samples": len(mhz), "reasons": sorted(reasons)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, \
            "fallback"


def profiled_traffic(n):
    """DRAM bytes per slice-GEMM launch from the committed ncu summary
    (dram__bytes_read.sum + dram__bytes_write.sum, one-pass capture).  A
    capture at exactly n is used as is; otherwise the nearest captured size
    is scaled by n^3 (every tile re-reads its K-panel of slices for each
    product) and the result says so."""
    path = os.path.join(ROOT, "profiles", "slice_gemm_ncu.txt")
    caps = {}
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch"):
                _, size, val = line.split()
                caps[int(size)] = float(val)
    except Exception:
        return None, None
    if not caps:
        return None, None
    if n in caps:
        return caps[n], f"ncu one-pass capture at n={n}"
    size = min(caps, key=lambda c: abs(c - n))
    return caps[size] * (n / size) ** 3, f"ncu capture at n={size} scaled by n^3"


# --------------------------------------------------------------------------
# reference arm: the oracle port of the reference CPU path on host cores
# --------------------------------------------------------------------------
def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from oracle import pyoracle as orc
    from openblas_gb300 import workloads as W
    n = args.n
    slab = 1024  # columns of C per step: a bounded sample of the n^3 product
    A = W.uniform(1, (n, n))
    B = W.uniform(2, (n, slab))
    Cm = np.zeros((n, slab), order="F")
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    for _ in range(args.warmup):
        orc.dgemm("N", "N", n, slab, n, 1.0, A, n, B, n, 0.0, Cm, n)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.dgemm("N", "N", n, slab, n, 1.0, A, n, B, n, 0.0, Cm, n)
    dt = (time.perf_counter() - t0) / args.steps
    val = 2.0 * n * n * slab / dt / 1e12
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, args.slices), "impl": "reference",
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"DGEMM NN {n}x{slab}x{n} column slab per step "
                                   f"(oracle C restatement of the reference's GEMM, OpenMP "
                                   f"{cores} threads)"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample():
    """Oracle DGEMM on the host cores over a bounded sample (rank 0, N=1)."""
    import numpy as np
    from oracle import pyoracle as orc
    from openblas_gb300 import workloads as W
    n = 2048
    A = W.uniform(1, (n, n))
    B = W.uniform(2, (n, n))
    Cm = np.zeros((n, n), order="F")
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    orc.dgemm("N", "N", n, n, n, 1.0, A, n, B, n, 0.0, Cm, n)
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.dgemm("N", "N", n, n, n, 1.0, A, n, B, n, 0.0, Cm, n)
    dt = (time.perf_counter() - t0) / reps
    return {"value": 2.0 * n ** 3 / dt / 1e12, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"DGEMM NN {n}^3, {reps} timed reps after 1 warm-up, oracle C restatement "
                      f"of the reference's GEMM with OpenMP over {cores} host threads"}


def dgesv_compare(lib, torch, gb, world, n=8192, nrhs=1, reps=3):
    g = torch.Generator(device="cuda")
    g.manual_seed(77)
    A = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand((nrhs, n), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    X = torch.zeros_like(B)
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    it, info = C.c_int(0), C.c_int(0)

    def mixed():
        st = lib.gb_dsgesv_dev(n, nrhs, A.data_ptr(), n, ipiv.data_ptr(), B.data_ptr(), n,
                               X.data_ptr(), n, C.byref(it), C.byref(info))
        if st != 0:
            raise RuntimeError(gb.last_error(lib))

    mixed()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        mixed()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t_mixed = allreduce_max(statistics.median(times), world)
    # backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf), FP64 on the GPU
    R = B.clone()
    lib.gb_dgemm_native_dev(b"N", b"N", n, nrhs, n, -1.0, A.data_ptr(), n, X.data_ptr(), n, 1.0,
                            R.data_ptr(), n)
    torch.cuda.synchronize()
    anorm = float(A.abs().sum(dim=0).max())  # rows of A are columns of the torch tensor
    berr = float(R.abs().max() / (anorm * X.abs().max() + B.abs().max()))
    iters = it.value
    # native FP64 getrf + getrs (one timed call, ~0.4 s)
    Af = torch.empty_like(A)
    Xn = torch.empty_like(B)
    dinfo = torch.zeros(1, dtype=torch.int32, device="cuda")
    Af.copy_(A)
    Xn.copy_(B)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lib.gb_dgetrf_dev(n, n, Af.data_ptr(), n, ipiv.data_ptr(), dinfo.data_ptr())
    lib.gb_dgetrs_dev(b"N", n, nrhs, Af.data_ptr(), n, ipiv.data_ptr(), Xn.data_ptr(), n)
    torch.cuda.synchronize()
    t_native = allreduce_max(time.perf_counter() - t0, world)
    flops = 2.0 / 3.0 * n ** 3 + 2.0 * n * n * nrhs
    return {"workload": f"DGESV N={n} NRHS={nrhs}, A,B uniform(-1,1) seeded", "unit": UNIT,
            "mixed": {"value": world * flops / t_mixed / 1e12, "ms": t_mixed * 1e3,
                      "iter": iters, "backward_error_eps": berr / 2.220446049250313e-16,
                      "bound_n_eps": n},
            "native_fp64": {"value": world * flops / t_native / 1e12, "ms": t_native * 1e3},
            "speedup_mixed_over_native": t_native / t_mixed}


def batched_compare(lib, torch, gb, count=20000, loop_sample=1000):
    """20,000 uneven problems (n uniform in [8,256]; 40% DGEMM, 40% DGESV with
    one right-hand side, 20% DPOTRF), FP64, one grouped persistent launch
    replayed from a CUDA graph; the per-problem loop of the same kernel is
    timed on the first `loop_sample` problems of the table and scaled."""
    from openblas_gb300 import batch as BT
    import numpy as np
    BT.bind(lib)
    rng = np.random.default_rng(1)
    sizes = rng.integers(8, 257, size=(count, 3))
    kinds = rng.choice(3, size=count, p=[0.4, 0.4, 0.2])
    ta = tb = tc = tp = 0
    for i in range(count):
        m, n, k = (int(x) for x in sizes[i])
        if kinds[i] == 0:
            ta, tb, tc = ta + m * k, tb + k * n, tc + m * n
        else:
            ta, tb, tp = ta + n * n, tb + n, tp + n
    bufA = torch.empty(ta, dtype=torch.float64, device="cuda")
    bufB = torch.empty(tb, dtype=torch.float64, device="cuda")
    bufC = torch.empty(max(tc, 1), dtype=torch.float64, device="cuda")
    piv = torch.zeros(tp + 1, dtype=torch.int32, device="cuda")
    info = torch.zeros(count, dtype=torch.int32, device="cuda")
    table = (BT.Problem * count)()
    oa = ob = oc = op = 0
    flops = np.zeros(count)
    spd = []
    for i in range(count):
        m, n, k = (int(x) for x in sizes[i])
        q = table[i]
        if kinds[i] == 0:
            q.type, q.m, q.n, q.k = 0, m, n, k
            q.transa, q.transb, q.alpha, q.beta = b"N", b"N", 1.0, 0.0
            q.A, q.lda = bufA.data_ptr() + 8 * oa, m
            q.B, q.ldb = bufB.data_ptr() + 8 * ob, k
            q.C, q.ldc = bufC.data_ptr() + 8 * oc, m
            oa, ob, oc = oa + m * k, ob + k * n, oc + m * n
            flops[i] = 2.0 * m * n * k
        else:
            q.type, q.n = int(kinds[i]), n
            q.A, q.lda = bufA.data_ptr() + 8 * oa, n
            q.info = info.data_ptr() + 4 * i
            if kinds[i] == 1:
                q.k, q.B, q.ldb, q.C = 1, bufB.data_ptr() + 8 * ob, n, piv.data_ptr() + 4 * op
                ob, op = ob + n, op + n
                flops[i] = 2.0 / 3.0 * n ** 3 + 2.0 * n * n
            else:
                q.uplo = b"L"
                spd.append((oa, n))
                flops[i] = n ** 3 / 3.0
            oa += n * n
    g = torch.Generator(device="cuda")

    def init():
        g.manual_seed(3)
        bufA.uniform_(-1, 1, generator=g)
        bufB.uniform_(-1, 1, generator=g)
        for (o, n) in spd:  # B + B^T + n I: symmetric positive definite
            blk = bufA[o:o + n * n].view(n, n)
            blk.add_(blk.T.clone()).add_(torch.eye(n, dtype=torch.float64, device="cuda") * n)

    out = {"workload": f"{count} problems, n uniform in [8,256]: 40% DGEMM (m,n,k independent), "
                       "40% DGETRF+DGETRS (1 RHS), 20% DPOTRF; FP64", "unit": UNIT}
    total = float(flops.sum())
    for flags, name in ((0, "grouped_graph_fp64"), (BT.GB_BATCH_MIXED, "grouped_graph_mixed")):
        init()
        plan = lib.gb_batch_plan_create(table, count, flags)
        lib.gb_batch_plan_tune(plan)
        init()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lib.gb_batch_execute(plan)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[name] = {"value": total / dt / 1e12, "ms": dt * 1e3,
                     "threads_per_cta": lib.gb_batch_plan_threads(plan),
                     "nonzero_info": int((info != 0).sum().item())}
        lib.gb_batch_plan_destroy(plan)
    # per-problem loop of the same kernel on a sample of the table
    sub = (BT.Problem * loop_sample)(*[table[i] for i in range(loop_sample)])
    init()
    plan = lib.gb_batch_plan_create(sub, loop_sample, 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lib.gb_batch_execute_loop(plan)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    lib.gb_batch_plan_destroy(plan)
    sflops = float(flops[:loop_sample].sum())
    out["per_problem_loop_fp64"] = {"value": sflops / dt / 1e12, "ms_sample": dt * 1e3,
                                    "sample": f"first {loop_sample} problems of the table"}
    out["speedup_grouped_over_loop"] = out["grouped_graph_fp64"]["value"] / \
        out["per_problem_loop_fp64"]["value"]
    return out


# --------------------------------------------------------------------------
# main arm
# --------------------------------------------------------------------------
def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch

    import openblas_gb300 as gb
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    lib = gb.load()
    n, S = args.n, args.slices
    # one stream for torch's allocations/fills and the library's kernels, so
    # every buffer is ordered with the work that uses it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    lib.gb_set_stream(C.c_void_p(stream.cuda_stream))

    g = torch.Generator(device="cuda")
    g.manual_seed(1234 + rank)
    A = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    Cd = torch.empty((n, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    def emulated_step():
        st = lib.gb_dgemm_emulated_dev(b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n,
                                       0.0, Cd.data_ptr(), n, S)
        if st != 0:
            raise RuntimeError(gb.last_error(lib))

    for _ in range(args.warmup):
        emulated_step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    lib.gb_profile_kernel_ms(b"slice_gemm", None, 1)
    lib.gb_profile_enable(1)
    launches0 = lib.gb_kernel_launches()
    barrier(world)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        emulated_step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    launches = lib.gb_kernel_launches() - launches0
    lib.gb_profile_enable(0)
    cnt = C.c_int(0)
    kern_ms = lib.gb_profile_kernel_ms(b"slice_gemm", C.byref(cnt), 1) / max(cnt.value, 1)
    clk = clocks.stop()
    ms = allreduce_max(e0.elapsed_time(e1) / args.steps, world)
    flops = 2.0 * n ** 3
    value = world * flops / (ms * 1e-3) / 1e12

    # native FP64 on the same operands (one timed call; ~0.9 s at 8192)
    Cn = torch.empty_like(Cd)
    st = lib.gb_dgemm_native_dev(b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0,
                                 Cn.data_ptr(), n)
    torch.cuda.synchronize()
    n0 = torch.cuda.Event(enable_timing=True)
    n1 = torch.cuda.Event(enable_timing=True)
    n0.record(stream)
    lib.gb_dgemm_native_dev(b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0,
                            Cn.data_ptr(), n)
    n1.record(stream)
    torch.cuda.synchronize()
    native_ms = n0.elapsed_time(n1)
    native_tflops = flops / (native_ms * 1e-3) / 1e12

    # error of the emulated result against the native FP64 one, normwise
    # against |A||B| (computed with the native FP64 GEMM on |A|, |B|)
    Ga = torch.empty_like(Cd)
    Aa, Ba = A.abs(), B.abs()
    lib.gb_dgemm_native_dev(b"N", b"N", n, n, n, 1.0, Aa.data_ptr(), n, Ba.data_ptr(), n, 0.0,
                            Ga.data_ptr(), n)
    emulated_step()
    torch.cuda.synchronize()
    eps = float(np.finfo(np.float64).eps)
    err_norm = float((Cd - Cn).abs().max() / Ga.max()) / eps
    err_comp = float(((Cd - Cn).abs() / Ga).max()) / eps
    del Aa, Ba, Ga, Cn

    # end to end through cblas_dgemm with pinned host buffers
    Ah = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Bh = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Ch = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    Ah.copy_(A.cpu())
    Bh.copy_(B.cpu())
    ns = gb.cblas()
    lib.gb_set_dgemm_mode(1)
    lib.gb_set_ozaki_slices(S)

    def e2e_step():
        ns.cblas_dgemm(102, 111, 111, n, n, n, 1.0, Ah.data_ptr(), n, Bh.data_ptr(), n, 0.0,
                       Ch.data_ptr(), n)

    e2e_step()
    e2e_steps = max(3, min(args.steps, 10))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    e2e_dt = allreduce_max((time.perf_counter() - t0) / e2e_steps, world)
    lib.gb_set_dgemm_mode(0)
    st, msg = gb.last_error(lib)
    if st not in (0,):
        raise RuntimeError(msg)

    # DGESV N=8192, NRHS=1: mixed precision (FP32 LU on the GPU + FP64
    # refinement) against native FP64 getrf+getrs, both on the same operands
    dgesv = batched = None
    if not args.no_extras:
        dgesv = dgesv_compare(lib, torch, gb, world)
        batched = batched_compare(lib, torch, gb)

    peaks, src = measured_peaks()
    slice_flops = S * (S + 1) / 2 * flops
    achieved = slice_flops / (kern_ms * 1e-3) / 1e12
    peak = float(peaks.get("bf16_tflops_sustained", 1700.0))
    traffic, traffic_src = profiled_traffic(n)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, S),
        "precision": {"method": "ozaki-7bit-slices-bf16-tcgen05", "slices": S,
                      "normwise_err_vs_native_fp64_eps": err_norm,
                      "componentwise_err_vs_native_fp64_eps": err_comp},
        "native_fp64": {"value": native_tflops * world, "unit": UNIT, "ms_per_step": native_ms,
                        "speedup_emulated_over_native": value / (native_tflops * world)},
        "e2e": {"value": world * flops / e2e_dt / 1e12, "unit": UNIT,
                "h2d_bytes_per_step": 2 * n * n * 8, "d2h_bytes_per_step": n * n * 8,
                "api": "cblas_dgemm (host pointers, pinned), GB_DGEMM_MODE=emulated"},
        "roofline": {"bound": "tensor", "kernel": "slice_gemm_kernel (tcgen05 kind::f16)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "peak_source": f"{src} bf16_tflops_sustained",
                     "kernel_ms_per_launch": kern_ms,
                     "algorithmic_flops_per_launch": slice_flops},
        "dgesv": dgesv,
        "batched": batched,
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if rank == 0 and world == 1:
        line["cpu_baseline"] = cpu_baseline_sample()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
