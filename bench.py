#!/usr/bin/env python3
"""Benchmark: DGEMM TFLOP/s at FP64 accuracy on one GB300 -- emulated FP64
(Ozaki 8-bit slices on the bf16 tensor cores) against native FP64.

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
    ap.add_argument("--slices", type=int, default=0,
                    help="8-bit slices of the emulated DGEMM (0: chosen from the operands and "
                         "the accuracy target, the library default)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the DGESV and batched legs (profiling runs)")
    ap.add_argument("--peaks", action="store_true",
                    help="measure the FP64 peak rates (DFMA, DMMA probes) and the native DGEMM's "
                         "fraction of them instead of the headline step")
    ap.add_argument("--batch", action="store_true",
                    help="run only the batched-solver comparison (one JSON line)")
    ap.add_argument("--batch-count", type=int, default=20000,
                    help="problems in the batched comparison")
    ap.add_argument("--suite", action="store_true",
                    help="measure every configuration of the level-3/LAPACK sweep (one JSON "
                         "line each) instead of the headline step")
    ap.add_argument("--suite-only", default="",
                    help="with --suite: comma-separated sections to run (dgemm1024, dgemm_sweep, "
                         "sgemm, dtrsm, dsyrk, emulated, complex, dgesv, illcond, dpotrf)")
    return ap.parse_args()


def workload_config(n, slices):
    how = f"{slices} 8-bit slices" if slices > 0 else \
        "per 256-column tile the modular scheme or the fewest 8-bit slices meeting 8 eps"
    return {
        "workload": f"DGEMM NN M=N=K={n}, alpha=1, beta=0, A,B,C uniform(-1,1) seeded; "
                    f"FP64-accuracy emulation ({how}) vs native FP64",
        "m": n, "n": n, "k": n, "transa": "N", "transb": "N", "slices": slices or "auto",
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
    """The slowest rank's value (replica timing); the tensor lives where the
    process group's backend wants it (NCCL on the GPU, gloo on the host)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
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


def profiled_traffic(n, kernel="slice_gemm"):
    """DRAM bytes per launch of the tensor-core kernel (`slice_gemm` or
    `residue_gemm`) from its committed ncu summary (dram__bytes_read.sum +
    dram__bytes_write.sum, one-pass capture).  A capture at exactly n is used
    as is; otherwise the nearest captured size is scaled by n^3 (every tile
    re-reads its K-panel of operands for each product) and the result says
    so."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_ncu.txt")
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
# --suite: every configuration of the sweep, one JSON line each
# --------------------------------------------------------------------------
def _events(torch, stream):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time_dev(torch, stream, fn, reps=3, warm=1):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(reps):
        e0, e1 = _events(torch, stream)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return statistics.median(out)


def _emit(d):
    print(json.dumps(d), flush=True)


def run_suite(args):
    import numpy as np
    import torch

    import openblas_gb300 as gb
    torch.cuda.set_device(0)
    lib = gb.load()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    lib.gb_set_stream(C.c_void_p(stream.cuda_stream))
    eps = float(np.finfo(np.float64).eps)

    def check(st):
        if st != 0:
            raise RuntimeError(gb.last_error(lib))

    sections = set(args.suite_only.split(",")) if args.suite_only else None

    def want(key):
        return sections is None or key in sections

    def urand(shape, seed, dtype=torch.float64):
        g = torch.Generator(device="cuda")
        g.manual_seed(seed)
        return (torch.rand(shape, dtype=dtype, device="cuda", generator=g) * 2 - 1)

    if want("dgemm1024"):
        # ---- DGEMM 1024^3 NN alpha=1.5 beta=0.5 (native), DMMCH-style ratio
        n = 1024
        A, B, C0 = urand((n, n), 1), urand((n, n), 2), urand((n, n), 3)
        Cd = C0.clone()
        ms = _time_dev(torch, stream, lambda: check(lib.gb_dgemm_native_dev(
            b"N", b"N", n, n, n, 1.5, A.data_ptr(), n, B.data_ptr(), n, 0.5, Cd.data_ptr(), n)))
        Cd.copy_(C0)
        check(lib.gb_dgemm_native_dev(b"N", b"N", n, n, n, 1.5, A.data_ptr(), n, B.data_ptr(), n, 0.5,
                                      Cd.data_ptr(), n))
        torch.cuda.synchronize()
        # torch tensors hold the column-major matrices transposed: C^T = B^T A^T
        Ah, Bh, Ch = A.cpu().numpy().T, B.cpu().numpy().T, C0.cpu().numpy().T
        ref = 1.5 * (Ah @ Bh) + 0.5 * Ch
        G = 1.5 * (np.abs(Ah) @ np.abs(Bh)) + 0.5 * np.abs(Ch)
        ratio = float(np.max(np.abs(Cd.cpu().numpy().T - ref) / (eps * G)))
        _emit({"suite": "dgemm_1024", "workload": "DGEMM NN 1024^3 alpha=1.5 beta=0.5, native FP64",
               "value": 2 * n ** 3 / ms / 1e9, "unit": UNIT, "ms": ms,
               "dmmch_ratio_eps": ratio, "dmmch_bound": 2 * (n + 2)})
        del A, B, C0, Cd

    if want("dgemm_sweep"):
        # ---- native DGEMM sweep, lda = M + 8, all four transposes
        for n in (2048, 4096, 8192, 16384):
            ld = n + 8
            A, B, Cd = urand((n, ld), 10 + n), urand((n, ld), 11 + n), torch.zeros((n, ld), dtype=torch.float64, device="cuda")
            for ta, tb in (("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")):
                if n == 16384 and (ta, tb) != ("N", "N"):
                    continue  # ~7 s per native call at 16384: one combination
                reps = 1 if n == 16384 else 2
                ms = _time_dev(torch, stream, lambda: check(lib.gb_dgemm_native_dev(
                    ta.encode(), tb.encode(), n, n, n, 1.0, A.data_ptr(), ld, B.data_ptr(), ld, 0.0,
                    Cd.data_ptr(), ld)), reps=reps, warm=0 if n == 16384 else 1)
                _emit({"suite": f"dgemm_native_{n}_{ta}{tb}",
                       "workload": f"DGEMM {ta}{tb} M=N=K={n}, lda=ldb=ldc={ld}, native FP64",
                       "value": 2 * n ** 3 / ms / 1e9, "unit": UNIT, "ms": ms})
            del A, B, Cd

    if want("sgemm"):
        # ---- SGEMM 16384^3 FP32: tensor-core (bf16x3) and SIMT forms
        n = 16384
        A, B = urand((n, n), 20, torch.float32), urand((n, n), 21, torch.float32)
        Cs = torch.zeros((n, n), dtype=torch.float32, device="cuda")
        res = {}
        for mode, name in ((2, "tensor_bf16x3"), (1, "simt_fp32")):
            lib.gb_set_sgemm_mode(mode)
            res[name] = _time_dev(torch, stream, lambda: check(lib.gb_sgemm_dev(
                b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0, Cs.data_ptr(), n)),
                reps=2)
        lib.gb_set_sgemm_mode(0)
        # accuracy of the tensor form on a 2048-row slab against FP64
        lib.gb_set_sgemm_mode(2)
        check(lib.gb_sgemm_dev(b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0,
                               Cs.data_ptr(), n))
        lib.gb_set_sgemm_mode(0)
        torch.cuda.synchronize()
        rows = 256
        a64 = A.double()
        Cref = torch.empty((n, n), dtype=torch.float64, device="cuda")
        b64 = B.double()
        check(lib.gb_dgemm_native_dev(b"N", b"N", rows, n, n, 1.0, a64.data_ptr(), n, b64.data_ptr(),
                                      n, 0.0, Cref.data_ptr(), n))
        Gs = torch.empty_like(Cref)
        aa, ba = a64.abs(), b64.abs()
        check(lib.gb_dgemm_native_dev(b"N", b"N", rows, n, n, 1.0, aa.data_ptr(), n, ba.data_ptr(),
                                      n, 0.0, Gs.data_ptr(), n))
        torch.cuda.synchronize()
        # column-major rows 0..rows-1 are the first `rows` entries of each torch row
        diff = (Cs.double()[:, :rows] - Cref[:, :rows]).abs() / Gs[:, :rows]
        feps = float(np.finfo(np.float32).eps)
        _emit({"suite": "sgemm_16384", "workload": "SGEMM NN 16384^3 FP32",
               "value": 2 * n ** 3 / res["tensor_bf16x3"] / 1e9, "unit": UNIT,
               "ms": res["tensor_bf16x3"], "method": "bf16x3 split, six tcgen05 products, FP32 TMEM",
               "simt_fp32": {"value": 2 * n ** 3 / res["simt_fp32"] / 1e9, "ms": res["simt_fp32"]},
               "componentwise_err_fp32_eps_first_256_rows": float(diff.max()) / feps,
               "bound_k_plus_2": n + 2})
        del A, B, Cs, a64, b64, aa, ba, Cref, Gs, diff

    if want("dtrsm"):
        # ---- DTRSM Left/Lower/NoTrans/NonUnit 8192^2, diagonal n + U(0,1)
        n = 8192
        L = urand((n, n), 30)
        L = torch.tril(L.T, -1).T.contiguous()  # strictly lower in column-major
        g = torch.Generator(device="cuda")
        g.manual_seed(31)
        L.view(-1)[:: n + 1] = n + torch.rand(n, dtype=torch.float64, device="cuda", generator=g)
        B0 = urand((n, n), 32)
        Bt = B0.clone()
        Lnorm = float(L.abs().sum(dim=0).max())  # row sums of the column-major L
        R = torch.empty((512, n), dtype=torch.float64, device="cuda")  # column-major n x 512
        trsm = {}
        for mode, name in ((0, "native"), (1, "emulated")):
            lib.gb_set_dgemm_mode(mode)
            ms = _time_dev(torch, stream, lambda: check(lib.gb_dtrsm_dev(
                b"L", b"L", b"N", b"N", n, n, 1.0, L.data_ptr(), n, Bt.data_ptr(), n)), reps=2)
            # residual of a fresh solve, first 512 right-hand sides:
            # max_j |L x_j - b_j|_inf / (|L|_inf |x_j|_inf), in units of eps
            Bt.copy_(B0)
            check(lib.gb_dtrsm_dev(b"L", b"L", b"N", b"N", n, n, 1.0, L.data_ptr(), n,
                                   Bt.data_ptr(), n))
            lib.gb_set_dgemm_mode(0)
            R.copy_(B0[:512])
            check(lib.gb_dgemm_native_dev(b"N", b"N", n, 512, n, 1.0, L.data_ptr(), n, Bt.data_ptr(),
                                          n, -1.0, R.data_ptr(), n))
            torch.cuda.synchronize()
            xn = Bt[:512].abs().amax(dim=1)
            res = float((R.abs().amax(dim=1) / (Lnorm * xn)).max()) / eps
            trsm[name] = {"value": n ** 3 / ms / 1e9, "ms": ms, "residual_eps": res}
        _emit({"suite": "dtrsm_8192", "workload": "DTRSM LLNN M=N=8192, native FP64",
               "value": trsm["native"]["value"], "unit": UNIT, "ms": trsm["native"]["ms"],
               "residual_eps": trsm["native"]["residual_eps"]})
        _emit({"suite": "dtrsm_8192_emulated",
               "workload": "DTRSM LLNN M=N=8192, emulated FP64 (recursive, 128-wide FP64 leaves in "
                           "one fused launch each, off-diagonal blocks on the emulated DGEMM, "
                           "automatic choice)",
               "unit": UNIT, **trsm["emulated"], "native_fp64_ms": trsm["native"]["ms"],
               "speedup_over_native": trsm["native"]["ms"] / trsm["emulated"]["ms"]})
        del L, B0, Bt, R

    if want("dsyrk"):
        # ---- DSYRK Lower/NoTrans n = k = 8192: native FP64 and emulated FP64
        n = 8192
        A = urand((n, n), 33)
        C0 = urand((n, n), 34)
        syrk = {}
        for mode, name in ((0, "native"), (1, "emulated")):
            lib.gb_set_dgemm_mode(mode)
            Cs = C0.clone()
            ms = _time_dev(torch, stream, lambda: check(lib.gb_dsyrk_dev(
                b"L", b"N", n, n, -1.0, A.data_ptr(), n, 1.0, Cs.data_ptr(), n)), reps=2)
            Cs.copy_(C0)
            check(lib.gb_dsyrk_dev(b"L", b"N", n, n, -1.0, A.data_ptr(), n, 1.0, Cs.data_ptr(), n))
            syrk[name] = (ms, Cs)
        lib.gb_set_dgemm_mode(0)
        torch.cuda.synchronize()
        # normwise difference on the stored (lower, column-major) triangle,
        # relative to max(|A||A^T| + |C|) (its largest entries lie on the
        # diagonal, sum_l A(i,l)^2, by Cauchy-Schwarz; |C| <= 1)
        low = torch.triu(torch.ones(n, n, dtype=torch.bool, device="cuda"))  # lower of col-major
        diff = float(((syrk["emulated"][1] - syrk["native"][1]).abs() * low).max())
        gmax = float((A * A).sum(dim=0).max()) + 1.0
        for name in ("native", "emulated"):
            d = {"suite": "dsyrk_8192" + ("" if name == "native" else "_emulated"),
                 "workload": f"DSYRK LN n=k=8192, {name} FP64", "unit": UNIT,
                 "value": n ** 3 / syrk[name][0] / 1e9, "ms": syrk[name][0]}
            if name == "emulated":
                d["normwise_err_vs_native_eps"] = diff / gmax / eps
                d["native_fp64_ms"] = syrk["native"][0]
                d["speedup_over_native"] = syrk["native"][0] / syrk["emulated"][0]
            _emit(d)
        del A, C0, syrk, low
        torch.cuda.empty_cache()

    if want("emulated"):
        # ---- emulated DGEMM: 8-bit slices 5..8, exponent spread e in {0, 8, 16}
        for n in (8192, 16384):
            for e in (0, 8, 16):
                gA, gB = torch.Generator(device="cuda"), torch.Generator(device="cuda")
                gA.manual_seed(40 + e)
                gB.manual_seed(50 + e)
                A = urand((n, n), 60 + e)
                B = urand((n, n), 70 + e)
                if e:
                    A = torch.ldexp(A, torch.randint(-e, e + 1, (n, n), device="cuda", generator=gA))
                    B = torch.ldexp(B, torch.randint(-e, e + 1, (n, n), device="cuda", generator=gB))
                Cn = None
                if n == 8192 or e == 0:
                    Cn = torch.empty((n, n), dtype=torch.float64, device="cuda")
                    t0 = time.perf_counter()
                    check(lib.gb_dgemm_native_dev(b"N", b"N", n, n, n, 1.0, A.data_ptr(), n,
                                                  B.data_ptr(), n, 0.0, Cn.data_ptr(), n))
                    torch.cuda.synchronize()
                    native_ms = (time.perf_counter() - t0) * 1e3
                    Ga = torch.empty_like(Cn)
                    Aa, Ba = A.abs(), B.abs()
                    check(lib.gb_dgemm_native_dev(b"N", b"N", n, n, n, 1.0, Aa.data_ptr(), n,
                                                  Ba.data_ptr(), n, 0.0, Ga.data_ptr(), n))
                    del Aa, Ba
                Ce = torch.empty((n, n), dtype=torch.float64, device="cuda")
                # S = 0: the automatic choice (the library default: modular
                # scheme or slice count per tile), "0s": automatic with digit
                # slices only
                variants = (0, "0s", 5, 6, 7, 8) if n == 8192 else (0, "0s", 7)
                for S in variants:
                    modular = 0 if S == "0s" else 1
                    Sv = 0 if S == "0s" else S
                    lib.gb_set_ozaki_modular(modular)
                    ms = _time_dev(torch, stream, lambda: check(lib.gb_dgemm_emulated_dev(
                        b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0,
                        Ce.data_ptr(), n, Sv)), reps=3 if n == 8192 else 2)
                    lib.gb_set_ozaki_modular(1)
                    tag = f"s{S}" if Sv else ("auto" if modular else "auto_slices")
                    chosen_m, chosen_s = lib.gb_last_ozaki_moduli(), lib.gb_last_ozaki_slices()
                    how = f"{Sv} slices" if Sv else \
                        f"automatic choice ({chosen_m} moduli, {chosen_s} slices)"
                    d = {"suite": f"dgemm_emulated_{n}_e{e}_{tag}",
                         "workload": f"emulated DGEMM NN {n}^3, A,B = U.*2^E, E in [-{e},{e}], {how}",
                         "value": 2 * n ** 3 / ms / 1e9, "unit": UNIT, "ms": ms}
                    if not Sv:
                        d["slices_chosen"] = chosen_s
                        d["moduli_chosen"] = chosen_m
                    if Cn is not None:
                        torch.cuda.synchronize()
                        diff = (Ce - Cn).abs()
                        d["normwise_err_vs_native_eps"] = float(diff.max() / Ga.max()) / eps
                        d["componentwise_err_vs_native_eps"] = float((diff / Ga).max()) / eps
                        d["native_fp64_ms"] = native_ms
                        d["speedup_over_native"] = native_ms / ms
                    _emit(d)
                del A, B, Ce
                if Cn is not None:
                    del Cn, Ga
                torch.cuda.empty_cache()

    if want("complex"):
        # ---- complex GEMM 8192^3 NN: ZGEMM (4M embedding) native and emulated,
        # ZGEMM3M emulated, CGEMM / CGEMM3M on the tensor-core FP32 engine;
        # rates count 8 n^3 real flops per complex GEMM (3M forms: effective rate)
        n = 8192
        one = np.array([1.0, 0.0])
        zero = np.array([0.0, 0.0])
        Az = torch.complex(urand((n, n), 80), urand((n, n), 81))
        Bz = torch.complex(urand((n, n), 82), urand((n, n), 83))
        Cn = torch.empty_like(Az)
        Ce = torch.empty_like(Az)

        def zcall(fn, Cout):
            return lambda: check(getattr(lib, fn)(b"N", b"N", n, n, n, one.ctypes.data, Az.data_ptr(),
                                                  n, Bz.data_ptr(), n, zero.ctypes.data,
                                                  Cout.data_ptr(), n))
        zres = {}
        lib.gb_set_dgemm_mode(0)
        zres["zgemm_native"] = _time_dev(torch, stream, zcall("gb_zgemm_dev", Cn), reps=1, warm=0)
        lib.gb_set_dgemm_mode(1)
        # error scale: max of |A||B| (complex moduli), the DMMCH denominator
        Am, Bm = Az.abs().contiguous(), Bz.abs().contiguous()
        Gz = torch.empty((n, n), dtype=torch.float64, device="cuda")
        check(lib.gb_dgemm_native_dev(b"N", b"N", n, n, n, 1.0, Am.data_ptr(), n, Bm.data_ptr(), n,
                                      0.0, Gz.data_ptr(), n))
        torch.cuda.synchronize()
        gmax = float(Gz.max())
        del Am, Bm, Gz
        zres["zgemm_emulated"] = _time_dev(torch, stream, zcall("gb_zgemm_dev", Ce), reps=3)
        torch.cuda.synchronize()
        zerr = float((Ce - Cn).abs().max()) / gmax / eps
        zres["zgemm3m_emulated"] = _time_dev(torch, stream, zcall("gb_zgemm3m_dev", Ce), reps=3)
        torch.cuda.synchronize()
        z3err = float((Ce - Cn).abs().max()) / gmax / eps
        lib.gb_set_dgemm_mode(0)
        for key, err in (("zgemm_native", None), ("zgemm_emulated", zerr), ("zgemm3m_emulated", z3err)):
            d = {"suite": f"{key}_{n}", "workload": f"{key.split('_')[0].upper()} NN {n}^3 complex128, "
                 f"{key.split('_')[1]} FP64 engine", "value": 8 * n ** 3 / zres[key] / 1e9,
                 "unit": UNIT, "ms": zres[key], "flops_counted": "8 n^3"}
            if err is not None:
                d["normwise_err_vs_native_zgemm_eps_of_max_AB"] = err
                d["speedup_over_native_zgemm"] = zres["zgemm_native"] / zres[key]
            _emit(d)
        del Az, Bz, Cn, Ce
        Ac = torch.complex(urand((n, n), 84, torch.float32), urand((n, n), 85, torch.float32))
        Bc = torch.complex(urand((n, n), 86, torch.float32), urand((n, n), 87, torch.float32))
        Cc = torch.empty_like(Ac)
        onef, zerof = one.astype(np.float32), zero.astype(np.float32)
        for fn in ("gb_cgemm_dev", "gb_cgemm3m_dev"):
            ms = _time_dev(torch, stream, lambda: check(getattr(lib, fn)(
                b"N", b"N", n, n, n, onef.ctypes.data, Ac.data_ptr(), n, Bc.data_ptr(), n,
                zerof.ctypes.data, Cc.data_ptr(), n)), reps=3)
            name = fn[3:-4]
            _emit({"suite": f"{name}_{n}", "workload": f"{name.upper()} NN {n}^3 complex64, "
                   "bf16x3 tensor-core FP32 engine", "value": 8 * n ** 3 / ms / 1e9, "unit": UNIT,
                   "ms": ms, "flops_counted": "8 n^3"})
        del Ac, Bc, Cc
        torch.cuda.empty_cache()

    if want("dgesv"):
        # ---- DGESV N in {8192, 16384, 32768}, NRHS in {1, 64}: mixed vs native
        for n in (8192, 16384, 32768):
            A = urand((n, n), 80 + n)
            ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
            dinfo = torch.zeros(1, dtype=torch.int32, device="cuda")
            Af = A.clone()
            t0 = time.perf_counter()
            check(lib.gb_dgetrf_dev(n, n, Af.data_ptr(), n, ipiv.data_ptr(), dinfo.data_ptr()))
            torch.cuda.synchronize()
            t_getrf = time.perf_counter() - t0
            for nrhs in (1, 64):
                Bm = urand((nrhs, n), 90 + nrhs)
                Xn = Bm.clone()
                t0 = time.perf_counter()
                check(lib.gb_dgetrs_dev(b"N", n, nrhs, Af.data_ptr(), n, ipiv.data_ptr(),
                                        Xn.data_ptr(), n))
                torch.cuda.synchronize()
                t_native = t_getrf + time.perf_counter() - t0
                X = torch.zeros_like(Bm)
                p2 = torch.zeros(n, dtype=torch.int32, device="cuda")
                it, info = C.c_int(0), C.c_int(0)

                Aw = A.clone()  # a fallback would overwrite its A with the FP64 LU

                def mixed():
                    check(lib.gb_dsgesv_dev(n, nrhs, Aw.data_ptr(), n, p2.data_ptr(), Bm.data_ptr(),
                                            n, X.data_ptr(), n, C.byref(it), C.byref(info)))

                mixed()
                torch.cuda.synchronize()
                ts = []
                for _ in range(2 if n == 32768 else 3):
                    t0 = time.perf_counter()
                    mixed()
                    torch.cuda.synchronize()
                    ts.append(time.perf_counter() - t0)
                t_mixed = statistics.median(ts)
                R = Bm.clone()
                check(lib.gb_dgemm_native_dev(b"N", b"N", n, nrhs, n, -1.0, A.data_ptr(), n,
                                              X.data_ptr(), n, 1.0, R.data_ptr(), n))
                torch.cuda.synchronize()
                anorm = float(A.abs().sum(dim=0).max())
                berr = float((R.abs().amax(dim=1) / (anorm * X.abs().amax(dim=1) + Bm.abs().amax(dim=1))).max())
                flops = 2.0 / 3.0 * n ** 3 + 2.0 * n * n * nrhs
                _emit({"suite": f"dgesv_{n}_{nrhs}", "workload": f"DGESV N={n} NRHS={nrhs}, uniform(-1,1)",
                       "value": flops / t_mixed / 1e12, "unit": UNIT, "ms": t_mixed * 1e3,
                       "iter": it.value, "info": info.value,
                       "backward_error_eps_max_over_rhs": berr / eps, "bound_n_eps": n,
                       "native_fp64": {"value": flops / t_native / 1e12, "ms": t_native * 1e3},
                       "speedup_mixed_over_native": t_native / t_mixed})
                del Bm, Xn, X, R, Aw
            del A, Af
            torch.cuda.empty_cache()

    if want("illcond"):
        # ---- ill-conditioned DGESV (GMRES-IR): A = U diag(logspace(0,-kappa)) V^T, U and
        # V the Q factors of seeded uniform matrices (QR on the device); N = 32768 is left
        # out, as its two FP64 QRs alone would take minutes
        for n in (4096, 8192, 16384):
            U, _ = torch.linalg.qr(urand((n, n), 121))
            V, _ = torch.linalg.qr(urand((n, n), 122))
            for kappa in (4, 8, 12):
                sv = torch.logspace(0.0, -float(kappa), n, dtype=torch.float64, device="cuda")
                A = ((U * sv) @ V.T).T.contiguous()  # column-major buffer of A
                Aw = A.clone()  # the FP64 fallback overwrites its A with the LU factors
                Bm = urand((1, n), 95)
                X = torch.zeros_like(Bm)
                p2 = torch.zeros(n, dtype=torch.int32, device="cuda")
                it, info = C.c_int(0), C.c_int(0)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                check(lib.gb_dsgesv_dev(n, 1, Aw.data_ptr(), n, p2.data_ptr(), Bm.data_ptr(), n,
                                        X.data_ptr(), n, C.byref(it), C.byref(info)))
                torch.cuda.synchronize()
                t_mixed = time.perf_counter() - t0
                R = Bm.clone()
                check(lib.gb_dgemm_native_dev(b"N", b"N", n, 1, n, -1.0, A.data_ptr(), n,
                                              X.data_ptr(), n, 1.0, R.data_ptr(), n))
                torch.cuda.synchronize()
                anorm = float(A.abs().sum(dim=0).max())
                berr = float(R.abs().max() / (anorm * X.abs().max() + Bm.abs().max()))
                _emit({"suite": f"dgesv_illcond_{n}_kappa1e{kappa}",
                       "workload": f"DGESV N={n} NRHS=1, A = U diag(logspace(0,-{kappa})) V^T "
                                   "(U, V: Q factors of seeded uniform matrices)",
                       "ms": t_mixed * 1e3, "iter": it.value, "info": info.value,
                       "backward_error_eps": berr / eps, "bound_n_eps": n,
                       "path": "FP32 LU + IR" if 0 <= it.value <= 30 else
                               ("GMRES-IR" if it.value >= 100 else "FP64-accurate fallback")})
                del A, Aw, Bm, X, R
            del U, V
            torch.cuda.empty_cache()

    if want("dpotrf"):
        # ---- DPOTRF N=32768, A = B B^T / N + I (B uniform), native and emulated updates
        n = 32768
        Bm = urand((n, n), 99)
        A0 = torch.empty((n, n), dtype=torch.float64, device="cuda")
        check(lib.gb_dgemm_emulated_dev(b"N", b"T", n, n, n, 1.0 / n, Bm.data_ptr(), n, Bm.data_ptr(),
                                        n, 0.0, A0.data_ptr(), n, 8))
        A0.view(-1)[:: n + 1] += 1.0
        del Bm
        torch.cuda.empty_cache()
        A = torch.empty_like(A0)
        dinfo = torch.zeros(1, dtype=torch.int32, device="cuda")
        out = {}
        for mode, name in ((1, "emulated_updates"), (0, "native_fp64")):
            lib.gb_set_dgemm_mode(mode)
            ts = []
            for _ in range(2 if mode == 1 else 1):
                A.copy_(A0)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                check(lib.gb_dpotrf_dev(b"L", n, A.data_ptr(), n, dinfo.data_ptr()))
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            out[name] = (statistics.median(ts), int(dinfo.item()))
            if mode == 1:
                # scaled residual of a 2048-column slab: |A0 - L L^T| / (n eps |A0|)
                cols = 2048
                Lw = A.clone()
                Lw.copy_(torch.triu(Lw))  # column-major lower = torch upper
                R = A0[:cols].clone()
                check(lib.gb_dgemm_emulated_dev(b"N", b"T", n, cols, n, -1.0, Lw.data_ptr(), n,
                                                Lw.data_ptr(), n, 1.0, R.data_ptr(), n, 8))
                torch.cuda.synchronize()
                resid = float(R.abs().sum(dim=1).max() / (n * eps * A0.abs().sum(dim=1).max()))
                del Lw, R
        lib.gb_set_dgemm_mode(0)
        # DSPOSV on the same matrix: FP32 Cholesky + FP64 refinement vs native
        # FP64 DPOTRF + DPOTRS (the native factor time is the one just measured)
        Bm = urand((1, n), 98)
        X = torch.zeros_like(Bm)
        it, info = C.c_int(0), C.c_int(0)
        A.copy_(A0)  # the mixed path leaves A alone unless it falls back
        check(lib.gb_dsposv_dev(b"L", n, 1, A.data_ptr(), n, Bm.data_ptr(), n, X.data_ptr(), n,
                                C.byref(it), C.byref(info)))
        ts = []
        for _ in range(2):
            A.copy_(A0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            check(lib.gb_dsposv_dev(b"L", n, 1, A.data_ptr(), n, Bm.data_ptr(), n, X.data_ptr(), n,
                                    C.byref(it), C.byref(info)))
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        t_sposv = statistics.median(ts)
        R = Bm.clone()
        check(lib.gb_dgemm_native_dev(b"N", b"N", n, 1, n, -1.0, A0.data_ptr(), n, X.data_ptr(), n,
                                      1.0, R.data_ptr(), n))
        torch.cuda.synchronize()
        anorm = float(A0.abs().sum(dim=0).max())
        berr_sposv = float(R.abs().max() / (anorm * X.abs().max() + Bm.abs().max())) / eps
        flops = n ** 3 / 3.0
        _emit({"suite": "dsposv_32768_1", "workload": "DSPOSV L N=32768 NRHS=1, A = B B^T/N + I",
               "value": (flops + 2.0 * n * n) / t_sposv / 1e12, "unit": UNIT, "ms": t_sposv * 1e3,
               "iter": it.value, "info": info.value, "backward_error_eps": berr_sposv,
               "bound_n_eps": n,
               "speedup_over_native_dpotrf": out["native_fp64"][0] / t_sposv})
        _emit({"suite": "dpotrf_32768", "workload": "DPOTRF L N=32768, A = B B^T/N + I",
               "value": flops / out["emulated_updates"][0] / 1e12, "unit": UNIT,
               "ms": out["emulated_updates"][0] * 1e3, "info": out["emulated_updates"][1],
               "scaled_residual_first_2048_cols": resid, "bound": 10,
               "native_fp64": {"value": flops / out["native_fp64"][0] / 1e12,
                               "ms": out["native_fp64"][0] * 1e3, "info": out["native_fp64"][1]},
               "speedup_emulated_over_native": out["native_fp64"][0] / out["emulated_updates"][0]})


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
        "same_config": False,
        "sample": f"each step computes a {n}x{slab} column slab ({slab / n:.3f} of the flops) of "
                  f"the configured {n}^3 product, and the line reports its rate; the whole "
                  f"product would take ~{n / slab:.0f}x the step time",
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


def batched_compare(lib, torch, gb, count=20000, loop_sample=1000, cpu_sample=2000):
    """20,000 uneven problems (n uniform in [8,256]; 40% DGEMM, 40% DGESV with
    one right-hand side, 20% DPOTRF), FP64, one grouped persistent launch
    replayed from a CUDA graph; the per-problem loop of the same kernel is
    timed on the first `loop_sample` problems of the table, and the host
    cores (the oracle's routines with OpenMP over problems) on the first
    `cpu_sample` problems."""
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
    sample_end = None
    for i in range(count):
        if i == cpu_sample:
            sample_end = (oa, ob, oc, op)
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
    for flags, name in ((0, "grouped_graph_fp64"), (BT.GB_BATCH_MIXED, "grouped_graph_mixed"),
                        (BT.GB_BATCH_MIXED | BT.GB_BATCH_EMULATED,
                         "grouped_graph_emulated_dgemm_mixed_dgesv")):
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
    # host cores: the oracle's batch loop on the first cpu_sample problems,
    # same inputs, all host threads (one problem per thread)
    if sample_end is not None:
        from oracle import pyoracle
        sa, sb, sc, sp = sample_end
        init()
        torch.cuda.synchronize()
        hA = bufA[:sa].cpu().numpy().copy()
        hB = bufB[:max(sb, 1)].cpu().numpy().copy()
        hC = bufC[:max(sc, 1)].cpu().numpy().copy()
        hp = np.zeros(max(sp, 1), np.int32)
        hinfo = np.zeros(cpu_sample, np.int32)
        ht = (BT.Problem * cpu_sample)()
        for i in range(cpu_sample):
            q, h = table[i], ht[i]
            for f, _ in BT.Problem._fields_:
                setattr(h, f, getattr(q, f))
            h.A = hA.ctypes.data + (q.A - bufA.data_ptr())
            if q.type == 0:
                h.B = hB.ctypes.data + (q.B - bufB.data_ptr())
                h.C = hC.ctypes.data + (q.C - bufC.data_ptr())
            else:
                h.info = hinfo.ctypes.data + 4 * i
                if q.type == 1:
                    h.B = hB.ctypes.data + (q.B - bufB.data_ptr())
                    h.C = hp.ctypes.data + (q.C - piv.data_ptr())
        ncores = os.cpu_count() or 1
        orc = pyoracle.lib()
        orc.orc_set_threads(ncores)
        t0 = time.perf_counter()
        orc.orc_batch(C.cast(ht, C.c_void_p), cpu_sample)
        cdt = time.perf_counter() - t0
        cflops = float(flops[:cpu_sample].sum())
        out["host_cores_oracle_fp64"] = {
            "value": cflops / cdt / 1e12, "ms_sample": cdt * 1e3, "cores": ncores, "kind": "port",
            "sample": f"first {cpu_sample} problems of the table, one problem per thread "
                      "(OpenMP over problems)",
            "nonzero_info": int((hinfo != 0).sum())}
        del hA, hB, hC
    sflops = float(flops[:loop_sample].sum())
    out["per_problem_loop_fp64"] = {"value": sflops / dt / 1e12, "ms_sample": dt * 1e3,
                                    "sample": f"first {loop_sample} problems of the table"}
    out["speedup_grouped_over_loop"] = out["grouped_graph_fp64"]["value"] / \
        out["per_problem_loop_fp64"]["value"]
    return out


# --------------------------------------------------------------------------
# FP64 peaks: the denominator of the native DGEMM's roofline
# --------------------------------------------------------------------------
def run_peaks(args):
    """The FP64 rate of this GPU measured two ways (probe kernels of independent
    DFMA chains and of mma.sync m8n8k4 f64 MMAs, one timed launch each after a
    warm-up) and the library's native DGEMM NN at 4096^3 and 8192^3 against
    the larger of the two (one JSON line)."""
    import torch

    import openblas_gb300 as gb
    probes = C.CDLL(os.path.join(ROOT, "openblas_gb300", "libgbprobes.so"))
    out = {"probe": "fp64 peaks", "unit": UNIT}
    for name in ("dfma", "dmma"):
        fn = getattr(probes, f"gbp_fp64_{name}_tflops")
        fn.restype, fn.argtypes = C.c_int, [C.POINTER(C.c_double)]
        v = C.c_double(0.0)
        out[f"fp64_{name}"] = v.value if fn(C.byref(v)) == 0 else None
    lib = gb.load()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    lib.gb_set_stream(C.c_void_p(stream.cuda_stream))
    peak = max(x for x in (out["fp64_dfma"], out["fp64_dmma"]) if x)
    out["fp64_nominal"] = 1.25  # GB300's dense FP64 figure
    out["peak_used"] = "max(fp64_dfma, fp64_dmma) probes"
    clocks = ClockSampler(0)
    clocks.start()
    for n in (4096, 8192):
        A = torch.rand((n, n), dtype=torch.float64, device="cuda") * 2 - 1
        B = torch.rand((n, n), dtype=torch.float64, device="cuda") * 2 - 1
        Cd = torch.empty((n, n), dtype=torch.float64, device="cuda")
        ms = _time_dev(torch, stream, lambda: lib.gb_dgemm_native_dev(
            b"N", b"N", n, n, n, 1.0, A.data_ptr(), n, B.data_ptr(), n, 0.0, Cd.data_ptr(), n),
            reps=2, warm=1)
        out[f"native_dgemm_{n}"] = 2 * n ** 3 / ms / 1e9
        out[f"native_dgemm_{n}_frac_of_fp64_peak"] = out[f"native_dgemm_{n}"] / peak
        out[f"native_dgemm_{n}_frac_of_fp64_nominal"] = out[f"native_dgemm_{n}"] / 1.25
        del A, B, Cd
    out["clocks"] = clocks.stop()
    print(json.dumps(out), flush=True)


# --------------------------------------------------------------------------
# main arm
# --------------------------------------------------------------------------
def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.suite:
        run_suite(args)
        return
    if args.peaks:
        run_peaks(args)
        return
    if args.batch:
        import torch

        import openblas_gb300 as gb
        lib = gb.load()
        out = batched_compare(lib, torch, gb, count=args.batch_count,
                              loop_sample=min(1000, args.batch_count),
                              cpu_sample=min(2000, args.batch_count))
        print(json.dumps(out), flush=True)
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
    # what the step runs with: the modular scheme (14 residue products per
    # output tile) or S digit slices (S(S+1)/2 products)
    moduli = 0 if S > 0 else lib.gb_last_ozaki_moduli()
    S_used = S if S > 0 else lib.gb_last_ozaki_slices()
    kernel = "residue_gemm" if moduli else "slice_gemm"
    products = moduli if moduli else S_used * (S_used + 1) // 2

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    lib.gb_profile_kernel_ms(kernel.encode(), None, 1)
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
    kern_ms = lib.gb_profile_kernel_ms(kernel.encode(), C.byref(cnt), 1) / max(cnt.value, 1)
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
    # each call timed on the host (the call blocks until C is in host
    # memory); the median of the calls is reported, with the mean beside it
    e2e_steps = max(5, min(args.steps, 15))
    barrier(world)
    e2e_times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    e2e_dt = allreduce_max(float(np.median(e2e_times)), world)
    e2e_mean = allreduce_max(float(np.mean(e2e_times)), world)
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
    # K runs in segments (4096 deep), one tensor-core launch per segment
    launches_per_step = max(cnt.value / args.steps, 1.0)
    slice_flops = products * flops / launches_per_step
    achieved = slice_flops / (kern_ms * 1e-3) / 1e12
    peak = float(peaks.get("bf16_tflops_sustained", 1700.0))
    traffic, traffic_src = profiled_traffic(n, kernel)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(n, S),
        "precision": {"method": ("ozaki-modular-residues-bf16-tcgen05" if moduli else
                                 "ozaki-8bit-slices-bf16-tcgen05"),
                      "moduli": moduli, "slices": S_used, "tensor_products_per_tile": products,
                      "slice_choice": "fixed" if S > 0 else
                      "automatic: per 256-column tile the modular scheme where its worst-case "
                      "bound is <= 8 eps, else the fewest slices that meet it",
                      "normwise_err_vs_native_fp64_eps": err_norm,
                      "componentwise_err_vs_native_fp64_eps": err_comp},
        "native_fp64": {"value": native_tflops * world, "unit": UNIT, "ms_per_step": native_ms,
                        "speedup_emulated_over_native": value / (native_tflops * world)},
        "e2e": {"value": world * flops / e2e_dt / 1e12, "unit": UNIT,
                "h2d_bytes_per_step": 2 * n * n * 8, "d2h_bytes_per_step": n * n * 8,
                "ms_per_call_median": e2e_dt * 1e3, "ms_per_call_mean": e2e_mean * 1e3,
                "calls": e2e_steps,
                "api": "cblas_dgemm (host pointers, pinned), GB_DGEMM_MODE=emulated"},
        "roofline": {"bound": "tensor",
                     "kernel": f"slice_gemm_kernel<{'true' if moduli else 'false'}> ({kernel}, "
                               "tcgen05 kind::f16)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "peak_source": f"{src} bf16_tflops_sustained",
                     "kernel_ms_per_launch": kern_ms,
                     "launches_per_step": launches_per_step,
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
