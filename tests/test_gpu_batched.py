"""Grouped uneven batch (one persistent launch, CUDA graph) against the oracle:
DGEMM within the DMMCH bound, DGESV with pivots identical to the oracle's LU
and the solve, DPOTRF factors, info codes on singular / non-SPD problems, the
mixed-precision DGESV variant within n*eps backward error, the per-problem
loop of the same kernel giving the same results, and the autotuner."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import EPS, dmmch_ratio

from openblas_gb300 import batch as BT
from openblas_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def make_batch(count, seed, lo=8, hi=96):
    """40% DGEMM, 40% DGESV (1 RHS), 20% DPOTRF with sizes uniform in [lo, hi]."""
    sizes = W.randint(seed, (count, 3), lo, hi)
    kinds = []
    for i in range(count):
        r = i % 5
        kinds.append(BT.GB_BATCH_DGEMM if r < 2 else BT.GB_BATCH_DGESV if r < 4 else BT.GB_BATCH_DPOTRF)
    probs = []
    for i, t in enumerate(kinds):
        m, n, k = (int(x) for x in sizes[i])
        s = seed * 100000 + 10 * i
        if t == BT.GB_BATCH_DGEMM:
            ta, tb = "NT"[i % 2], "NT"[(i // 2) % 2]
            A, B, Cm = W.gemm_operands(s, m, n, k, ta, tb, pad=1)
            probs.append(dict(type=t, m=m, n=n, k=k, ta=ta, tb=tb, alpha=1.0 - 0.25 * (i % 3),
                              beta=[0.0, 1.0, 0.5][i % 3], A=A, B=B, C=Cm))
        elif t == BT.GB_BATCH_DGESV:
            A = W.uniform(s, (n, n))
            if i == 3:
                A[:, n // 2] = 0.0  # singular: info = n//2 + 1, no solve
            probs.append(dict(type=t, n=n, A=A, B=W.uniform(s + 1, (n, 1))))
        else:
            A = W.spd(s, n)
            if i == 4:
                A[n // 3, n // 3] = -1.0
            probs.append(dict(type=t, n=n, uplo="LU"[i % 2], A=A))
    return probs


def upload(probs):
    torch = pytest.importorskip("torch")
    keep, table = [], (BT.Problem * len(probs))()

    def dev(a):
        t = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # column-major buffer
        keep.append(t)
        return t

    for q, p in zip(table, probs):
        q.type = p["type"]
        if p["type"] == BT.GB_BATCH_DGEMM:
            q.m, q.n, q.k = p["m"], p["n"], p["k"]
            q.transa, q.transb = p["ta"].encode(), p["tb"].encode()
            q.alpha, q.beta = p["alpha"], p["beta"]
            for name in "ABC":
                t = dev(p[name])
                p["d" + name] = t
                setattr(q, name, t.data_ptr())
            q.lda, q.ldb, q.ldc = p["A"].shape[0], p["B"].shape[0], p["C"].shape[0]
        else:
            q.n = p["n"]
            tA = dev(p["A"])
            p["dA"] = tA
            q.A, q.lda = tA.data_ptr(), p["n"]
            info = torch.full((1,), -9, dtype=torch.int32, device="cuda")
            keep.append(info)
            p["dinfo"] = info
            q.info = info.data_ptr()
            if p["type"] == BT.GB_BATCH_DGESV:
                tB = dev(p["B"])
                p["dB"] = tB
                q.B, q.ldb, q.k = tB.data_ptr(), p["n"], 1
                piv = torch.zeros(p["n"], dtype=torch.int32, device="cuda")
                keep.append(piv)
                p["dpiv"] = piv
                q.C = piv.data_ptr()
            else:
                q.uplo = p["uplo"].encode()
    return table, keep


def fetch(t):
    return t.cpu().numpy().T.copy(order="F")


def check(probs, orc, mixed=False):
    for i, p in enumerate(probs):
        if p["type"] == BT.GB_BATCH_DGEMM:
            m, n, k = p["m"], p["n"], p["k"]
            A, B, Cm = p["A"], p["B"], p["C"]
            Co = Cm.copy(order="F")
            orc.dgemm(p["ta"], p["tb"], m, n, k, p["alpha"], A, A.shape[0], B, B.shape[0], p["beta"],
                      Co, Co.shape[0])
            G = orc.dgemm_absbound(p["ta"], p["tb"], m, n, k, p["alpha"], A, A.shape[0], B,
                                   B.shape[0], p["beta"], Cm, Cm.shape[0])
            got = fetch(p["dC"])
            assert dmmch_ratio(got[:m], Co[:m], G, k) <= 2 * (k + 2), i
        elif p["type"] == BT.GB_BATCH_DGESV:
            n = p["n"]
            Ao = p["A"].copy(order="F")
            po = np.zeros(n, np.int32)
            io = orc.dgetrf(n, n, Ao, n, po)
            info = int(p["dinfo"].item())
            assert info == io, i
            if info:
                continue
            x = fetch(p["dB"])
            r = np.abs(p["B"] - p["A"] @ x).max()
            den = np.abs(p["A"]).sum(axis=1).max() * np.abs(x).max() + np.abs(p["B"]).max()
            assert r / den <= n * EPS, i
            if not mixed:
                assert np.array_equal(p["dpiv"].cpu().numpy(), po), i
        else:
            n, uplo = p["n"], p["uplo"]
            Ao = p["A"].copy(order="F")
            io = orc.dpotrf(uplo, n, Ao, n)
            info = int(p["dinfo"].item())
            assert info == io, i
            if info:
                continue
            got = fetch(p["dA"])
            tri = np.tril if uplo == "L" else np.triu
            assert np.abs(tri(got) - tri(Ao)).max() <= 1e-12 * max(1.0, np.abs(Ao).max()), i


def _run(gblib, probs, flags=0, loop=False, tune=False):
    BT.bind(gblib)
    table, keep = upload(probs)
    plan = gblib.gb_batch_plan_create(table, len(probs), flags)
    assert plan
    try:
        if tune:
            assert gblib.gb_batch_plan_tune(plan) == 0
            assert gblib.gb_batch_plan_threads(plan) in (128, 256, 512)
            table, keep = upload(probs)  # tuning executed the batch: fresh inputs
            gblib.gb_batch_plan_destroy(plan)
            plan = gblib.gb_batch_plan_create(table, len(probs), flags)
        st = gblib.gb_batch_execute_loop(plan) if loop else gblib.gb_batch_execute(plan)
        assert st == 0
        assert gblib.gb_synchronize() == 0
    finally:
        gblib.gb_batch_plan_destroy(plan)
    return keep


def test_grouped_batch_vs_oracle(orc, gblib, gb_clean):
    probs = make_batch(150, 3)
    keep = _run(gblib, probs)
    check(probs, orc)
    del keep


def test_loop_baseline_same_results(orc, gblib, gb_clean):
    probs = make_batch(40, 4)
    keep = _run(gblib, probs, loop=True)
    check(probs, orc)
    del keep


def test_mixed_dgesv_variant(orc, gblib, gb_clean):
    probs = make_batch(100, 5, 16, 160)
    keep = _run(gblib, probs, flags=BT.GB_BATCH_MIXED)
    check(probs, orc, mixed=True)
    del keep


def test_autotune_then_run(orc, gblib, gb_clean):
    probs = make_batch(60, 6, 32, 200)
    keep = _run(gblib, probs, tune=True)
    check(probs, orc)
    del keep


def test_emulated_dgemm_and_mixed_dgesv_variant(orc, gblib, gb_clean):
    """GB_BATCH_EMULATED | GB_BATCH_MIXED: the DGEMM problems on the
    emulated-FP64 kernel (Ozaki digit slices on the bf16 tensor cores) within
    the DMMCH bound, the DGESV problems on FP32 LU + FP64 refinement within
    n*eps backward error, the DPOTRF problems in FP64."""
    probs = make_batch(120, 7, 8, 200)
    keep = _run(gblib, probs, flags=BT.GB_BATCH_EMULATED | BT.GB_BATCH_MIXED)
    check(probs, orc, mixed=True)
    del keep


def test_emulated_dgemm_exact_on_integers_and_special_tiles(gblib, gb_clean):
    """Integer operands are represented exactly by the 7 digit slices, so the
    emulated batch DGEMM equals the exact product; a tile holding NaN/Inf
    and a K beyond 4096 take the FP64 loop and propagate IEEE values."""
    torch = pytest.importorskip("torch")
    probs = []
    for i, (m, n, k) in enumerate([(70, 45, 300), (33, 64, 64), (96, 96, 17)]):
        A = np.asfortranarray(W.randint(40 + i, (m, k), -(2 ** 20), 2 ** 20).astype(np.float64))
        B = np.asfortranarray(W.randint(50 + i, (k, n), -255, 255).astype(np.float64))
        probs.append(dict(type=BT.GB_BATCH_DGEMM, m=m, n=n, k=k, ta="N", tb="N", alpha=1.0,
                          beta=0.0, A=A, B=B, C=np.zeros((m, n), order="F")))
    A = W.uniform(60, (40, 50))
    A[3, 7] = np.nan
    A[30, 1] = np.inf
    probs.append(dict(type=BT.GB_BATCH_DGEMM, m=40, n=20, k=50, ta="N", tb="N", alpha=1.0,
                      beta=0.0, A=A, B=W.uniform(61, (50, 20)), C=np.zeros((40, 20), order="F")))
    probs.append(dict(type=BT.GB_BATCH_DGEMM, m=24, n=16, k=5000, ta="T", tb="N", alpha=0.5,
                      beta=0.0, A=W.uniform(62, (5000, 24)), B=W.uniform(63, (5000, 16)),
                      C=np.zeros((24, 16), order="F")))
    keep = _run(gblib, probs, flags=BT.GB_BATCH_EMULATED)
    for p in probs[:3]:
        exact = (p["A"].astype(object) @ p["B"].astype(object)).astype(np.float64)
        assert np.array_equal(fetch(p["dC"]), exact)
    p = probs[3]
    ref = p["A"] @ p["B"]
    got = fetch(p["dC"])
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(np.isinf(got), np.isinf(ref))
    fin = np.isfinite(ref)
    assert np.abs(got[fin] - ref[fin]).max() <= 1e-12 * np.abs(ref[fin]).max()
    p = probs[4]
    ref = 0.5 * p["A"].T @ p["B"]
    assert np.abs(fetch(p["dC"]) - ref).max() <= 1e-11 * np.abs(ref).max()
    del keep
