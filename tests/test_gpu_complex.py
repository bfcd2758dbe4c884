"""Complex GEMM on the GPU: ZGEMM/CGEMM (4M, one real GEMM on the
[Ar -Ai; Ai Ar] embedding) and ZGEMM3M/CGEMM3M (three real products),
interface/gemm.c compiled with COMPLEX.

OpenBLAS golden outputs for every op pair N/T/R/C and the alpha/beta edge
values (beta = 0 over NaN, alpha = 0, k = 0); larger shapes against the
oracle on both FP64 engines (native DFMA, emulated Ozaki) and both FP32
engines (tensor-core bf16x3 when the real product has m, n >= 1024, FFMA
below); CBLAS row-major and conjugate forms; the device entries.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import zgemm_ratio
from openblas_gb300 import workloads as W
from tests.golden import gen_golden as GG

pytestmark = pytest.mark.gpu


def _eps(dt):
    return float(np.finfo(np.float32 if dt == np.complex64 else np.float64).eps)


@pytest.mark.parametrize("name,dt", GG.ZGEMM_ROUTINES)
def test_golden(golden, F, gb_clean, name, dt):
    eps = _eps(dt)
    for idx, (m, n, k, ta, tb, al, be) in enumerate(GG.zgemm_cases()):
        A, B, Cm = GG.complex_operands(idx, m, n, k, ta, tb, dt)
        C0 = Cm.copy(order="F")
        if be == 0:
            Cm[:m, :n] = np.nan
        getattr(F, name)(ta, tb, m, n, k, al, A, A.shape[0], B, B.shape[0], be, Cm, Cm.shape[0])
        ref = golden[f"{name}_{idx}"]
        r = zgemm_ratio(Cm, ref, A, B, C0, m, n, k, ta, tb, al, be, eps,
                        normwise=name.endswith("3m"))
        assert r <= 4 * (k + 2), (name, idx, m, n, k, ta, tb, r)
        assert np.array_equal(Cm[m:], C0[m:])


def _operands(seed, m, n, k, ta, tb, dt, pad=0):
    ra, ca = (m, k) if ta in "NR" else (k, m)
    rb, cb = (k, n) if tb in "NR" else (n, k)

    def cplx(s, r, c):
        X = W.uniform(s, (r + pad, c)) + 1j * W.uniform(s + 1, (r + pad, c))
        return np.asfortranarray(X.astype(dt))
    return cplx(seed, ra, ca), cplx(seed + 2, rb, cb), cplx(seed + 4, m + pad, n)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("ta,tb", [("N", "N"), ("C", "T"), ("R", "C"), ("T", "R")])
def test_zgemm_vs_oracle(orc, F, gblib, gb_clean, mode, ta, tb):
    """Both FP64 engines behind ZGEMM; the emulated one is bounded normwise."""
    m, n, k = 700, 600, 500
    A, B, Cm = _operands(14000, m, n, k, ta, tb, np.complex128, pad=3)
    C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
    al, be = 0.8 - 0.6j, -0.5 + 0.25j
    gblib.gb_set_dgemm_mode(mode)
    try:
        F.zgemm(ta, tb, m, n, k, al, A, A.shape[0], B, B.shape[0], be, Cm, Cm.shape[0])
    finally:
        gblib.gb_set_dgemm_mode(0)
    orc.zgemm(ta, tb, m, n, k, al, A, A.shape[0], B, B.shape[0], be, Co, Co.shape[0])
    r = zgemm_ratio(Cm, Co, A, B, C0, m, n, k, ta, tb, al, be, _eps(np.complex128),
                    normwise=mode == 1)
    assert r <= 2 * (k + 2), r
    assert np.array_equal(Cm[m:], C0[m:])


def test_zgemm_emulated_several_k_segments(orc, F, gblib, gb_clean):
    """The 4M embedding doubles K (2k = 5000 here): the emulated engine runs
    it as two K segments accumulating into the product; normwise bound."""
    m, n, k = 300, 260, 2500
    A, B, Cm = _operands(14050, m, n, k, "C", "N", np.complex128)
    C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
    al, be = 0.6 + 0.8j, 0.25 - 1.0j
    gblib.gb_set_dgemm_mode(1)
    try:
        F.zgemm("C", "N", m, n, k, al, A, k, B, k, be, Cm, m)
    finally:
        gblib.gb_set_dgemm_mode(0)
    orc.zgemm("C", "N", m, n, k, al, A, k, B, k, be, Co, m)
    r = zgemm_ratio(Cm, Co, A, B, C0, m, n, k, "C", "N", al, be, _eps(np.complex128),
                    normwise=True)
    assert r <= 2 * (k + 2), r


@pytest.mark.parametrize("ta,tb", [("N", "T"), ("C", "N")])
def test_zgemm3m_vs_oracle(orc, F, gb_clean, ta, tb):
    m, n, k = 650, 520, 390
    A, B, Cm = _operands(14100, m, n, k, ta, tb, np.complex128)
    C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
    al, be = 1.25 + 0.5j, 0.0
    F.zgemm3m(ta, tb, m, n, k, al, A, m if ta in "NR" else k, B, k if tb in "NR" else n, be,
              Cm, m)
    orc.zgemm3m(ta, tb, m, n, k, al, A, m if ta in "NR" else k, B, k if tb in "NR" else n, be,
                Co, m)
    r = zgemm_ratio(Cm, Co, A, B, C0, m, n, k, ta, tb, al, be, _eps(np.complex128),
                    normwise=True)
    assert r <= 2 * (k + 2), r


@pytest.mark.parametrize("name", ["cgemm", "cgemm3m"])
@pytest.mark.parametrize("m,n,k", [(1100, 1100, 300), (200, 170, 90)])
def test_cgemm_vs_oracle(orc, F, gb_clean, name, m, n, k):
    """FP32 complex: the bf16x3 tensor-core engine at the larger shape (the
    real products are 2m x n x 2k for 4M, m x n x k for 3M), FFMA at the
    smaller."""
    ta, tb = "C", "N"
    A, B, Cm = _operands(14200, m, n, k, ta, tb, np.complex64)
    C0, Co = Cm.copy(order="F"), Cm.copy(order="F")
    al, be = 0.5 + 1.0j, 1.0 - 0.5j
    getattr(F, name)(ta, tb, m, n, k, al, A, k, B, k, be, Cm, m)
    getattr(orc, name)(ta, tb, m, n, k, al, A, k, B, k, be, Co, m)
    r = zgemm_ratio(Cm, Co, A, B, C0, m, n, k, ta, tb, al, be, _eps(np.complex64),
                    normwise=name.endswith("3m"))
    assert r <= 2 * (k + 2), r


def test_cblas_row_major_and_conj(gblib, gb_clean):
    """Row-major calls with ConjNoTrans/ConjTrans equal numpy on the same
    row-major data (interface/gemm.c:423-471 operand swap)."""
    from openblas_gb300 import cblas
    ns = cblas()
    m, n, k = 37, 29, 23
    A = np.ascontiguousarray(W.uniform(14300, (m, k)) + 1j * W.uniform(14301, (m, k)))
    B = np.ascontiguousarray(W.uniform(14302, (n, k)) + 1j * W.uniform(14303, (n, k)))
    Cr = np.ascontiguousarray(W.uniform(14304, (m, n)) + 1j * W.uniform(14305, (m, n)))
    al = np.array([0.3, -0.7])
    be = np.array([1.1, 0.2])
    ref = (0.3 - 0.7j) * (A.conj() @ B.conj().T) + (1.1 + 0.2j) * Cr
    for fn in ("cblas_zgemm", "cblas_zgemm3m"):
        Cg = Cr.copy()
        getattr(ns, fn)(101, 114, 113, m, n, k, al.ctypes.data, A.ctypes.data, k,
                        B.ctypes.data, k, be.ctypes.data, Cg.ctypes.data, n)
        assert np.abs(Cg - ref).max() <= 64 * k * np.finfo(np.float64).eps * np.abs(ref).max()
    A32, B32, C32 = (x.astype(np.complex64) for x in (A, B, Cr))
    al32, be32 = al.astype(np.float32), be.astype(np.float32)  # kept alive across the call
    for fn in ("cblas_cgemm", "cblas_cgemm3m"):
        Cg = C32.copy()
        getattr(ns, fn)(101, 114, 113, m, n, k, al32.ctypes.data, A32.ctypes.data, k,
                        B32.ctypes.data, k, be32.ctypes.data, Cg.ctypes.data, n)
        assert np.abs(Cg - ref).max() <= 64 * k * np.finfo(np.float32).eps * np.abs(ref).max()


def test_device_entries(orc, gblib, gb_clean):
    torch = pytest.importorskip("torch")
    m, n, k = 300, 260, 210
    A, B, Cm = _operands(14400, m, n, k, "T", "N", np.complex128)
    al = np.array([1.5, 0.5])
    be = np.array([0.0, 0.0])
    for fn in ("gb_zgemm_dev", "gb_zgemm3m_dev"):
        dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
        dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
        dC = torch.full((n, m), complex("nan"), dtype=torch.complex128).cuda()
        assert getattr(gblib, fn)(b"T", b"N", m, n, k, al.ctypes.data, dA.data_ptr(), k,
                                  dB.data_ptr(), k, be.ctypes.data, dC.data_ptr(), m) == 0
        assert gblib.gb_synchronize() == 0
        got = dC.cpu().numpy().T
        Co = np.zeros((m, n), np.complex128, order="F")
        orc.zgemm("T", "N", m, n, k, 1.5 + 0.5j, A, k, B, k, 0.0, Co, m)
        r = zgemm_ratio(got, Co, A, B, Cm, m, n, k, "T", "N", 1.5 + 0.5j, 0.0,
                        _eps(np.complex128), normwise=True)
        assert r <= 2 * (k + 2), (fn, r)
