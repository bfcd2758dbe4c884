"""DGETRF and DGESV at the LU benchmark's sizes, on the GPU.

* DGETRF on A = uniform(-1, 1) of order N in {8192, 16384, 32768} (seed
  7100 + N): the pivot vector must equal OpenBLAS's dgetrf_ on the same matrix
  (fixtures made by tests/golden/gen_golden_large.py; the pivot rule is the
  IAMAX first maximum of lapack/getf2/getf2_k.c:97-116) and the scaled
  residual ||PA - LU||_1 / (n eps ||A||_1) must be <= 10, with native FP64 and
  with emulated-FP64 trailing updates.
* Mixed-precision DGESV (gb_dsgesv_dev) on A = U diag(logspace(0, -kappa)) V^T
  at N = 8192, kappa in {1e4, 1e8, 1e12}: backward error
  ||b - Ax||_inf / (||A||_inf ||x||_inf + ||b||_inf) <= n eps, whatever path
  (refinement, GMRES-IR or the FP64-accurate fallback) finishes the solve.

The matrices are generated on the device with the same counter-based
generator as the fixtures (openblas_gb300.workloads.uniform_device).  The
residual products run on the library's emulated-FP64 GEMM in column blocks.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import pytest

from conftest import EPS
from openblas_gb300 import workloads as W

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PIVOTS = os.path.join(HERE, "golden", "getrf_pivots_large.npz")


@pytest.fixture(scope="module")
def pivots():
    return np.load(PIVOTS)


def _perm_from_ipiv(ipiv):
    """Row order of P*A for 1-based LAPACK interchanges applied in sequence."""
    perm = np.arange(ipiv.size)
    for i, p in enumerate(ipiv - 1):
        if p != i:
            perm[i], perm[p] = perm[p], perm[i]
    return perm


def lu_residual_device(gblib, torch, A0t, LUt, ipiv, nb=4096):
    """||PA - LU||_1 / (n eps ||A||_1) for square n x n matrices held column-major
    as the transposed torch tensors A0t, LUt (row j of the tensor is column j)."""
    n = A0t.shape[0]
    perm = torch.from_numpy(_perm_from_ipiv(ipiv)).to(A0t.device)
    Rt = A0t[:, perm].contiguous()                     # P*A, column-major
    Lt = torch.triu(LUt, 1)                            # strict lower L, column-major
    Lt.diagonal().fill_(1.0)
    Ut = torch.tril(LUt)                               # U, column-major
    torch.cuda.synchronize()
    for j0 in range(0, n, nb):
        j1 = min(n, j0 + nb)
        # R(:, j0:j1) -= L(:, 0:j1) * U(0:j1, j0:j1)  (U is zero below row j1)
        st = gblib.gb_dgemm_emulated_dev(b"N", b"N", n, j1 - j0, j1, -1.0, Lt.data_ptr(), n,
                                         Ut[j0:j1].data_ptr(), n, 1.0, Rt[j0:j1].data_ptr(), n,
                                         0)
        assert st == 0
    assert gblib.gb_synchronize() == 0
    torch.cuda.synchronize()
    rn = Rt.abs().sum(dim=1).max().item()
    an = A0t.abs().sum(dim=1).max().item()
    del Rt, Lt, Ut
    return rn / (n * EPS * an)


@pytest.mark.parametrize("mode", ["native", "emulated"])
@pytest.mark.parametrize("n", [8192, 16384, 32768])
def test_dgetrf_pivots_match_openblas_at_scale(gblib, pivots, gb_clean, n, mode):
    torch = pytest.importorskip("torch")
    if mode == "native" and n == 32768:
        pytest.skip("native FP64 LU at 32768 takes ~20 s; covered by the emulated-update run")
    A0t = W.uniform_device(7100 + n, (n, n), "cuda")
    LUt = A0t.clone()
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    gblib.gb_set_dgemm_mode(0 if mode == "native" else 1)
    try:
        st = gblib.gb_dgetrf_dev(n, n, LUt.data_ptr(), n, ipiv.data_ptr(), info.data_ptr())
        assert st == 0
        assert gblib.gb_synchronize() == 0
    finally:
        gblib.gb_set_dgemm_mode(0)
    torch.cuda.synchronize()
    p = ipiv.cpu().numpy()
    assert int(info.item()) == int(pivots[f"info{n}"])
    gold = pivots[f"piv{n}"]
    diff = np.flatnonzero(p != gold)
    assert diff.size == 0, f"{diff.size} pivots differ, first at column {diff[:5]}"
    assert lu_residual_device(gblib, torch, A0t, LUt, p) <= 10


def _ill_conditioned_device(torch, seed, n, kappa_exp):
    """U diag(logspace(0, -kappa)) V^T with U, V the Q factors of seeded
    uniform matrices (as workloads.ill_conditioned, QR on the device)."""
    U, _ = torch.linalg.qr(W.uniform_device(seed, (n, n), "cuda").T)
    V, _ = torch.linalg.qr(W.uniform_device(seed + 1, (n, n), "cuda").T)
    s = torch.logspace(0.0, -float(kappa_exp), n, dtype=torch.float64, device="cuda")
    A = (U * s) @ V.T
    del U, V
    return A.T.contiguous()        # column-major buffer of A


@pytest.mark.parametrize("kappa_exp", [4, 8, 12])
def test_dsgesv_ill_conditioned_8192(gblib, gb_clean, kappa_exp):
    torch = pytest.importorskip("torch")
    n = 8192
    At = _ill_conditioned_device(torch, 8800 + kappa_exp, n, kappa_exp)
    A0t = At.clone()
    b = W.uniform_device(8810 + kappa_exp, (n,), "cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    it, info = C.c_int(0), C.c_int(0)
    torch.cuda.synchronize()
    st = gblib.gb_dsgesv_dev(n, 1, At.data_ptr(), n, ipiv.data_ptr(), b.data_ptr(), n,
                             x.data_ptr(), n, C.byref(it), C.byref(info))
    assert st == 0 and info.value == 0
    assert gblib.gb_synchronize() == 0
    A = A0t.T                                            # row-major view of A
    r = (b - A @ x).abs().max().item()
    den = A.abs().sum(dim=1).max().item() * x.abs().max().item() + b.abs().max().item()
    berr = r / den
    print(f"kappa=1e{kappa_exp}: ITER={it.value} berr={berr / EPS:.2f} eps")
    assert berr <= n * EPS, (it.value, berr / EPS)


def _cluster_spectrum_device(torch, seed, n, kappa_exp, nsmall=8):
    """U diag(s) V^T with s = 1 except the last `nsmall` values, 10^-kappa."""
    U, _ = torch.linalg.qr(W.uniform_device(seed, (n, n), "cuda").T)
    V, _ = torch.linalg.qr(W.uniform_device(seed + 1, (n, n), "cuda").T)
    s = torch.ones(n, dtype=torch.float64, device="cuda")
    s[-nsmall:] = 10.0 ** -kappa_exp
    A = (U * s) @ V.T
    del U, V
    return A.T.contiguous()


@pytest.mark.parametrize("kappa_exp", [8, 12])
def test_gmres_ir_finishes_when_few_directions_are_small(gblib, gb_clean, kappa_exp):
    """N = 4096, kappa = 1e8 / 1e12 with 8 tiny singular values: the FP32
    factors precondition every other direction, so GMRES-IR (ITER = 100 +
    GMRES iterations) finishes the solve to n*eps backward error without the
    FP64-accurate fallback."""
    torch = pytest.importorskip("torch")
    n = 4096
    At = _cluster_spectrum_device(torch, 8900 + kappa_exp, n, kappa_exp)
    A0t = At.clone()
    b = W.uniform_device(8910 + kappa_exp, (n,), "cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    it, info = C.c_int(0), C.c_int(0)
    torch.cuda.synchronize()
    st = gblib.gb_dsgesv_dev(n, 1, At.data_ptr(), n, ipiv.data_ptr(), b.data_ptr(), n,
                             x.data_ptr(), n, C.byref(it), C.byref(info))
    assert st == 0 and info.value == 0
    assert gblib.gb_synchronize() == 0
    assert 100 <= it.value < 200, it.value
    A = A0t.T
    r = (b - A @ x).abs().max().item()
    den = A.abs().sum(dim=1).max().item() * x.abs().max().item() + b.abs().max().item()
    assert r / den <= n * EPS
