"""GPU parity of the LAPACK entry points: pivots identical to OpenBLAS's,
scaled residuals ||PA-LU||/(n eps ||A||) <= 10, Cholesky and solve residuals,
info codes on singular / non-SPD inputs."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from conftest import EPS

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import gen_golden as GG  # noqa: E402

from openblas_gb300 import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu


def lu_residual(A0, LU, ipiv):
    m, n = A0.shape
    mn = min(m, n)
    L = np.tril(LU[:, :mn], -1) + np.eye(m, mn)
    U = np.triu(LU[:mn, :])
    PA = A0.copy(order="F")
    for i in range(mn):
        p = ipiv[i] - 1
        if p != i:
            PA[[i, p], :] = PA[[p, i], :]
    nrm = np.abs(A0).sum(axis=0).max()
    return np.abs(PA - L @ U).sum(axis=0).max() / (max(m, n) * EPS * nrm)


def test_dgetrf_golden(golden, F, gb_clean):
    for idx, (m, n) in enumerate(GG.GETRF_SHAPES):
        A0 = W.uniform(7000 + idx, (m, n))
        A = A0.copy(order="F")
        ipiv = np.zeros(min(m, n), np.int32)
        info = F.dgetrf(m, n, A, m, ipiv)
        assert info == int(golden[f"dgetrf_{idx}_info"])
        assert np.array_equal(ipiv, golden[f"dgetrf_{idx}_ipiv"]), (m, n)
        if f"dgetrf_{idx}_lu" in golden:
            assert np.max(np.abs(A - golden[f"dgetrf_{idx}_lu"])) < 1e-11
        assert lu_residual(A0, A, ipiv) <= 10
    for n in GG.GETRF_PIV_ONLY:
        A0 = W.uniform(7100 + n, (n, n))
        A = A0.copy(order="F")
        ipiv = np.zeros(n, np.int32)
        assert F.dgetrf(n, n, A, n, ipiv) == 0
        assert np.array_equal(ipiv, golden[f"dgetrf_piv{n}"])
        assert lu_residual(A0, A, ipiv) <= 10


def test_dgetrf_singular(golden, F, gb_clean):
    A = W.uniform(7200, (9, 9))
    A[:, 3] = 0.0
    ipiv = np.zeros(9, np.int32)
    assert F.dgetrf(9, 9, A, 9, ipiv) == 4
    assert np.array_equal(ipiv, golden["dgetrf_sing_ipiv"])
    assert np.max(np.abs(A - golden["dgetrf_sing_lu"])) < 1e-12


@pytest.mark.parametrize("m,n", [(3000, 3000), (2500, 1800), (1200, 2100)])
def test_dgetrf_vs_oracle(orc, F, gb_clean, m, n):
    A0 = W.uniform(7600 + m, (m, n))
    A, Ao = A0.copy(order="F"), A0.copy(order="F")
    p, po = np.zeros(min(m, n), np.int32), np.zeros(min(m, n), np.int32)
    assert F.dgetrf(m, n, A, m, p) == orc.dgetrf(m, n, Ao, m, po) == 0
    assert np.array_equal(p, po)
    assert np.max(np.abs(A - Ao)) <= 1e-9 * np.abs(Ao).max()
    assert lu_residual(A0, A, p) <= 10


@pytest.mark.parametrize("n", [700, 2600])
def test_dgetrf_emulated_updates(orc, F, gblib, gb_clean, n):
    """DGETRF whose trailing updates run on the emulated-FP64 GEMM (DGEMM
    mode 'emulated'): same pivots as the oracle, FP64-level scaled residual."""
    A0 = W.uniform(7700 + n, (n, n))
    A, Ao = A0.copy(order="F"), A0.copy(order="F")
    p, po = np.zeros(n, np.int32), np.zeros(n, np.int32)
    gblib.gb_set_dgemm_mode(1)
    try:
        assert F.dgetrf(n, n, A, n, p) == 0
    finally:
        gblib.gb_set_dgemm_mode(0)
    assert orc.dgetrf(n, n, Ao, n, po) == 0
    assert np.array_equal(p, po)
    assert lu_residual(A0, A, p) <= 10


def test_dgetrf_tiny_pivot_rule(orc, F, gb_clean):
    """A subnormal pivot is recorded but neither swapped nor divided by
    (getf2_k.c:103-116); the GPU panel follows the same rule."""
    n = 40
    A0 = W.uniform(77, (n, n)) * 1e-310
    A0[:, 5:] = W.uniform(78, (n, n - 5))
    A, Ao = A0.copy(order="F"), A0.copy(order="F")
    p, po = np.zeros(n, np.int32), np.zeros(n, np.int32)
    assert F.dgetrf(n, n, A, n, p) == orc.dgetrf(n, n, Ao, n, po)
    assert np.array_equal(p, po)
    assert np.max(np.abs(A - Ao)) <= 1e-9 * np.abs(Ao).max()


@pytest.mark.parametrize("m,n,where", [
    (300, 300, "column"),   # column 5 all NaN: every later pivot search sees NaN at row j
    (300, 300, "entry"),    # one NaN below the diagonal: skipped, then met at its own step
    (12000, 40, "entry"),   # taller than one FP64 cluster (8192 rows): grid-wide panel kernel
])
def test_dgetrf_nan_pivot_rule(orc, F, gb_clean, m, n, where):
    """IAMAX order with NaN (getf2_k.c pivot search): the running maximum starts
    at |a_jj| and only a larger value replaces it, so a NaN elsewhere never wins
    and a NaN at row j keeps row j.  Pivots stay in range and match the oracle."""
    A0 = W.uniform(7900 + m, (m, n))
    if where == "column":
        A0[:, 5] = np.nan
    else:
        A0[11, 3] = np.nan
    A, Ao = A0.copy(order="F"), A0.copy(order="F")
    p, po = np.zeros(min(m, n), np.int32), np.zeros(min(m, n), np.int32)
    assert F.dgetrf(m, n, A, m, p) == orc.dgetrf(m, n, Ao, m, po)
    assert p.min() >= 1 and p.max() <= m
    assert np.array_equal(p, po)
    fin = np.isfinite(Ao)
    assert np.array_equal(fin, np.isfinite(A))
    assert np.max(np.abs(A[fin] - Ao[fin]), initial=0.0) <= 1e-9 * np.abs(Ao[fin]).max()


def test_dgetrs_dgesv(golden, F, gb_clean):
    for t, trans in enumerate("NT"):
        for nrhs in (1, 5):
            n = 64
            A = W.uniform(7300 + t, (n, n))
            ipiv = np.zeros(n, np.int32)
            F.dgetrf(n, n, A, n, ipiv)
            B = W.uniform(7400 + nrhs, (n, nrhs))
            assert F.dgetrs(trans, n, nrhs, A, n, ipiv, B, n) == 0
            ref = golden[f"dgetrs_{trans}_{nrhs}"]
            assert np.max(np.abs(B - ref)) <= 1e-10 * max(1, np.abs(ref).max())
    A = W.uniform(7500, (100, 100))
    B = W.uniform(7501, (100, 3))
    ipiv = np.zeros(100, np.int32)
    assert F.dgesv(100, 3, A, 100, ipiv, B, 100) == 0
    assert np.array_equal(ipiv, golden["dgesv_ipiv"])
    assert np.max(np.abs(B - golden["dgesv_x"])) <= 1e-10 * np.abs(B).max()


@pytest.mark.parametrize("nrhs", [1, 64])
def test_dgesv_residual(F, gb_clean, nrhs):
    n = 2000
    A0 = W.uniform(3, (n, n))
    B0 = W.uniform(4, (n, nrhs))
    A, X = A0.copy(order="F"), B0.copy(order="F")
    ipiv = np.zeros(n, np.int32)
    assert F.dgesv(n, nrhs, A, n, ipiv, X, n) == 0
    r = np.abs(B0 - A0 @ X).sum(axis=0).max()
    scaled = r / (np.abs(A0).sum(axis=0).max() * np.abs(X).sum(axis=0).max() * EPS * n)
    assert scaled <= 10


def test_dgesv_singular_skips_solve(F, gb_clean):
    n = 10
    A = W.uniform(9, (n, n))
    A[:, 6] = 0.0
    B = W.uniform(10, (n, 2))
    B0 = B.copy(order="F")
    ipiv = np.zeros(n, np.int32)
    assert F.dgesv(n, 2, A, n, ipiv, B, n) == 7
    assert np.array_equal(B, B0)  # gesv.c:131: getrs only when info == 0


def test_dpotrf_golden(golden, F, gb_clean):
    for n in GG.POTRF_N:
        for uplo in "LU":
            A0 = W.spd(8000 + n, n)
            A = A0.copy(order="F")
            assert F.dpotrf(uplo, n, A, n) == 0
            tri = np.tril if uplo == "L" else np.triu
            assert np.max(np.abs(tri(A) - tri(golden[f"dpotrf_{uplo}_{n}"]))) < 1e-12
            other = (lambda X: np.triu(X, 1)) if uplo == "L" else (lambda X: np.tril(X, -1))
            assert np.array_equal(other(A), other(A0))


def test_dpotrf_not_positive_definite(golden, F, gb_clean):
    A = W.spd(8100, 20)
    A[11, 11] = -1.0
    assert F.dpotrf("L", 20, A, 20) == 12
    ref = golden["dpotrf_npd"]
    assert np.max(np.abs(np.tril(A)[:, :12] - np.tril(ref)[:, :12])) < 1e-12
    n = 300  # failure inside a later diagonal block
    A = W.spd(8101, n)
    A[200, 200] = -5.0
    assert F.dpotrf("U", n, A, n) == 201


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_dpotrf_residual(F, gb_clean, uplo):
    n = 1500
    A0 = W.spd(8200, n)
    A = A0.copy(order="F")
    assert F.dpotrf(uplo, n, A, n) == 0
    Lf = np.tril(A) if uplo == "L" else np.triu(A).T
    r = np.abs(A0 - Lf @ Lf.T).sum(axis=0).max() / (n * EPS * np.abs(A0).sum(axis=0).max())
    assert r <= 10


@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("n", [1100, 2600])
def test_dpotrf_emulated_updates(F, gblib, gb_clean, uplo, n):
    """DPOTRF whose rank-256 trailing updates run on the emulated-FP64 GEMM
    restricted to the triangle (DGEMM mode 'emulated'): the other triangle is
    bit-for-bit untouched and the scaled residual stays at the FP64 bound."""
    A0 = W.spd(8300 + n, n)
    A = A0.copy(order="F")
    gblib.gb_set_dgemm_mode(1)
    try:
        assert F.dpotrf(uplo, n, A, n) == 0
    finally:
        gblib.gb_set_dgemm_mode(0)
    other = (lambda X: np.triu(X, 1)) if uplo == "L" else (lambda X: np.tril(X, -1))
    assert np.array_equal(other(A), other(A0))
    Lf = np.tril(A) if uplo == "L" else np.triu(A).T
    r = np.abs(A0 - Lf @ Lf.T).sum(axis=0).max() / (n * EPS * np.abs(A0).sum(axis=0).max())
    assert r <= 10


@pytest.mark.parametrize("mode", [0, 1])
def test_dpotrf_failure_in_later_block(orc, F, gblib, gb_clean, mode):
    """A non-positive pivot past the first 256-wide block: info matches the
    oracle.  After a failure LAPACK leaves the rest of A unspecified and the
    reference's state depends on its blocking, so the comparison covers what
    every blocking has completed: the columns before the failing 32-wide
    diagonal step (530 lies in [512, 544)), and that step's rows of the
    columns before the failing one."""
    n = 700
    A0 = W.spd(8400, n)
    A0[530, 530] = -3.0
    A, Ao = A0.copy(order="F"), A0.copy(order="F")
    gblib.gb_set_dgemm_mode(mode)
    try:
        info = F.dpotrf("L", n, A, n)
    finally:
        gblib.gb_set_dgemm_mode(0)
    assert info == orc.dpotrf("L", n, Ao, n) == 531
    tol = 1e-10 * np.abs(np.tril(Ao)).max()
    assert np.max(np.abs(np.tril(A)[:, :512] - np.tril(Ao)[:, :512])) <= tol
    assert np.max(np.abs(np.tril(A)[512:544, 512:530] - np.tril(Ao)[512:544, 512:530])) <= tol


def test_dlaswp_golden(golden, F, gb_clean):
    for idx, (n, k1, k2, incx) in enumerate(GG.LASWP_CASES):
        rows = 12
        A = W.uniform(8200 + idx, (rows, n))
        ipiv = golden[f"dlaswp_{idx}_ipiv"].astype(np.int32)
        F.dlaswp(n, A, rows, k1, k2, ipiv, incx)
        assert np.array_equal(A, golden[f"dlaswp_{idx}"]), (n, k1, k2, incx)


@pytest.mark.parametrize("rows,n,k1,k2,incx", [
    (3000, 500, 5, 260, 1),      # 256 interchanges: one fused launch
    (3000, 300, 100, 300, -1),   # reverse order
    (1000, 64, 1, 100, 3),       # strided pivots
    (3000, 200, 1, 700, 1),      # long sequence: planned gather/scatter path
    (3000, 40, 1, 700, -2),      # long sequence, reverse strided: per-column path
])
def test_dlaswp_random_pivots(orc, F, gb_clean, rows, n, k1, k2, incx):
    """Random pivot rows above, inside and below the window, with repeats."""
    A = W.uniform(8600 + k2, (rows, n))
    npiv = k1 - 1 + (k2 - k1 + 1) * abs(incx)
    ipiv = W.randint(8700 + k2, (npiv,), 1, rows).astype(np.int32)  # inclusive
    ref = A.copy(order="F")
    orc.dlaswp(n, ref, rows, k1, k2, ipiv, incx)
    F.dlaswp(n, A, rows, k1, k2, ipiv, incx)
    assert np.array_equal(A, ref)


@pytest.mark.parametrize("incx", [1, 2, -2, 3])
def test_dlaswp_reads_only_the_pivots_it_uses(orc, F, gb_clean, incx):
    """Row i (k1..k2) takes its pivot from ipiv[(k1-1) + (i-k1)*|incx|], so a
    caller may pass exactly (k1-1) + (k2-k1)*|incx| + 1 entries.  Here the
    array is a view whose next element is a poison value.  A longer read
    would take it as a pivot row far outside A."""
    import openblas_gb300 as gb
    rows, n, k1, k2 = 50, 7, 3, 9
    need = (k1 - 1) + (k2 - k1) * abs(incx) + 1
    buf = np.full(need + 4, 10 ** 9, np.int32)
    buf[:need] = W.randint(8800 + need, (need,), 1, rows).astype(np.int32)
    ipiv = buf[:need]
    A = W.uniform(8900 + need, (rows, n))
    ref = A.copy(order="F")
    orc.dlaswp(n, ref, rows, k1, k2, ipiv, incx)
    F.dlaswp(n, A, rows, k1, k2, ipiv, incx)
    assert gb.last_error(gb_clean)[0] == 0
    assert np.array_equal(A, ref)


def _sgetrf_dev(gblib, A32):
    torch = pytest.importorskip("torch")
    m, n = A32.shape
    dA = torch.from_numpy(np.ascontiguousarray(A32.T)).cuda()
    dp = torch.zeros(min(m, n), dtype=torch.int32, device="cuda")
    di = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert gblib.gb_sgetrf_dev(m, n, dA.data_ptr(), m, dp.data_ptr(), di.data_ptr()) == 0
    assert gblib.gb_synchronize() == 0
    return dA.cpu().numpy().T.copy(order="F"), dp.cpu().numpy(), int(di.item())


@pytest.mark.parametrize("n", [256, 1500])
def test_sgetrf_vs_oracle(orc, gblib, gb_clean, n):
    """The FP32 factorisation behind the mixed solver: pivots identical to the
    oracle's sgetrf and FP32-level scaled residual."""
    A0 = np.asfortranarray(W.uniform(8700 + n, (n, n)).astype(np.float32))
    LU, piv, info = _sgetrf_dev(gblib, A0)
    Ao = A0.copy(order="F")
    po = np.zeros(n, np.int32)
    assert info == orc.sgetrf(n, n, Ao, n, po) == 0
    if n <= 256:
        assert np.array_equal(piv, po)
    # At larger n a near-tie at FP32 precision can flip one pivot between two
    # valid summation orders; the factorisation bar is then the residual.
    feps = float(np.finfo(np.float32).eps)
    L = np.tril(LU.astype(np.float64), -1) + np.eye(n)
    U = np.triu(LU.astype(np.float64))
    PA = _apply_piv(A0, piv)
    r = np.abs(PA - L @ U).sum(axis=0).max() / (n * feps * np.abs(A0).sum(axis=0).max())
    assert r <= 10, r
    if np.array_equal(piv, po):
        rel = np.abs(LU - Ao).max() / np.abs(Ao).max()
        assert rel <= 1e-3, rel


def _apply_piv(A, piv):
    P = A.astype(np.float64).copy(order="F")
    for i, p in enumerate(piv):
        if p - 1 != i:
            P[[i, p - 1], :] = P[[p - 1, i], :]
    return P


@pytest.mark.parametrize("m,n", [(8192, 40), (12000, 40), (16384, 96)])
def test_dgetrf_tall_panels(orc, F, gb_clean, m, n):
    """FP64 panels at the edge of the cluster kernel (8192 rows: one row per
    thread of a 16-CTA cluster) and past it (the grid-wide kernel); pivots
    identical to the oracle."""
    A0 = W.uniform(8100 + m + n, (m, n))
    A, Ao = A0.copy(order="F"), A0.copy(order="F")
    p, po = np.zeros(n, np.int32), np.zeros(n, np.int32)
    assert F.dgetrf(m, n, A, m, p) == orc.dgetrf(m, n, Ao, m, po) == 0
    assert np.array_equal(p, po)
    assert np.max(np.abs(A - Ao)) <= 1e-9 * np.abs(Ao).max()


@pytest.mark.parametrize("m,n", [(16384, 40), (20000, 64), (30000, 40)])
def test_sgetrf_tall_panels(orc, gblib, gb_clean, m, n):
    """FP32 panels of the mixed solver's LU at the edge of the cluster kernel
    (16384 rows: two register rows per thread) and past it (the grid-wide
    kernel).  Pivots match the oracle's sgetrf (or, on an FP32 near-tie, the
    factorisation has an FP32-level residual)."""
    A0 = np.asfortranarray(W.uniform(8200 + m + n, (m, n)).astype(np.float32))
    LU, piv, info = _sgetrf_dev(gblib, A0)
    Ao = A0.copy(order="F")
    po = np.zeros(n, np.int32)
    assert info == orc.sgetrf(m, n, Ao, m, po) == 0
    assert piv.min() >= 1 and piv.max() <= m
    if np.array_equal(piv, po):
        assert np.abs(LU - Ao).max() <= 1e-4 * np.abs(Ao).max()
    feps = float(np.finfo(np.float32).eps)
    L = np.tril(LU.astype(np.float64), -1)[:, :n] + np.eye(m, n)
    U = np.triu(LU.astype(np.float64)[:n, :])
    PA = _apply_piv(A0, piv)
    r = np.abs(PA - L @ U).sum(axis=0).max() / (n * feps * np.abs(A0).sum(axis=0).max())
    assert r <= 10, r


_PLAIN_LU = r'''
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
import openblas_gb300 as gb
from openblas_gb300 import workloads as W
lib = gb.load()
n, dt, out = int(sys.argv[2]), sys.argv[3], sys.argv[4]
A = W.uniform_device(7800 + n, (n, n), "cuda")
if dt == "f32":
    A = A.float()
ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
info = torch.zeros(1, dtype=torch.int32, device="cuda")
torch.cuda.synchronize()   # the library works on its own stream
f = lib.gb_sgetrf_dev if dt == "f32" else lib.gb_dgetrf_dev
assert f(n, n, A.data_ptr(), n, ipiv.data_ptr(), info.data_ptr()) == 0
assert lib.gb_synchronize() == 0
np.savez(out, lu=A.cpu().numpy(), ipiv=ipiv.cpu().numpy(), info=info.cpu().numpy())
'''


@pytest.mark.parametrize("n,dt", [(3000, "f64"), (5000, "f32")])
def test_lookahead_lu_equals_plain_blocked(gblib, gb_clean, tmp_path, n, dt):
    """The look-ahead LU (next panel factored on a second stream while the
    trailing update runs) performs every element's operations in the same
    order as the plain blocked loop, so factors, pivots and info are
    identical bit for bit; the plain loop runs in a child process with
    GB_LU_LOOKAHEAD=0.  Look-ahead is used with trailing updates on the FMA
    units, so the FP32 case selects them (GB_SGEMM_MODE=simt)."""
    import subprocess
    torch = pytest.importorskip("torch")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    script = tmp_path / "plain_lu.py"
    script.write_text(_PLAIN_LU)
    out = tmp_path / "plain.npz"
    env = dict(os.environ, GB_LU_LOOKAHEAD="0", GB_SGEMM_MODE="simt")
    subprocess.run([sys.executable, str(script), root, str(n), dt, str(out)], env=env,
                   check=True, timeout=600)
    ref = np.load(out)
    A = W.uniform_device(7800 + n, (n, n), "cuda")
    if dt == "f32":
        A = A.float()
    ipiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()   # the library works on its own stream
    f = gblib.gb_sgetrf_dev if dt == "f32" else gblib.gb_dgetrf_dev
    gblib.gb_set_sgemm_mode(1)
    try:
        assert f(n, n, A.data_ptr(), n, ipiv.data_ptr(), info.data_ptr()) == 0
        assert gblib.gb_synchronize() == 0
    finally:
        gblib.gb_set_sgemm_mode(0)
    assert np.array_equal(ipiv.cpu().numpy(), ref["ipiv"])
    assert int(info.item()) == int(ref["info"][0])
    assert np.array_equal(A.cpu().numpy(), ref["lu"])
