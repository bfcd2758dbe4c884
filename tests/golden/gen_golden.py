"""Generate golden vectors from an OpenBLAS build for the hot-path routines.

The OpenBLAS used is the one bundled with scipy (libscipy_openblas, OpenBLAS
0.3.31.dev, DYNAMIC_ARCH; its exported ABI carries a ``scipy_`` prefix).  It
is called through ctypes with exactly the Fortran-77 ABI the drop-in library
exports (dgemm_, zgemm_, cgemm_, zgemm3m_, cgemm3m_, dtrsm_, dtrmm_, dsyrk_, dsyr2k_, dgemmt_, dgetrf_, dgetrs_,
dgesv_, dpotrf_, dpotrs_, dlaswp_, dsgesv_, dsposv_, sgetrf_).  The routines on this path are the same algorithms as the
0.3.28.dev reference tree (interface/, driver/level3, lapack/).

Inputs come from openblas_gb300.workloads (seeded counter-based splitmix64)
and are regenerated by the tests; only the outputs are stored.  Run from the
repository root:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import ctypes
import glob
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from openblas_gb300 import abi  # noqa: E402
from openblas_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "openblas_golden.npz")


def openblas():
    import scipy
    cands = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs",
                                   "libscipy_openblas*.so"))
    if not cands:
        raise SystemExit("scipy's bundled OpenBLAS not found")
    lib = ctypes.CDLL(cands[0])
    lib.scipy_openblas_get_config.restype = ctypes.c_char_p
    cfg = lib.scipy_openblas_get_config().decode()
    return abi.Fortran(abi.bind(lib, "scipy_")), cfg


# --------------------------------------------------------------------------
# case tables (shared with tests/test_oracle_golden.py)
# --------------------------------------------------------------------------
GEMM_SHAPES = [(1, 1, 1), (2, 2, 2), (3, 5, 7), (7, 3, 9), (35, 35, 35), (64, 33, 48), (9, 35, 1),
               (5, 7, 0)]
GEMM_AB = [(0.0, 0.0), (0.0, 1.3), (1.0, 0.0), (1.0, 1.0), (0.7, 1.3), (1.5, 0.5)]
TRSM_SHAPES = [(1, 1), (5, 3), (35, 9)]
TRSM_ALPHA = [0.0, 1.0, 0.7]
SYRK_SHAPES = [(1, 1), (7, 3), (35, 35), (33, 64)]
SYRK_AB = [(0.0, 0.0), (1.0, 0.0), (0.7, 1.3)]
GETRF_SHAPES = [(1, 1), (2, 2), (7, 7), (64, 64), (100, 100), (257, 257), (100, 60), (60, 100)]
GETRF_PIV_ONLY = [512, 1024]
POTRF_N = [1, 7, 64, 200]
LASWP_CASES = [(7, 1, 9, 1), (7, 3, 9, 1), (7, 1, 9, -1), (5, 2, 8, 2), (5, 2, 8, -2)]
DSGESV_CASES = [(50, 1), (200, 3)]
GEMMT_SHAPES = [(1, 1), (7, 3), (35, 35), (33, 64)]
GEMMT_AB = [(0.0, 1.3), (1.0, 0.0), (0.7, 1.3)]


def trmm_operands(idx, side, uplo, m, n):
    na = m if side == "L" else n
    A = W.uniform(9000 + idx, (na, na))   # both triangles filled: only one may be read
    B = W.uniform(9500 + idx, (m, n))
    return A, B


# complex GEMM: every op pair (N, T, R, C) on two shapes, edge shapes on two
# op pairs; alpha/beta as (re, im)
ZGEMM_SHAPES = [(3, 5, 7), (35, 9, 33)]
ZGEMM_AB = [(1.0 + 0.0j, 0.0j), (0.7 - 0.4j, 0.3 + 1.2j)]
ZGEMM_EDGE_SHAPES = [(1, 1, 1), (5, 7, 0)]
ZGEMM_EDGE_AB = [(0.0j, 0.0j), (0.0j, 1.5 - 0.5j), (1.0 + 0.0j, 1.0 + 0.0j), (0.7 - 0.4j, 0.0j)]
ZGEMM_ROUTINES = [("zgemm", np.complex128), ("cgemm", np.complex64),
                  ("zgemm3m", np.complex128), ("cgemm3m", np.complex64)]


def zgemm_cases():
    """(m, n, k, ta, tb, alpha, beta) in the order of the stored outputs."""
    cases = []
    for (m, n, k) in ZGEMM_SHAPES:
        for ta in "NTRC":
            for tb in "NTRC":
                for (al, be) in ZGEMM_AB:
                    cases.append((m, n, k, ta, tb, al, be))
    for (m, n, k) in ZGEMM_EDGE_SHAPES:
        for (ta, tb) in (("N", "N"), ("C", "T")):
            for (al, be) in ZGEMM_EDGE_AB:
                cases.append((m, n, k, ta, tb, al, be))
    return cases


def complex_operands(idx, m, n, k, ta, tb, dtype):
    """A, B, C (complex, column-major, ld = rows + 2) for case idx; C holds NaN
    when beta = 0 (it must be overwritten, not propagated)."""
    ra, ca = (m, k) if ta in "NR" else (k, m)
    rb, cb = (k, n) if tb in "NR" else (n, k)

    def cplx(seed, r, c):
        X = W.uniform(seed, (r + 2, c)) + 1j * W.uniform(seed + 50000, (r + 2, c))
        return np.asfortranarray(X.astype(dtype))
    return cplx(11000 + idx, ra, ca), cplx(12000 + idx, rb, cb), cplx(13000 + idx, m, n)


DPOTRS_CASES = [("L", 40, 1), ("U", 40, 5), ("L", 129, 3), ("U", 129, 1)]
DSPOSV_CASES = [("L", 60, 1), ("U", 200, 3), ("L", 150, 2)]
C1 = dict(m=1024, n=1024, k=1024, alpha=1.5, beta=0.5)


def gemm_case_seed(idx: int) -> int:
    return 1000 + 17 * idx


def main():
    ob, cfg = openblas()
    g = {"openblas_config": np.array(cfg)}
    # ---- DGEMM (interface/gemm.c) -------------------------------------
    idx = 0
    for (m, n, k) in GEMM_SHAPES:
        for (alpha, beta) in GEMM_AB:
            for ta in "NT":
                for tb in "NT":
                    A, B, Cm = W.gemm_operands(gemm_case_seed(idx), m, n, k, ta, tb, pad=3)
                    if beta == 0.0:
                        Cm[:m, :n] = np.nan  # beta==0 must overwrite, not propagate
                    ob.dgemm(ta, tb, m, n, k, alpha, A, A.shape[0], B, B.shape[0], beta, Cm,
                             Cm.shape[0])
                    g[f"dgemm_{idx}"] = Cm[:m, :n].copy(order="F")
                    idx += 1
    # C1: 1024^3 NN alpha=1.5 beta=0.5 -- column sums + a strided sample
    A, B, Cm = W.gemm_operands(42, C1["m"], C1["n"], C1["k"])
    ob.dgemm("N", "N", 1024, 1024, 1024, 1.5, A, 1024, B, 1024, 0.5, Cm, 1024)
    g["dgemm_c1_colsum"] = Cm.sum(axis=0)
    g["dgemm_c1_sample"] = Cm[::37, ::41].copy(order="F")
    # ---- SGEMM --------------------------------------------------------
    A, B, Cm = W.gemm_operands(77, 35, 33, 64, "N", "T", dtype=np.float32)
    ob.sgemm("N", "T", 35, 33, 64, 0.7, A, 35, B, 33, 1.3, Cm, 35)
    g["sgemm_0"] = Cm.copy(order="F")
    # ---- DTRSM (interface/trsm.c) ------------------------------------
    idx = 0
    for (m, n) in TRSM_SHAPES:
        for side in "LR":
            for uplo in "UL":
                for ta in "NT":
                    for diag in "UN":
                        for alpha in TRSM_ALPHA:
                            na = m if side == "L" else n
                            A = W.trsm_lower(3000 + idx, na)
                            if uplo == "U":
                                A = np.asfortranarray(A.T)
                            B = W.uniform(4000 + idx, (m, n))
                            ob.dtrsm(side, uplo, ta, diag, m, n, alpha, A, na, B, m)
                            g[f"dtrsm_{idx}"] = B
                            idx += 1
    # ---- DSYRK (interface/syrk.c) ------------------------------------
    idx = 0
    for (n, k) in SYRK_SHAPES:
        for uplo in "UL":
            for tr in "NT":
                for (alpha, beta) in SYRK_AB:
                    ra, ca = (n, k) if tr == "N" else (k, n)
                    A = W.uniform(5000 + idx, (ra, ca))
                    Cm = W.uniform(6000 + idx, (n, n))
                    ob.dsyrk(uplo, tr, n, k, alpha, A, ra, beta, Cm, n)
                    g[f"dsyrk_{idx}"] = Cm
                    idx += 1
    # ---- DTRMM (interface/trsm.c built as TRMM) -----------------------
    idx = 0
    for (m, n) in TRSM_SHAPES:
        for side in "LR":
            for uplo in "UL":
                for ta in "NT":
                    for diag in "UN":
                        for alpha in TRSM_ALPHA:
                            A, B = trmm_operands(idx, side, uplo, m, n)
                            ob.dtrmm(side, uplo, ta, diag, m, n, alpha, A, A.shape[0], B, m)
                            g[f"dtrmm_{idx}"] = B
                            idx += 1
    # ---- DSYR2K (interface/syr2k.c) ----------------------------------
    idx = 0
    for (n, k) in SYRK_SHAPES:
        for uplo in "UL":
            for tr in "NT":
                for (alpha, beta) in SYRK_AB:
                    ra, ca = (n, k) if tr == "N" else (k, n)
                    A = W.uniform(9700 + idx, (ra, ca))
                    B = W.uniform(9800 + idx, (ra, ca))
                    Cm = W.uniform(9900 + idx, (n, n))
                    ob.dsyr2k(uplo, tr, n, k, alpha, A, ra, B, ra, beta, Cm, n)
                    g[f"dsyr2k_{idx}"] = Cm
                    idx += 1
    # ---- DGEMMT (interface/gemmt.c) ----------------------------------
    idx = 0
    for (m, k) in GEMMT_SHAPES:
        for uplo in "UL":
            for ta in "NT":
                for tb in "NT":
                    for (alpha, beta) in GEMMT_AB:
                        A = W.uniform(10000 + idx, (m, k) if ta == "N" else (k, m))
                        B = W.uniform(10100 + idx, (k, m) if tb == "N" else (m, k))
                        Cm = W.uniform(10200 + idx, (m, m))
                        ob.dgemmt(uplo, ta, tb, m, k, alpha, A, A.shape[0], B, B.shape[0],
                                  beta, Cm, m)
                        g[f"dgemmt_{idx}"] = Cm
                        idx += 1
    # ---- ZGEMM / CGEMM / ZGEMM3M / CGEMM3M (interface/gemm.c, COMPLEX) --
    for name, dt in ZGEMM_ROUTINES:
        for idx, (m, n, k, ta, tb, al, be) in enumerate(zgemm_cases()):
            A, B, Cm = complex_operands(idx, m, n, k, ta, tb, dt)
            if be == 0:
                Cm[:m, :n] = np.nan
            getattr(ob, name)(ta, tb, m, n, k, al, A, A.shape[0], B, B.shape[0], be, Cm,
                              Cm.shape[0])
            g[f"{name}_{idx}"] = Cm[:m, :n].copy(order="F")
    # ---- DGETRF / DGETRS / DGESV (interface/lapack) -------------------
    for idx, (m, n) in enumerate(GETRF_SHAPES):
        A = W.uniform(7000 + idx, (m, n))
        ipiv = np.zeros(min(m, n), np.int32)
        info = ob.dgetrf(m, n, A, m, ipiv)
        g[f"dgetrf_{idx}_ipiv"], g[f"dgetrf_{idx}_info"] = ipiv, info
        if m * n <= 100 * 100:
            g[f"dgetrf_{idx}_lu"] = A
    for n in GETRF_PIV_ONLY:
        A = W.uniform(7100 + n, (n, n))
        ipiv = np.zeros(n, np.int32)
        g[f"dgetrf_piv{n}_info"] = ob.dgetrf(n, n, A, n, ipiv)
        g[f"dgetrf_piv{n}"] = ipiv
    # singular: exact zero column 3 and a zero row makes a later pivot zero
    A = W.uniform(7200, (9, 9))
    A[:, 3] = 0.0
    ipiv = np.zeros(9, np.int32)
    g["dgetrf_sing_info"] = ob.dgetrf(9, 9, A, 9, ipiv)
    g["dgetrf_sing_ipiv"], g["dgetrf_sing_lu"] = ipiv, A
    for t, trans in enumerate("NT"):
        for nrhs in (1, 5):
            n = 64
            A = W.uniform(7300 + t, (n, n))
            ipiv = np.zeros(n, np.int32)
            ob.dgetrf(n, n, A, n, ipiv)
            B = W.uniform(7400 + nrhs, (n, nrhs))
            ob.dgetrs(trans, n, nrhs, A, n, ipiv, B, n)
            g[f"dgetrs_{trans}_{nrhs}"] = B
    A = W.uniform(7500, (100, 100))
    B = W.uniform(7501, (100, 3))
    ipiv = np.zeros(100, np.int32)
    g["dgesv_info"] = ob.dgesv(100, 3, A, 100, ipiv, B, 100)
    g["dgesv_x"], g["dgesv_ipiv"] = B, ipiv
    # ---- DPOTRF ------------------------------------------------------
    for n in POTRF_N:
        for uplo in "LU":
            A = W.spd(8000 + n, n)
            g[f"dpotrf_{uplo}_{n}_info"] = ob.dpotrf(uplo, n, A, n)
            g[f"dpotrf_{uplo}_{n}"] = A
    A = W.spd(8100, 20)
    A[11, 11] = -1.0  # not positive definite at step 12
    g["dpotrf_npd_info"] = ob.dpotrf("L", 20, A, 20)
    g["dpotrf_npd"] = A
    # ---- DLASWP ------------------------------------------------------
    for idx, (n, k1, k2, incx) in enumerate(LASWP_CASES):
        rows = 12
        A = W.uniform(8200 + idx, (rows, n))
        npiv = k1 - 1 + (k2 - k1 + 1) * abs(incx)
        ipiv = (W.randint(8300 + idx, (npiv,), 1, rows)).astype(np.int32)
        ob.dlaswp(n, A, rows, k1, k2, ipiv, incx)
        g[f"dlaswp_{idx}_ipiv"], g[f"dlaswp_{idx}"] = ipiv, A
    # ---- DSGESV (lapack-netlib/SRC/dsgesv.f) ------------------------
    for idx, (n, nrhs) in enumerate(DSGESV_CASES):
        A = W.uniform(8400 + idx, (n, n))
        B = W.uniform(8500 + idx, (n, nrhs))
        X = np.zeros((n, nrhs), order="F")
        ipiv = np.zeros(n, np.int32)
        work = np.zeros((n, nrhs), order="F")
        swork = np.zeros(n * (n + nrhs), np.float32)
        info, it = ob.dsgesv(n, nrhs, A, n, ipiv, B, n, X, n, work, swork)
        g[f"dsgesv_{idx}_x"], g[f"dsgesv_{idx}_iter"] = X, it
        g[f"dsgesv_{idx}_ipiv"], g[f"dsgesv_{idx}_info"] = ipiv, info
    # ill-conditioned: FP32 refinement cannot converge -> FP64 fallback
    n = 60
    A = W.ill_conditioned(8600, n, 12)
    B = W.uniform(8601, (n, 1))
    X = np.zeros((n, 1), order="F")
    ipiv = np.zeros(n, np.int32)
    work = np.zeros((n, 1), order="F")
    swork = np.zeros(n * (n + 1), np.float32)
    info, it = ob.dsgesv(n, 1, A, n, ipiv, B, n, X, n, work, swork)
    g["dsgesv_ill_x"], g["dsgesv_ill_iter"], g["dsgesv_ill_ipiv"] = X, it, ipiv
    # ---- DPOTRS (lapack-netlib/SRC/dpotrs.f) ------------------------
    for idx, (uplo, n, nrhs) in enumerate(DPOTRS_CASES):
        A = W.spd(8800 + idx, n)
        assert ob.dpotrf(uplo, n, A, n) == 0
        B = W.uniform(8810 + idx, (n, nrhs))
        g[f"dpotrs_{idx}_info"] = ob.dpotrs(uplo, n, nrhs, A, n, B, n)
        g[f"dpotrs_{idx}_x"] = B
    # ---- DSPOSV (lapack-netlib/SRC/dsposv.f) ------------------------
    for idx, (uplo, n, nrhs) in enumerate(DSPOSV_CASES):
        A = W.spd(8900 + idx, n)
        B = W.uniform(8910 + idx, (n, nrhs))
        X = np.zeros((n, nrhs), order="F")
        work = np.zeros((n, nrhs), order="F")
        swork = np.zeros(n * (n + nrhs), np.float32)
        info, it = ob.dsposv(uplo, n, nrhs, A, n, B, n, X, n, work, swork)
        g[f"dsposv_{idx}_x"], g[f"dsposv_{idx}_iter"], g[f"dsposv_{idx}_info"] = X, it, info
    # ill-conditioned SPD: the FP32 Cholesky fails or refinement stalls -> FP64
    n = 60
    A = W.spd_ill_conditioned(8920, n, 10)
    B = W.uniform(8921, (n, 1))
    X = np.zeros((n, 1), order="F")
    work = np.zeros((n, 1), order="F")
    swork = np.zeros(n * (n + 1), np.float32)
    info, it = ob.dsposv("L", n, 1, A, n, B, n, X, n, work, swork)
    g["dsposv_ill_x"], g["dsposv_ill_iter"], g["dsposv_ill_info"] = X, it, info
    # not positive definite: FP32 and FP64 Cholesky both fail, info = column
    n = 30
    A = W.spd(8930, n)
    A[17, 17] = -1.0
    B = W.uniform(8931, (n, 1))
    X = np.zeros((n, 1), order="F")
    info, it = ob.dsposv("L", n, 1, A, n, B, n, X, n, work[:n], swork)
    g["dsposv_npd_iter"], g["dsposv_npd_info"] = it, info
    # ---- SGETRF pivots (FP32 factorisation of the mixed solver) -------
    for n in (128, 256):
        A = W.uniform(8700 + n, (n, n)).astype(np.float32)
        ipiv = np.zeros(n, np.int32)
        g[f"sgetrf_{n}_info"] = ob.sgetrf(n, n, A, n, ipiv)
        g[f"sgetrf_{n}_ipiv"] = ipiv
        if n <= 128:
            g[f"sgetrf_{n}_lu"] = A
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB) from {cfg}")


if __name__ == "__main__":
    main()
