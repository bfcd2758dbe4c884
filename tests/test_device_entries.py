"""Device-pointer entry points (gb_*_dev) on a machine without a GPU.

Each one checks its arguments before it touches CUDA: a bad argument reaches
xerbla with the position the matching Fortran routine uses (interface/gemm.c,
trsm.c, syrk.c, syr2k.c, gemmt.c; lapack/getrf.c, getrs.c, potrf.c and the
LAPACK dsgesv.f/dsposv.f/dpotrs.f argument lists) and the call returns
GB_ERR_INVALID_VALUE.  A valid call on a machine without a usable device
fails loudly with GB_ERR_NO_DEVICE: there is no CPU fallback.  Pointers are
null throughout; no entry may dereference one before those checks."""
from __future__ import annotations

import ctypes as C

import pytest

from openblas_gb300 import _lib

GB_ERR_INVALID_VALUE = 1
GB_ERR_NO_DEVICE = 3


@pytest.fixture(scope="module")
def L():
    return _lib.load()


def _gemm(fn, ta=b"N", tb=b"N", m=4, n=4, k=4, lda=4, ldb=4, ldc=4):
    return lambda L: getattr(L, fn)(ta, tb, m, n, k, 1.0, None, lda, None, ldb, 0.0, None, ldc)


def _emu(ta=b"N", tb=b"N", m=4, n=4, k=4, lda=4, ldb=4, ldc=4):
    return lambda L: L.gb_dgemm_emulated_dev(ta, tb, m, n, k, 1.0, None, lda, None, ldb, 0.0,
                                             None, ldc, 0)


def _zgemm(fn, ta=b"N", tb=b"N", m=4, n=4, k=4, lda=4, ldb=4, ldc=4):
    return lambda L: getattr(L, fn)(ta, tb, m, n, k, None, None, lda, None, ldb, None, None, ldc)


def _tri(fn, side=b"L", uplo=b"L", ta=b"N", diag=b"N", m=4, n=4, lda=4, ldb=4):
    return lambda L: getattr(L, fn)(side, uplo, ta, diag, m, n, 1.0, None, lda, None, ldb)


def _syrk(uplo=b"L", tr=b"N", n=4, k=4, lda=4, ldc=4):
    return lambda L: L.gb_dsyrk_dev(uplo, tr, n, k, 1.0, None, lda, 0.0, None, ldc)


def _syr2k(uplo=b"L", tr=b"N", n=4, k=4, lda=4, ldb=4, ldc=4):
    return lambda L: L.gb_dsyr2k_dev(uplo, tr, n, k, 1.0, None, lda, None, ldb, 0.0, None, ldc)


def _gemmt(uplo=b"L", ta=b"N", tb=b"N", m=4, k=4, lda=4, ldb=4, ldc=4):
    return lambda L: L.gb_dgemmt_dev(uplo, ta, tb, m, k, 1.0, None, lda, None, ldb, 0.0, None, ldc)


def _getrf(fn, m=4, n=4, lda=4):
    return lambda L: getattr(L, fn)(m, n, None, lda, None, None)


def _noalloc(m=4, n=4, lda=4):
    return lambda L: L.gb_dgetrf_noalloc_dev(m, n, None, lda, None, None, None)


def _getrs(fn, tr=b"N", n=4, nrhs=1, lda=4, ldb=4):
    return lambda L: getattr(L, fn)(tr, n, nrhs, None, lda, None, None, ldb)


def _potrf(uplo=b"L", n=4, lda=4):
    return lambda L: L.gb_dpotrf_dev(uplo, n, None, lda, None)


def _potrs(uplo=b"L", n=4, nrhs=1, lda=4, ldb=4):
    return lambda L: L.gb_dpotrs_dev(uplo, n, nrhs, None, lda, None, ldb)


def _sgesv(n=4, nrhs=1, lda=4, ldb=4, ldx=4):
    return lambda L: L.gb_dsgesv_dev(n, nrhs, None, lda, None, None, ldb, None, ldx, None, None)


def _sposv(uplo=b"L", n=4, nrhs=1, lda=4, ldb=4, ldx=4):
    return lambda L: L.gb_dsposv_dev(uplo, n, nrhs, None, lda, None, ldb, None, ldx, None, None)


BAD = [
    ("dgemm-transa", _gemm("gb_dgemm_dev", ta=b"X"), "DGEMM", 1),
    ("dgemm-k", _gemm("gb_dgemm_dev", k=-1), "DGEMM", 5),
    ("dgemm-ldb", _gemm("gb_dgemm_dev", tb=b"T", n=5), "DGEMM", 10),
    ("dgemm-native-ldc", _gemm("gb_dgemm_native_dev", ldc=3), "DGEMM", 13),
    ("dgemm-emulated-lda", _emu(lda=3), "DGEMM", 8),
    ("sgemm-n", _gemm("gb_sgemm_dev", n=-1), "SGEMM", 4),
    ("zgemm-transb", _zgemm("gb_zgemm_dev", tb=b"X"), "ZGEMM", 2),
    ("cgemm-lda", _zgemm("gb_cgemm_dev", ta=b"C", k=5, lda=4), "CGEMM", 8),
    ("zgemm3m-m", _zgemm("gb_zgemm3m_dev", m=-1), "ZGEMM3M", 3),
    ("cgemm3m-ldc", _zgemm("gb_cgemm3m_dev", ldc=2), "CGEMM3M", 13),
    ("dtrsm-side", _tri("gb_dtrsm_dev", side=b"X"), "DTRSM", 1),
    ("dtrsm-lda", _tri("gb_dtrsm_dev", side=b"R", n=5, lda=4, ldb=4), "DTRSM", 9),
    ("dtrmm-diag", _tri("gb_dtrmm_dev", diag=b"X"), "DTRMM", 4),
    ("dtrmm-ldb", _tri("gb_dtrmm_dev", m=5, lda=5, ldb=4), "DTRMM", 11),
    ("dsyrk-trans", _syrk(tr=b"X"), "DSYRK", 2),
    ("dsyrk-ldc", _syrk(ldc=3), "DSYRK", 10),
    ("dsyr2k-ldb", _syr2k(tr=b"T", k=5, lda=5, ldb=4), "DSYR2K", 9),
    ("dgemmt-uplo", _gemmt(uplo=b"X"), "DGEMMT", 1),
    ("dgemmt-ldb", _gemmt(tb=b"T", m=5, lda=5, ldb=4, ldc=5), "DGEMMT", 10),
    ("dgetrf-lda", _getrf("gb_dgetrf_dev", lda=3), "DGETRF", 4),
    ("sgetrf-m", _getrf("gb_sgetrf_dev", m=-1), "SGETRF", 1),
    ("dgetrf-noalloc-n", _noalloc(n=-1), "DGETRF", 2),
    ("dgetrs-trans", _getrs("gb_dgetrs_dev", tr=b"X"), "DGETRS", 1),
    ("sgetrs-ldb", _getrs("gb_sgetrs_dev", ldb=3), "SGETRS", 8),
    ("dpotrf-uplo", _potrf(uplo=b"X"), "DPOTRF", 1),
    ("dpotrs-lda", _potrs(lda=3), "DPOTRS", 5),
    ("dsgesv-nrhs", _sgesv(nrhs=-1), "DSGESV", 2),
    ("dsgesv-ldx", _sgesv(ldx=3), "DSGESV", 9),
    ("dsposv-ldb", _sposv(ldb=3), "DSPOSV", 7),
]


@pytest.mark.parametrize("case,call,name,pos", BAD, ids=[b[0] for b in BAD])
def test_device_entry_argument_errors(L, case, call, name, pos):
    L.gb_clear_error()
    assert call(L) == GB_ERR_INVALID_VALUE
    got_name, got_pos = _lib.last_xerbla(L)
    assert (got_name.strip(), got_pos) == (name, pos)


GOOD = [
    ("dgemm", _gemm("gb_dgemm_dev")),
    ("dgemm-native", _gemm("gb_dgemm_native_dev")),
    ("dgemm-emulated", _emu()),
    ("sgemm", _gemm("gb_sgemm_dev")),
    ("zgemm", _zgemm("gb_zgemm_dev")),
    ("cgemm3m", _zgemm("gb_cgemm3m_dev")),
    ("dtrsm", _tri("gb_dtrsm_dev")),
    ("dtrmm", _tri("gb_dtrmm_dev")),
    ("dsyrk", _syrk()),
    ("dsyr2k", _syr2k()),
    ("dgemmt", _gemmt()),
    ("dgetrf", _getrf("gb_dgetrf_dev")),
    ("sgetrf", _getrf("gb_sgetrf_dev")),
    ("dgetrf-noalloc", _noalloc()),
    ("dgetrs", _getrs("gb_dgetrs_dev")),
    ("dlaswp", lambda L: L.gb_dlaswp_dev(4, None, 4, 1, 4, None, 1)),
    ("dpotrf", _potrf()),
    ("dpotrs", _potrs()),
    ("dsgesv", _sgesv()),
    ("dsposv", _sposv()),
]


def _cuda_usable() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # noqa: BLE001 - torch absent means no device either
        return False


@pytest.mark.skipif(_cuda_usable(), reason="a CUDA device is present")
@pytest.mark.parametrize("case,call", GOOD, ids=[g[0] for g in GOOD])
def test_device_entry_without_device_fails_loudly(L, case, call):
    L.gb_clear_error()
    assert call(L) == GB_ERR_NO_DEVICE
    st, msg = _lib.last_error(L)
    assert st == GB_ERR_NO_DEVICE and msg


@pytest.mark.skipif(_cuda_usable(), reason="a CUDA device is present")
def test_host_entries_without_device_report_and_leave_outputs():
    """The host-pointer (Fortran) entries have no status to return: without a
    device they record GB_ERR_NO_DEVICE and leave the caller's arrays as they
    were -- nothing is computed on the CPU instead."""
    import numpy as np

    import openblas_gb300 as gb
    L = gb.load()
    F = gb.fortran()
    A = np.asfortranarray(np.arange(16.0).reshape(4, 4))
    C = np.full((4, 4), 7.0, order="F")
    L.gb_clear_error()
    F.dgemm("N", "N", 4, 4, 4, 1.0, A, 4, A, 4, 0.0, C, 4)
    assert gb.last_error(L)[0] == GB_ERR_NO_DEVICE
    assert np.all(C == 7.0)
    L.gb_clear_error()
    piv = np.zeros(4, np.int32)
    A0 = A.copy(order="F")
    F.dgetrf(4, 4, A, 4, piv)
    assert gb.last_error(L)[0] == GB_ERR_NO_DEVICE
    assert np.array_equal(A, A0)


def test_error_state_is_per_thread(L):
    """Each host thread has its own error record: threads that raise different
    argument errors at the same time each read back their own (ctypes drops
    the interpreter lock during the call, so the calls overlap)."""
    import threading

    cases = [(dict(ta=b"X"), 1), (dict(tb=b"X"), 2), (dict(m=-1), 3), (dict(n=-1), 4),
             (dict(k=-1), 5), (dict(lda=3), 8), (dict(ldb=3), 10), (dict(ldc=3), 13)]
    errors = []
    start = threading.Barrier(len(cases))

    def worker(kw, pos):
        call = _gemm("gb_dgemm_dev", **kw)
        start.wait()
        for _ in range(300):
            L.gb_clear_error()
            if call(L) != GB_ERR_INVALID_VALUE or _lib.last_xerbla(L) != ("DGEMM ", pos):
                errors.append((pos, _lib.last_xerbla(L)))
                return

    threads = [threading.Thread(target=worker, args=c) for c in cases]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:5]


def test_argument_error_wins_over_missing_device(L):
    """The argument check comes first even when no device could be used, so the
    xerbla position is the same on every machine."""
    L.gb_clear_error()
    assert _gemm("gb_dgemm_dev", m=-1)(L) == GB_ERR_INVALID_VALUE
    assert _lib.last_xerbla(L)[1] == 3


def test_forked_child_reports_no_device_with_the_reason(gblib):
    """A child forked after the parent called into the library cannot use the
    parent's CUDA context (memory.c's pthread_atfork re-initialisation has no
    GPU counterpart): every entry point then returns GB_ERR_NO_DEVICE and the
    message names fork, before any CUDA call."""
    import ctypes as C
    import os
    import openblas_gb300 as gb
    dummy = C.c_void_p(0)
    gblib.gb_dgetrf_dev(0, 0, dummy, 1, dummy, dummy)  # the parent touches the library
    gblib.gb_clear_error()
    r, w = os.pipe()
    pid = os.fork()
    if pid == 0:  # child: report the status and message through the pipe, then leave
        os.close(r)
        try:
            st = gblib.gb_dgetrf_dev(4, 4, dummy, 4, dummy, dummy)
            code, msg = gb.last_error(gblib)
            os.write(w, f"{st}|{code}|{msg}".encode())
        finally:
            os._exit(0)
    os.close(w)
    out = b""
    while True:
        chunk = os.read(r, 4096)
        if not chunk:
            break
        out += chunk
    os.close(r)
    os.waitpid(pid, 0)
    st, code, msg = out.decode().split("|", 2)
    assert int(st) == 3 and int(code) == 3, out
    assert "fork" in msg
