"""Concurrent calls from host threads, after the reference's
cpp_thread_test/dgemm_thread_safety.cpp.

Several host threads call the blocking cblas_dgemm at the same time, each on
its own matrices.  ctypes releases the interpreter lock during the call, so
the calls overlap.  Each thread has its own stream and error state, and the
one-time setup per device runs under a lock.  As in the reference test, every
concurrent result must equal the result of the same call made alone; here the
comparison is bit for bit, since both come from the same kernel on the same
data."""
from __future__ import annotations

import threading

import numpy as np
import pytest

import openblas_gb300 as gb
from openblas_gb300 import abi
from openblas_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _dgemm(ns, A, B, C, n):
    ns.cblas_dgemm(abi.CblasColMajor, abi.CblasNoTrans, abi.CblasNoTrans, n, n, n, 1.0,
                   A.ctypes.data, n, B.ctypes.data, n, 0.1, C.ctypes.data, n)


def test_concurrent_cblas_dgemm_matches_serial(gblib, gb_clean):
    ns = gb.cblas()
    n, nthreads, rounds = 384, 8, 4
    mats = [(W.uniform(9000 + 3 * t, (n, n)), W.uniform(9001 + 3 * t, (n, n)),
             W.uniform(9002 + 3 * t, (n, n))) for t in range(nthreads)]
    serial = []
    for A, B, C0 in mats:
        C = C0.copy(order="F")
        _dgemm(ns, A, B, C, n)
        serial.append(C)
    failures = []
    start = threading.Barrier(nthreads)

    def worker(t):
        A, B, C0 = mats[t]
        start.wait()
        for r in range(rounds):
            C = C0.copy(order="F")
            _dgemm(ns, A, B, C, n)
            if not np.array_equal(C, serial[t]):
                failures.append((t, r, float(np.abs(C - serial[t]).max())))
            status, msg = gb.last_error(gblib)
            if status != 0:
                failures.append((t, r, msg))

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(nthreads)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not failures, failures[:4]
