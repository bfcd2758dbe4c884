"""The LU entry point that allocates no device memory.

gb_dgetrf_noalloc_dev serves callers that cannot let a library allocate
(their own arena owns HBM, a fixed memory budget, or no tolerance for the
latency of cudaMalloc/cudaFree).  Its scratch lives in a fixed device array
inside the library.  Here it is called through the C ABI twice in a row, on
different matrices, and each result is checked against the allocating entry
point gb_dgetrf_dev on the same input: identical pivots, identical info, and
LU factors within the tolerance the LU tests use.  The file runs last so a
failure here comes after every other test has run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from openblas_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GB_ERR_UNSUPPORTED = 6


def _factor(gblib, fn, A, stream_ptr):
    torch = pytest.importorskip("torch")
    m, n = A.shape
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()   # column-major buffer
    dp = torch.zeros(min(m, n), dtype=torch.int32, device="cuda")
    di = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    if fn == "noalloc":
        st = gblib.gb_dgetrf_noalloc_dev(m, n, dA.data_ptr(), m, dp.data_ptr(), di.data_ptr(),
                                         C.c_void_p(stream_ptr))
    else:
        st = gblib.gb_dgetrf_dev(m, n, dA.data_ptr(), m, dp.data_ptr(), di.data_ptr())
    assert st == 0
    torch.cuda.synchronize()
    assert gblib.gb_synchronize() == 0
    return dA.cpu().numpy().T, dp.cpu().numpy(), int(di.item())


def test_noalloc_lu_matches_allocating_entry(gblib):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.Stream()
    gblib.gb_set_stream(C.c_void_p(stream.cuda_stream))
    try:
        for seed, (m, n) in ((401, (1500, 1500)), (402, (2100, 1700))):
            A = W.uniform(seed, (m, n))
            A[:, 37] *= 0.0 if seed == 402 else 1.0  # second call: an exact zero pivot
            LUn, pn, in_ = _factor(gblib, "noalloc", A, stream.cuda_stream)
            LUa, pa, ia = _factor(gblib, "alloc", A, stream.cuda_stream)
            assert in_ == ia
            assert np.array_equal(pn, pa)
            assert np.max(np.abs(LUn - LUa)) <= 1e-12 * max(1.0, np.abs(LUa).max())
    finally:
        gblib.gb_set_stream(None)


def test_noalloc_rejects_sizes_beyond_its_scratch(gblib):
    m = 524288 + 1
    dummy = C.c_void_p(0)
    st = gblib.gb_dgetrf_noalloc_dev(m, 4, dummy, m, dummy, dummy, dummy)
    assert st == GB_ERR_UNSUPPORTED
    gblib.gb_clear_error()
