"""ctypes view of the grouped-batch API (gb_batch_* in include/gbblas.h)."""
from __future__ import annotations

import ctypes as C

GB_BATCH_DGEMM, GB_BATCH_DGESV, GB_BATCH_DPOTRF = 0, 1, 2
GB_BATCH_MIXED = 1
GB_BATCH_EMULATED = 2


class Problem(C.Structure):
    _fields_ = [("type", C.c_int), ("m", C.c_int), ("n", C.c_int), ("k", C.c_int),
                ("transa", C.c_char), ("transb", C.c_char), ("uplo", C.c_char), ("pad", C.c_char),
                ("alpha", C.c_double), ("beta", C.c_double),
                ("A", C.c_void_p), ("B", C.c_void_p), ("C", C.c_void_p),
                ("lda", C.c_int), ("ldb", C.c_int), ("ldc", C.c_int),
                ("info", C.c_void_p)]


def bind(lib: C.CDLL) -> None:
    lib.gb_batch_plan_create.restype = C.c_void_p
    lib.gb_batch_plan_create.argtypes = [C.POINTER(Problem), C.c_int, C.c_int]
    for name in ("gb_batch_plan_tune", "gb_batch_plan_threads", "gb_batch_execute",
                 "gb_batch_execute_loop"):
        fn = getattr(lib, name)
        fn.restype = C.c_int
        fn.argtypes = [C.c_void_p]
    lib.gb_batch_plan_destroy.restype = None
    lib.gb_batch_plan_destroy.argtypes = [C.c_void_p]
