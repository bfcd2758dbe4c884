"""DGETRF pivot vectors from OpenBLAS at the large benchmark sizes.

The matrices are the LU benchmark's: A = uniform(-1, 1) of order N in
{8192, 16384, 32768}, drawn from openblas_gb300.workloads.uniform with seed
7100 + N (the same rule as the 512/1024 pivot cases of gen_golden.py).  Only
the pivot vectors and info are stored (32 KB, 64 KB and 128 KB of int32
before compression); the tests regenerate A on the GPU with the same
counter-based generator.

OpenBLAS here is scipy's bundled build (libscipy_openblas, 0.3.31.dev,
DYNAMIC_ARCH), called through ctypes with the Fortran-77 dgetrf_ ABI.  Its
pivots do not depend on the thread count (partial pivoting with the IAMAX
first-maximum rule of lapack/getf2/getf2_k.c:97-116; the LU values differ in
the last bits between thread counts, the pivots do not).  Run from the
repository root:  python tests/golden/gen_golden_large.py [N ...]
It takes a few minutes on 8 cores and about 3 x 8 GiB of host memory at N =
32768.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from openblas_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "getrf_pivots_large.npz")
SIZES = [8192, 16384, 32768]


def seed_for(n: int) -> int:
    return 7100 + n


def main(sizes):
    from gen_golden import openblas
    ob, cfg = openblas()
    g = {}
    if os.path.exists(OUT):
        with np.load(OUT) as old:
            g.update({k: old[k] for k in old.files})
    g["openblas_config"] = np.array(cfg)
    for n in sizes:
        t0 = time.time()
        A = W.uniform(seed_for(n), (n, n))
        ipiv = np.zeros(n, np.int32)
        info = ob.dgetrf(n, n, A, n, ipiv)
        g[f"piv{n}"] = ipiv
        g[f"info{n}"] = np.int32(info)
        del A
        print(f"N={n}: info={info}, {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e3:.0f} KB) from {cfg}")


if __name__ == "__main__":
    main([int(a) for a in sys.argv[1:]] or SIZES)
