"""The seeded input generators: the torch form (used to build the large LU
and DGESV matrices on the GPU) gives the numpy form's numbers bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from openblas_gb300 import workloads as W


@pytest.mark.parametrize("seed,shape,chunk", [
    (7, (37, 11), 97),               # chunk boundaries inside columns
    (7100 + 8192, (300,), 64),       # the large-LU seeds, vector form
    (12345, (1000, 3), 1 << 26),
    (2**31 + 5, (65, 65), 1000),     # seed * 2^32 wraps modulo 2^64
])
def test_uniform_device_matches_numpy(seed, shape, chunk):
    torch = pytest.importorskip("torch")
    a = W.uniform(seed, shape)
    t = W.uniform_device(seed, shape, device="cpu", chunk=chunk)
    assert t.dtype == torch.float64
    b = t.numpy().T if len(shape) == 2 else t.numpy()
    assert np.array_equal(a, b)


def test_uniform_device_range():
    pytest.importorskip("torch")
    a = W.uniform(5, (64, 64), 0.0, 1.0)
    b = W.uniform_device(5, (64, 64), "cpu", 0.0, 1.0).numpy().T
    assert np.array_equal(a, b)
    assert b.min() >= 0.0 and b.max() < 1.0
