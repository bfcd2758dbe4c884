"""Facts about the sm_103a toolchain that the emulated-FP64 design rests on,
checked by assembling one-instruction inline-PTX kernels with nvcc (no GPU).

The Ozaki scheme is usually written with INT8 slices multiplied exactly by
INT8 tensor-core GEMMs.  On sm_103a the tensor cores' tcgen05.mma has no
INT8 kind: ptxas rejects .kind::i8 for that target (it accepts it for
sm_100a).  The bf16 kind assembles, and bf16 holds integers up to 256
exactly, which is why the emulated DGEMM cuts its operands into 8-bit digits
carried in bf16 with exact FP32 accumulation over 256-deep chunks."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

KERNEL = r"""
#include <stdint.h>
__global__ void k(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
               " tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n}\n"
               :: "r"(d), "l"(a), "l"(b), "r"(id), "r"(acc) : "memory");
}
"""


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    pytest.skip("nvcc not found")


def _assemble(tmp_path, kind, arch):
    src = tmp_path / f"k_{kind}_{arch}.cu"
    src.write_text(KERNEL.replace("KIND", kind))
    r = subprocess.run([_nvcc(), "-c", str(src), "-o", str(src) + ".o", "-gencode",
                        f"arch=compute_{arch},code=sm_{arch}"], capture_output=True, text=True)
    return r.returncode, r.stdout + r.stderr


def test_tcgen05_has_no_int8_kind_on_sm_103a(tmp_path):
    rc, out = _assemble(tmp_path, "i8", "103a")
    assert rc != 0 and "not supported" in out, out
    rc, out = _assemble(tmp_path, "i8", "100a")
    assert rc == 0, out


def test_tcgen05_bf16_kind_assembles_on_sm_103a(tmp_path):
    rc, out = _assemble(tmp_path, "f16", "103a")
    assert rc == 0, out
