"""Build recipe for libgbblas.so (the product library) with nvcc.

Each translation unit under csrc/ is compiled for sm_103a only, in parallel,
then linked into openblas_gb300/libgbblas.so (in-tree; git-ignored).  No
build system and no PyTorch extension machinery: the library is a plain C
ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(HERE, "libgbblas.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep:
        return obj
    cmd = [nvcc(), "-c", src, "-o", obj + ".tmp", "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
           "-I", os.path.join(ROOT, "include"), "--expt-relaxed-constexpr"] + ARCH
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    if force:
        for f in glob.glob(os.path.join(BUILD, "*.o")):
            os.remove(f)
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if (not force and os.path.exists(SO)
            and os.path.getmtime(SO) >= max(os.path.getmtime(o) for o in objs)):
        return SO
    cmd = [nvcc(), "-shared", "-o", SO + ".tmp"] + objs + ARCH + ["-lcudart", "-ldl"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(SO + ".tmp", SO)
    return SO


PROBES = os.path.join(HERE, "probes")
PROBES_SO = os.path.join(HERE, "libgbprobes.so")


def build_probes(verbose: bool = False) -> str:
    """libgbprobes.so: the peak-rate probes behind ``bench.py --peaks``
    (measurement infrastructure, not part of the BLAS library)."""
    srcs = sorted(glob.glob(os.path.join(PROBES, "*.cu")))
    if os.path.exists(PROBES_SO) and os.path.getmtime(PROBES_SO) >= max(
            os.path.getmtime(f) for f in srcs):
        return PROBES_SO
    cmd = [nvcc(), "-shared", "-o", PROBES_SO + ".tmp", "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC"] + srcs + ARCH + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(PROBES_SO + ".tmp", PROBES_SO)
    return PROBES_SO


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_probes(verbose="-v" in sys.argv))
