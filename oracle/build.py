"""Build recipe for the oracle shared library (oracle/_ref-free C restatement).

TEST INFRASTRUCTURE ONLY: produces oracle/liborc.so, loaded by the tests,
the smoke check and bench.py's CPU-baseline leg.  Plain gcc, no build system.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "liborc.so")


def build(force=False, verbose=False):
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(SO)
            and os.path.getmtime(SO) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return SO
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=fast", "-fPIC", "-shared",
           "-std=gnu11", "-o", SO + ".tmp", src, "-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(SO + ".tmp", SO)
    return SO


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
