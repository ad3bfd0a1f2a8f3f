"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/ucl_oracle.c into oracle/liboracle.so with gcc.  The tests
check the GPU path against it; nothing in the product links it.
``-ffp-contract=off`` keeps results independent of FMA contraction so the
same inputs give the same bits on the x86 build host and the Arm GPU host.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "ucl_oracle.c")
OUT = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", OUT + ".tmp", "-lm", "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
