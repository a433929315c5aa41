"""ORACLE build recipe — test infrastructure only.

Compiles oracle/rr_oracle.c (the plain-C FP64 restatement of the RoadRunner
path) into oracle/_build/librr_oracle.so with gcc and OpenMP.  The flags keep
IEEE semantics (-ffp-contract=off, no fast-math) so the oracle follows the
reference's rounding on both x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "rr_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "librr_oracle.so")


def build(force: bool = False) -> str:
    """Build the oracle shared library if it is missing or stale; return its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-std=c11", "-D_GNU_SOURCE", SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
