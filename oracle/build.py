"""Build recipe for the oracle (test infrastructure; see clm_oracle.c header).

    python oracle/build.py        -> oracle/build/libclmoracle.so

Plain gcc, -O2 -ffp-contract=off (no fused multiply-add, as in the Float64
reference), OpenMP over columns.  Portable C: builds the same on x86_64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "build")
LIB = os.path.join(OUT_DIR, "libclmoracle.so")


def build(force=False, verbose=False):
    src = os.path.join(HERE, "clm_oracle.c")
    csrc = os.path.join(HERE, "..", "clm.jl_gb300", "csrc")
    deps = [src, os.path.join(HERE, "..", "include", "clmgb.h"), os.path.join(csrc, "clm_math.h"),
            os.path.join(csrc, "clm_math_tables.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(d) for d in deps)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-std=c11", "-Wall", "-Wno-unused-function", src, "-o", tmp, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
