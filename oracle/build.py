"""Build recipe for the oracle (test infrastructure only).

Compiles ``oracle/glassman_oracle.c`` -- the CPU restatement of the reference's
generic FFT backend -- into ``oracle/_build/liboracle.so``.  The reference
itself (Fortran + MPI) cannot be compiled in this environment: there is no
Fortran compiler and no MPI, so no ``oracle/_ref`` build exists.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "glassman_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", "-fPIC", "-shared", SRC, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
