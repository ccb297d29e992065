"""Build recipe for the C oracle (test infrastructure only).

Compiles oracle/so4_oracle.c into oracle/_build/libso4oracle.so with gcc and
OpenMP.  -ffp-contract=off keeps every multiply and add separately rounded so
that the oracle gives the same bits on x86_64 and aarch64 hosts.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "so4_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libso4oracle.so")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-Wall", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
