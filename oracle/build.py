"""Build recipe for the oracle shared library (test infrastructure only).

Compiles the CPU restatement in this directory into ``oracle/_build/liboracle.so``.
``-ffp-contract=off`` keeps every multiply and add separately rounded, as Rust
does, so the oracle's arithmetic matches the reference bit for bit.
The flags are portable: the same recipe builds on x86-64 and on Arm hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCES = ["ordering.cpp", "solvers.cpp", "circuit.cpp", "bbd.cpp", "ac.cpp", "transient.cpp",
           "capi.cpp"]
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES] + [os.path.join(HERE, "oracle.h")]
    if not force and os.path.exists(LIB):
        mt = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= mt for s in srcs):
            return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-pthread", "-o", LIB + ".tmp"]
    cmd += [os.path.join(HERE, s) for s in SOURCES]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
