"""Build recipe for the C++ oracle shared library (test infrastructure).

g++ -O3 -ffp-contract=off: Rust never fuses a*b+c, and aarch64 GCC would
otherwise contract to FMA by default, silently breaking bit-exact parity.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "librforacle.so")
SRCS = [os.path.join(HERE, "rf_oracle.cpp")]
FLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
         "-fPIC", "-shared", "-Wall", "-Wextra"]


def build(force=False):
    """Compile oracle/_build/librforacle.so if missing or stale; return path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = SRCS + [os.path.join(HERE, "rf_oracle.h"), __file__]
    if not force and os.path.exists(LIB):
        mt = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= mt for d in deps):
            return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++"] + FLAGS + SRCS + ["-o", tmp])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
