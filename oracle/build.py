"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/woo_oracle.cpp into oracle/_build/libwoo_oracle.so with OpenMP and
without floating-point contraction (-ffp-contract=off), so that every FP64 result is
the correctly rounded value of the written operation sequence on x86-64 and aarch64
alike. No host-specific flags (no -march=native).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "woo_oracle.cpp")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwoo_oracle.so")


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "woo_oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    cmd = [os.environ.get("CXX", "g++"), "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB, SRC]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
