"""Build recipe of the CPU oracle (test infrastructure only).

Compiles oracle/woo_oracle.cpp twice:
* oracle/_build/libwoo_oracle.so, the parity build: OpenMP and no floating-point contraction
  (-ffp-contract=off), so that every FP64 result is the correctly rounded value of the written
  operation sequence on x86-64 and aarch64 alike;
* oracle/_build/libwoo_oracle_fast.so, the timing build of the CPU baseline: OpenMP, -O3 with
  fused multiply-adds allowed (-ffp-contract=fast) and no errno handling in the math calls
  (-fno-math-errno), the flags a release build of a CPU code uses.
Neither uses host-specific code generation (-march/-mcpu=native): the same source builds on
the x86-64 and aarch64 machines that run it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "woo_oracle.cpp")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libwoo_oracle.so")
LIB_FAST = os.path.join(OUT, "libwoo_oracle_fast.so")
FLAGS = {LIB: ["-O3", "-ffp-contract=off"], LIB_FAST: ["-O3", "-ffp-contract=fast", "-fno-math-errno"]}


def build(force=False, verbose=False):
    """Build both libraries (in parallel) if stale; returns the parity build's path."""
    os.makedirs(OUT, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "woo_oracle.h")]
    procs = []
    for lib, flags in FLAGS.items():
        if not force and os.path.exists(lib) and all(os.path.getmtime(d) <= os.path.getmtime(lib) for d in deps):
            continue
        cmd = [os.environ.get("CXX", "g++")] + flags + ["-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", lib, SRC]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    for p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + out.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
