"""Build recipe for libwoogpu.so (in-tree, sm_103a only).

Each .cu translation unit is compiled in parallel with nvcc and linked into
woodem_gb300/libwoogpu.so. The FP64 translation units are compiled with
--fmad=false (no contraction of a*b+c), so their results are the correctly
rounded values of the operation sequences written in the source.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwoogpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code of the library (cell matrices, contact listing) is also compiled without contraction
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-diag-suppress", "177,550"]
# translation unit -> extra flags
UNITS = {
    "wg_step.cu": ["--fmad=false"],
    "wg_collide.cu": ["--fmad=false"],
    "wg_api.cu": ["--fmad=false"],
    "wg_step32.cu": ["--fmad=true", "-Xcompiler", "-ffp-contract=fast"],
    "wg_noalloc.cu": ["--fmad=false"],
    "wg_pack.cpp": [],
    "wg_pack_gpu.cu": ["--fmad=false"],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "woo_gpu.h"))
    headers.append(os.path.abspath(__file__))  # the flags below
    procs = []
    objs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        if not os.path.exists(src):
            continue
        obj = os.path.join(OUT, unit.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((unit, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join("%s:\n%s" % f for f in failed))
    if force or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
