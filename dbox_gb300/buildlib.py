"""Build libdbox_gpu.so (the C-ABI GPU library) for sm_103a, in-tree.

Flags that matter for parity with the reference's float32 arithmetic:
  --fmad=false          no fused multiply-add contraction in device code
  -prec-div/-prec-sqrt  IEEE round-to-nearest division and square root
  -ftz=false            keep denormals
  -ffp-contract=off     same for the host-side creation code
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdbox_gpu.so")
SOURCES = [os.path.join(CSRC, "step.cu"), os.path.join(CSRC, "api.cu"), os.path.join(CSRC, "mlp.cu"),
           os.path.join(CSRC, "query.cu")]
HEADERS = [os.path.join(CSRC, n) for n in os.listdir(CSRC) if n.endswith((".h", ".cuh"))] + [
    os.path.join(HERE, "..", "include", "dbox_gpu.h")]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-lineinfo",
              "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "--expt-relaxed-constexpr"]


def nvcc():
    for cand in ("/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand == "nvcc" or os.path.exists(cand):
            return cand
    return "nvcc"


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SOURCES + HEADERS)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    objs = []
    procs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd), cmd))
        objs.append(obj)
    for p, cmd in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    link = [nvcc(), ARCH, "-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
    subprocess.check_call(link)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
