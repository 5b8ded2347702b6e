"""Builds libdvm_gpu.so (the C-ABI GPU library) in-tree for sm_103a.

    python 2d_dvm_microflows_gb300/build.py

Each .cu translation unit is compiled in parallel with nvcc, then linked into a shared
library next to this file. The C++ host driver (host/dvm_host.cpp) is built against it.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdvm_gpu.so")
HOST = os.path.join(HERE, "dvm_host")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
SOURCES = ["dvm_kernels.cu", "dvm_api.cu", "dvm_noalloc.cu", "dvm_server.cu", "dvm_vis.cpp"]
# the output writer restates the reference's FP64 sums operation by operation: no contraction
# into fused multiply-adds (the host compiler's default on aarch64)
EXTRA = {"dvm_vis.cpp": ["-Xcompiler", "-ffp-contract=off"]}


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + NVFLAGS + EXTRA.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(_compile, SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    host_src = os.path.join(HERE, "host", "dvm_host.cpp")
    if os.path.exists(host_src):
        cxx = shutil.which("g++") or "g++"
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
        # the initial states restate the reference's FP64 operations: no fused multiply-adds
        cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(REPO, "include"),
               "-I", cuda_inc,
               host_src, "-o", HOST, "-L", HERE, "-ldvm_gpu", "-Wl,-rpath,$ORIGIN", "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("host driver build failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
