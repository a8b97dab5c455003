"""Build libkgr.so (the CUDA kernels and the C ABI of include/kgr.h) in-tree.

    python -m artemis_gb300.build          # or artemis_gb300.build.build()

Every CUDA translation unit is compiled for sm_103a only, with FMA
contraction off (-fmad=false) and IEEE division and square root, so that the
kernels round exactly like the CPU restatement they are checked against.
Host C++ is compiled with -ffp-contract=off for the same reason.
Objects go to artemis_gb300/_build/, the library to artemis_gb300/lib/.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libkgr.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-Xptxas", "-O3",
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
             "-Wno-unused-function"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + \
        [os.path.join(ROOT, "include", "kgr.h")]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + _headers())


def _compile(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, ptxas_info=False):
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu, cpp = sources()
    inc = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(home, "include")]
    jobs, objs = [], []
    for f in cu:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, src) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc] + ARCH + CUDA_FLAGS + extra + inc + ["-c", src, "-o", obj])
    for f in cpp:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _stale(obj, src):
            jobs.append([os.environ.get("CXX", "g++")] + CXX_FLAGS + inc + ["-c", src, "-o", obj])
    outputs = []
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outputs = list(ex.map(_compile, jobs))
    if jobs or not os.path.exists(LIB):
        link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
        _compile(link)
    if verbose:
        for o in outputs:
            if o.strip():
                print(o)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
