"""Build recipe of libtealeaf_gb300.so and the tea_leaf executable.

Every CUDA translation unit is compiled for GB300 only
(-gencode arch=compute_103a,code=sm_103a) and in parallel; host C++ units with
g++.  Outputs go to tealeaf_cuda_gb300/_build/ (git-ignored).  Objects are
rebuilt when a source or any header of the package is newer.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libtealeaf_gb300.so")
EXE = os.path.join(OUT, "tea_leaf")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["tl_kernels.cu", "tl_chunk.cu", "tl_solve.cu", "tl_legacy.cu", "tl_mixed.cu",
              "tl_noalloc.cu", "tl_conv.cu", "tl_warm.cu"]
CPP_SOURCES = ["tl_deck.cpp", "tl_driver.cpp", "tl_host_numerics.cpp"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
             "-I" + INCLUDE, "-I" + os.path.join(CUDA_HOME, "include")]


def _headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "tealeaf_capi.h"))
    return hs


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stdout + p.stderr


def build(verbose=False, ptxas_info=False):
    """Compile everything that is out of date; returns the library path."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(OUT, exist_ok=True)
    deps = _headers()
    jobs = []
    for f in CU_SOURCES:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        if _stale(obj, src, deps) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([NVCC] + GENCODE + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    for f in CPP_SOURCES:
        src, obj = os.path.join(SRC, f), os.path.join(OUT, f + ".o")
        if _stale(obj, src, deps):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    objs = [os.path.join(OUT, f + ".o") for f in CU_SOURCES + CPP_SOURCES]
    if jobs or not os.path.exists(LIB):
        _run([NVCC] + GENCODE + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    main = os.path.join(SRC, "tea_leaf_main.cpp")
    if jobs or not os.path.exists(EXE) or _stale(EXE, main, deps):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, main, "-o", EXE, "-L" + OUT,
              "-ltealeaf_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


def clean():
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
