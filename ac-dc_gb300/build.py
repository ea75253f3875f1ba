"""Builds the native libraries of the GB300 PCDM package in-tree.

  lib/libacdc_gpu.so   CUDA kernels + C-ABI (nvcc, sm_103a only)
  lib/libacdc_host.so  generators and loaders (g++, OpenMP)
  lib/acdc_solver      drop-in console solver (the MultiCoreSolver CLI on the GPU engine)

Each translation unit is compiled in parallel; outputs are rebuilt only when a
source or header is newer.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
CPP = os.path.join(PKG, "cpp")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fopenmp", "-I" + INCLUDE, "-I" + CSRC]
GXX_FLAGS = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c++17", "-I" + INCLUDE,
             "-I" + CSRC]

GPU_LIB = os.path.join(LIBDIR, "libacdc_gpu.so")
HOST_LIB = os.path.join(LIBDIR, "libacdc_host.so")
SOLVER_BIN = os.path.join(LIBDIR, "acdc_solver")


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libacdc_gpu.so")


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(INCLUDE, "*.h")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build_gpu(verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    objs, jobs = [], []
    for src in sources:
        obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out:
                print(out)
    if _stale(GPU_LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", GPU_LIB] + objs + ["-ldl", "-Xcompiler", "-fopenmp"])
    return GPU_LIB


def build_host():
    os.makedirs(LIBDIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "host_*.cpp")))
    if _stale(HOST_LIB, sources + _headers()):
        _run(["g++"] + GXX_FLAGS + ["-shared", "-o", HOST_LIB] + sources)
    return HOST_LIB


def build_solver():
    """The drop-in console solver (C++ engine over libacdc_gpu.so)."""
    main = os.path.join(CPP, "acdc_solver_main.cpp")
    if not os.path.exists(main):
        return None
    deps = [main] + glob.glob(os.path.join(CPP, "**", "*.h"), recursive=True) + _headers()
    if _stale(SOLVER_BIN, deps + [GPU_LIB, HOST_LIB]):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, "-I" + CPP, main, "-o", SOLVER_BIN,
              "-L" + LIBDIR, "-lacdc_gpu", "-lacdc_host", "-Wl,-rpath,$ORIGIN", "-fopenmp"])
    return SOLVER_BIN


def build_all(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        fg = ex.submit(build_gpu, verbose)
        fh = ex.submit(build_host)
        fg.result()
        fh.result()
    build_solver()


if __name__ == "__main__":
    build_all(verbose=True)
    print("built", GPU_LIB, HOST_LIB)
