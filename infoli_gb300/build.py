"""Build the native parts in-tree (no cmake, no pip):

  infoli_gb300/_build/libinfoli_gpu.so   C ABI + CUDA kernels (sm_103a)
  infoli_gb300/_build/infoli.x           reference-compatible CLI (C host code)
  infoli_gb300/_build/infoli_kat.x       same, regression-test build
                                          (the reference's -DG_CAL_FROM_FILE / omp_test)

Translation units compile in parallel; CUDA code is compiled for sm_103a only.
Usage: python -m infoli_gb300.build   (or infoli_gb300.build.build()).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["infoli_kernels.cu", "infoli_capi.cu", "infoli_static.cu", "infoli_batch.cu", "infoli_serve.cu",
              "infoli_init.cu"]
CXX_SOURCES = ["infoli_planner.cpp"]
C_SOURCES = ["infoli_host.c", "infoli_trace.c"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libinfoli_gpu.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile everything; returns the path of libinfoli_gpu.so."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INC, "infoli_gpu.h"))
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
                         "-I", INC, "-c", src, "-o", obj])
    for f in CXX_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-fopenmp", "-I", INC, "-c", src, "-o", obj])
    for f in C_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["gcc", "-O3", "-std=gnu11", "-fPIC", "-Wall", "-fopenmp", "-I", INC,
                         "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    lib = os.path.join(OUT, "libinfoli_gpu.so")
    if force or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", lib, *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    # reference-compatible CLI, linked against the library (rpath $ORIGIN)
    main_c = os.path.join(HOST, "infoli_main.c")
    for exe, extra in (("infoli.x", []), ("infoli_kat.x", ["-DG_CAL_FROM_FILE"])):
        target = os.path.join(OUT, exe)
        if force or _stale(target, [main_c, lib, os.path.join(INC, "infoli_gpu.h")]):
            _run(["gcc", "-O2", "-std=gnu11", "-Wall", *extra, "-I", INC, main_c, "-L", OUT,
                  "-linfoli_gpu", "-Wl,-rpath,$ORIGIN", "-lm", "-o", target])
    # infoli.x reads default.conf from its own directory, like the reference
    conf_src = os.path.join(HOST, "default.conf")
    conf_dst = os.path.join(OUT, "default.conf")
    if force or _stale(conf_dst, [conf_src]):
        shutil.copyfile(conf_src, conf_dst)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
