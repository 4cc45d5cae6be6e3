"""Build the native libraries in-tree.

  libmpcd_gpu.so  CUDA kernels + C ABI (include/*.h), sm_103a only
  cilia           drop-in executable `cilia sim.cfg` (host C++ over the C ABI)

Translation units compile in parallel; outputs land next to this file
(`_build/`).  Usage: python build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", CSRC, "-I", os.path.join(REPO, "include")] + ARCH
CU_SOURCES = ["fluid_kernels.cu", "md_kernels.cu", "md_df.cu", "md_pair.cu", "md_cluster.cu", "md_plan.cu", "engine.cu", "static_step.cu",
              "batch_kernels.cu", "batch.cu"]
HOST_SOURCES = ["host/libconfig_lite.cpp", "host/objects.cpp", "host/cilia_capi.cpp", "host/server.cpp"]
CXX = os.environ.get("CXX", "g++")
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-pthread", "-I", os.path.join(CSRC, "host"), "-I", os.path.join(REPO, "include")]

LIB = os.path.join(OUT, "libmpcd_gpu.so")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = []
    for root, _, files in os.walk(CSRC):
        hs += [os.path.join(root, f) for f in files if f.endswith((".h", ".cuh", ".hpp"))]
    inc = os.path.join(REPO, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _compile(src, force):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if force or _newer(obj, [src] + _headers()):
        cmd = [NVCC] + NVFLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def _compile_host(src, force):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if force or _newer(obj, [src] + _headers()):
        r = subprocess.run([CXX] + CXXFLAGS + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {src}:\n{r.stderr}")
    return obj


EXE = os.path.join(OUT, "cilia")


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cu = [os.path.join(CSRC, s) for s in CU_SOURCES]
    host = [os.path.join(CSRC, s) for s in HOST_SOURCES]
    main = os.path.join(CSRC, "host", "main.cpp")
    with cf.ThreadPoolExecutor(max_workers=len(cu) + len(host) + 1) as ex:
        fut_cu = [ex.submit(_compile, s, force) for s in cu]
        fut_host = [ex.submit(_compile_host, s, force) for s in host + [main]]
        objs = [f.result() for f in fut_cu] + [f.result() for f in fut_host[:-1]]
        main_obj = fut_host[-1].result()
    if force or _newer(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    if force or _newer(EXE, [LIB, main_obj]):
        cmd = [CXX, "-pthread", "-o", EXE, main_obj, "-L", OUT, "-lmpcd_gpu", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of cilia failed:\n{r.stderr}")
    if verbose:
        print("built", LIB, "and", EXE)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
