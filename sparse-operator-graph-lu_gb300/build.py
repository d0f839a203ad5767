"""Build recipe for the in-tree native library and CLI (no cmake).

Produces, inside this package directory:
  lib/libsoglu_gb300.so   host planner + sm_103a executor behind the C ABI
  bin/solve               the `./solve file.mtx` command line front end
Host C++ is compiled with g++ (portable flags only: the same sources build on
x86-64 and aarch64); CUDA sources with nvcc for sm_103a only.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libsoglu_gb300.so")
CLI = os.path.join(PKG, "bin", "solve")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SRC = ["order.cpp", "planner.cpp", "mtx.cpp", "tasks.cpp", "batch.cpp", "plan_api.cpp", "runtime.cpp", "server.cpp"]
CUDA_SRC = ["factor.cu", "factor_f64.cu", "factor_f32_s1.cu", "factor_f32_s2.cu", "solve.cu"]
HEADERS = ["plan.h", "tasks.h", "kernels.h", "api_internal.h", "factor_impl.cuh", "factor_units.h", "tc_gemm.cuh"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function", f"-I{CUDA}/include",
            f"-I{ROOT}/include"]
NVFLAGS = ["-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC", f"-I{ROOT}/include"]


def _cuda_libdir() -> str:
    for d in ("lib64", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib", "lib"):
        p = os.path.join(CUDA, d)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(CUDA, "lib64")


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile (incrementally) and return the path of libsoglu_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "soglu_gb300.h")]
    steps = []
    objs = []
    for s in HOST_SRC:
        src, obj = os.path.join(CSRC, s), os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append(["g++", *CXXFLAGS, "-c", src, "-o", obj])
    for s in CUDA_SRC:
        src, obj = os.path.join(CSRC, s), os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append([NVCC, *NVFLAGS, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for cmd in steps:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, steps))
    libdir = _cuda_libdir()
    if _stale(LIB, objs):
        _run(["g++", "-shared", "-o", LIB, *objs, f"-L{libdir}", "-lcudart", "-fopenmp", "-pthread",
              f"-Wl,-rpath,{libdir}"])
    cli_src = os.path.join(CSRC, "solve_main.cpp")
    if _stale(CLI, [cli_src, LIB] + hdrs):
        _run(["g++", *CXXFLAGS, cli_src, "-o", CLI, f"-L{os.path.dirname(LIB)}", "-lsoglu_gb300",
              f"-Wl,-rpath,{os.path.dirname(LIB)}", f"-L{libdir}", "-lcudart", f"-Wl,-rpath,{libdir}"])
    return LIB


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    for p in (LIB, CLI):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    if "clean" in sys.argv:
        clean()
    print(build(verbose="-v" in sys.argv))
