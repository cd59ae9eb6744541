"""Builds libcrt_gb300.so in-tree for sm_103a.

    python -m cudart_gb300.build [-v]

Each .cu file is one nvcc invocation (run in parallel); host-only C++ goes
through g++.  Everything is compiled with -fmad=false / -ffp-contract=off:
the kernels must round every multiply and add separately to match the
reference's host arithmetic bit for bit (the traversal's slab tests use
explicit fmaf()).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcrt_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["scene.cu", "trace.cu", "render.cu", "wavefront.cu", "tune.cu", "bvh_gpu.cu"]
CPP_SOURCES = ["bvh8.cpp", "ingest.cpp"]

NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true",
                     "-prec-sqrt=true", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-O2,-ffp-contract=off,-fvisibility=hidden"]
CXX_FLAGS = ["-O3", "-fPIC", "-std=c++17", "-ffp-contract=off", "-pthread", "-fvisibility=hidden"]


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"build step failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout}")
    if verbose and p.stdout.strip():
        print(p.stdout, flush=True)
    return p.stdout


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


CLI_SRC = os.path.join(HERE, "cli", "crt_render.cpp")
CLI = os.path.join(HERE, "crt_render")


def _build_cli(cxx: str, verbose: bool) -> None:
    """The command-line renderer, linked against the in-tree library."""
    if not _stale(CLI, [CLI_SRC, LIB, os.path.join(HERE, "..", "include", "crt_gb300.h")]):
        return
    tmp = CLI + ".tmp"
    _run([cxx, "-O2", "-std=c++17", CLI_SRC, "-o", tmp, "-L" + HERE, "-lcrt_gb300",
          "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath-link,{CUDA_HOME}/lib64"], verbose)
    os.replace(tmp, CLI)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every CUDA/C++ source of the library and link the .so."""
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "crt_gb300.h"))
    jobs, objs = [], []
    for f in CU_SOURCES:
        src, obj = os.path.join(SRC, f), os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([NVCC] + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    cxx = shutil.which("g++") or "g++"
    for f in CPP_SOURCES:
        src, obj = os.path.join(SRC, f), os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([cxx] + CXX_FLAGS + ["-c", src, "-o", obj])
    outputs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(lambda c: _run(c, verbose), jobs):
            outputs.append(out)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _run([NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs +
             ["-Xlinker", f"-rpath,{CUDA_HOME}/lib64", "-lpthread"], verbose)
        os.replace(tmp, LIB)
    _build_cli(cxx, verbose)
    if ptxas_info:
        print("\n".join(outputs))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
