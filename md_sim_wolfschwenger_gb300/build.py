"""Builds the CUDA library libmd_gb300.so (sm_103a) and the drop-in executable.

Every translation unit is compiled in parallel with nvcc / g++ and linked into
md_sim_wolfschwenger_gb300/_lib/.  Portable host flags only (the library is
built on x86 here and on Arm next to the GPU).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libmd_gb300.so")
EXE = os.path.join(OUT, "md_run")

CUDA_SOURCES = ["md_cells.cu", "md_real.cu", "md_kspace.cu", "md_integrate.cu", "md_ctx.cu", "md_batch.cu",
                "md_noalloc.cu", "md_post.cu", "md_ktc.cu",
                "md_place.cu"]
HOST_SOURCES = ["md_host.cpp", "md_serve.cpp", "md_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC,
              "--expt-relaxed-constexpr", "-Wno-deprecated-gpu-targets"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    for p in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "md_gb300.h")]


def _compile(src, verbose=False, ptxas_v=False):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if not _newer(obj, [src] + _headers()):
        return obj
    if src.endswith(".cu"):
        cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_v else []) + ["-c", src, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-I" + cuda_include(), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose or ptxas_v:
        sys.stderr.write(r.stderr)
    return obj


def build(force=False, verbose=False, ptxas_v=False) -> str:
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES + HOST_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, ptxas_v), srcs))
    if _newer(LIB, objs):
        tmp = LIB + f".{os.getpid()}.tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    run_src = os.path.join(CSRC, "md_run.cpp")
    if os.path.exists(run_src) and _newer(EXE, [run_src, LIB] + _headers()):
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-o", EXE, run_src, "-L" + OUT, "-lmd_gb300",
                                                           "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"md_run build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv)
    print(LIB)
