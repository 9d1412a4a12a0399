"""Build libgpuai.so (CUDA kernels + C ABI) and the host tools for sm_103a.

Everything is compiled in-tree with nvcc/g++ directly (no cmake):

  gpu_ai_gb300/lib/libgpuai.so   kernels + C ABI (include/gpuai.h)
  gpu_ai_gb300/lib/run_ai        the run_ai driver (playout/game tests, players)
  gpu_ai_gb300/lib/libgpuai_checked.so  (build(checks=True)) the same library with
                                 the kernels' bounds checks compiled in
                                 (-DGPUAI_CHECKS): a failed check skips the
                                 access and sets a status bit, reported as
                                 GPUAI_ERR_LIMIT; load it with GPUAI_LIB=<path>

Translation units are compiled in parallel; a unit is rebuilt only when one of
its inputs is newer than its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(CSRC, "host")
LIB = os.path.join(PKG, "lib")
OBJ = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "-I" + INCLUDE, "-I" + CSRC] + ARCH
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-pthread", "-I" + INCLUDE, "-I" + CSRC]

CUDA_UNITS = ["kernels.cu", "capi.cu", "noalloc.cu", "search.cu", "net.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers(d: str):
    return [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".hpp", ".cuh"))]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _host_units():
    if not os.path.isdir(HOST):
        return []
    return sorted(f for f in os.listdir(HOST) if f.endswith(".cpp") and f != "run_ai.cpp")


def build(verbose: bool = False, checks: bool = False) -> str:
    """Compile libgpuai.so (and run_ai when the host sources exist); return the
    .so path.  checks=True builds libgpuai_checked.so instead: the same code
    with the kernels' bounds checks (-DGPUAI_CHECKS)."""
    os.makedirs(LIB, exist_ok=True)
    obj_dir = OBJ + ("_checked" if checks else "")
    os.makedirs(obj_dir, exist_ok=True)
    extra = ["-DGPUAI_CHECKS"] if checks else []
    hdrs = _headers(CSRC) + _headers(INCLUDE) + (_headers(HOST) if os.path.isdir(HOST) else [])
    jobs = []
    objs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(obj_dir, u + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs + [__file__]):
            jobs.append([nvcc()] + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    host_objs = []
    for u in _host_units():
        src = os.path.join(HOST, u)
        obj = os.path.join(obj_dir, u + ".o")
        host_objs.append(obj)
        if _stale(obj, [src] + hdrs + [__file__]):
            jobs.append(["g++"] + CXX_FLAGS + extra + ["-c", src, "-o", obj])
    run_ai_src = os.path.join(HOST, "run_ai.cpp")
    run_ai_obj = os.path.join(OBJ, "run_ai.cpp.o")
    if not checks and os.path.exists(run_ai_src) and _stale(run_ai_obj, [run_ai_src] + hdrs + [__file__]):
        jobs.append(["g++"] + CXX_FLAGS + ["-c", run_ai_src, "-o", run_ai_obj])
    with ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    so = os.path.join(LIB, "libgpuai_checked.so" if checks else "libgpuai.so")
    all_objs = objs + host_objs
    if _stale(so, all_objs):
        _run([nvcc(), "-shared", "-Xcompiler", "-fPIC"] + ARCH + ["-o", so] + all_objs + ["-lpthread"], verbose)
    if checks:
        return so
    if os.path.exists(run_ai_src):
        exe = os.path.join(LIB, "run_ai")
        if _stale(exe, [run_ai_obj, so]):
            _run(["g++", "-o", exe, run_ai_obj, "-L" + LIB, "-lgpuai", "-Wl,-rpath,$ORIGIN", "-pthread"], verbose)
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, checks="--checks" in sys.argv))
