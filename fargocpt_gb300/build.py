"""Builds the engine library in-tree: fargocpt_gb300/libfargocpt_gb300.so.

nvcc compiles each CUDA translation unit for sm_103a only
(-gencode arch=compute_103a,code=sm_103a) in parallel, then links a shared
library with the CUDA runtime linked statically, so loading it needs no
CUDA runtime search path.  No PyTorch, no CMake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfargocpt_gb300.so")
SOURCES = ["api.cu", "kernels_fp64.cu", "kernels_pair.cu", "kernels_fp32.cu", "batch_fp32.cu",
           "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "fargocpt_gb300.h"))
    flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH,
             "-Xptxas", "-v"] if verbose else ["-std=c++17", "-O3", "-lineinfo",
                                                "-Xcompiler", "-fPIC", *ARCH]

    def compile_one(src: str) -> str:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        if not force and _newer(o, [s, *headers]):
            return o
        cmd = [nvcc(), "-c", s, "-o", o, *flags]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or not _newer(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB, *objs, *ARCH, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
