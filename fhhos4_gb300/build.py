"""Build recipe of libfhg.so (CUDA kernels + C ABI) for sm_103a, in-tree.

``python -m fhhos4_gb300.build`` or ``fhhos4_gb300.build.build()``. nvcc only (no cmake):
the translation units compile in parallel, then link into fhhos4_gb300/_build/libfhg.so.
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
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libfhg.so")
HHO_LIB = os.path.join(OUT_DIR, "libfhg_hho.so")
SOURCES = ["fhg_kernels.cu", "fhg_kernels_pair.cu", "fhg_coarse.cu", "fhg_api.cu", "fhg_noalloc.cu", "fhg_learned.cu", "fhg_post.cu", "fhg_condense.cu"]
HHO_SOURCES = ["hho_gen.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfhg")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *_flags(), *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, flush=True)
        return obj

    def build_hho():
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        tmp = HHO_LIB + ".tmp"
        cmd = [cxx, "-std=c++17", "-O3", "-fPIC", "-shared", "-w", "-o", tmp,
               *[os.path.join(CSRC, s) for s in HHO_SOURCES], "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host generator build failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, HHO_LIB)

    with cf.ThreadPoolExecutor(len(SOURCES) + 1) as ex:
        hho = ex.submit(build_hho)
        objs = list(ex.map(compile_one, SOURCES))
        hho.result()
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
