"""In-tree build of ``libradisgb.so`` (CUDA kernels + C ABI) for sm_103a.

``python -m radis_gb300._build`` or ``radis_gb300._build.build()``.  Uses nvcc
directly (no CMake, no torch extension machinery); translation units are
compiled in parallel and linked against the shared CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
BUILD = os.path.join(os.path.dirname(PKG), "_build")
LIB = os.path.join(PKG, "libradisgb.so")
SOURCES = ["rg_kernels.cu", "rg_api.cu", "rg_hull.cpp", "rg_skeleton.cpp", "rg_partition.cpp", "rg_hitran.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libradisgb.so")
    return cand


def _deps():
    files = [os.path.join(CSRC, s) for s in SOURCES]
    files += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    files.append(os.path.join(INCLUDE, "radis_gb300.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]

    def compile_one(src):
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc, *common, *ARCH, "-lineinfo", "-c", path, "-o", obj]
            if ptxas_v:
                cmd.insert(1, "-Xptxas=-v")
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_v:
        for obj, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, "-cudart", "shared", "-o", tmp, *[o for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv))
