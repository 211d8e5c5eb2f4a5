"""Builds libktruss_gb300.so (and the ktruss CLI) in-tree for sm_103a.

    python ktruss-explorer_gb300/build.py [--force]

CUDA sources are compiled with nvcc -gencode arch=compute_103a,code=sm_103a, host sources
with g++; translation units build in parallel and are skipped when up to date.  Outputs:
    ktruss-explorer_gb300/lib/libktruss_gb300.so
    ktruss-explorer_gb300/bin/ktruss
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
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib", "libktruss_gb300.so")
CLI = os.path.join(PKG, "bin", "ktruss")
COMPAT = os.path.join(PKG, "lib", "libktruss_compat.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr"] + ARCH + os.environ.get("KT_NVCC_FLAGS", "").split()
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]

LIB_SOURCES = ["kt_host.cpp", "kt_gen.cpp", "kt_sort.cu", "kt_build.cu", "kt_support.cu", "kt_peel.cu",
               "kt_engine.cu", "kt_noalloc.cu", "kt_selector.cu", "kt_ingest.cu", "kt_variants.cu"]
CLI_SOURCES = ["ktruss_cli.cpp"]
COMPAT_SOURCES = ["ktruss_compat.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libktruss_gb300")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, force: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if not force and not _stale(obj, [path] + _headers()):
        return obj
    inc = ["-I", INCLUDE, "-I", CSRC]
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + inc + ["-c", path, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + inc + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    srcs = LIB_SOURCES + CLI_SOURCES + COMPAT_SOURCES
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = dict(zip(srcs, ex.map(lambda s: _compile(s, force), srcs)))
    lib_objs = [objs[s] for s in LIB_SOURCES]
    if force or _stale(LIB, lib_objs):
        cmd = [_nvcc(), "-shared"] + ARCH + ["-o", LIB] + lib_objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print("linked", LIB)
    cli_objs = [objs[s] for s in CLI_SOURCES]
    if force or _stale(CLI, cli_objs + [LIB]):
        cmd = [os.environ.get("CXX", "g++"), "-o", CLI] + cli_objs + [
            "-L", os.path.dirname(LIB), "-lktruss_gb300", "-Wl,-rpath,$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print("linked", CLI)
    compat_objs = [objs[s] for s in COMPAT_SOURCES]
    if force or _stale(COMPAT, compat_objs + [LIB]):
        cmd = [os.environ.get("CXX", "g++"), "-shared", "-o", COMPAT] + compat_objs + [
            "-L", os.path.dirname(LIB), "-lktruss_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print("linked", COMPAT)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
