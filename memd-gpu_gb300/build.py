"""Build of libmemd_gb300.so (nvcc, sm_103a only).

Every translation unit compiles in parallel into memd-gpu_gb300/_build/ and is
linked into memd-gpu_gb300/lib/libmemd_gb300.so.  No CMake: a plain list of
nvcc / g++ commands, so the same build runs on the x86 development container
(cross-compiling sm_103a) and on the aarch64 GPU host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libmemd_gb300.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
           f"-I{INCLUDE}", f"-I{CSRC}"] + ARCH
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}",
            "-I/usr/local/cuda/include"]

CU_SOURCES = ["memd_api.cu", "memd_directions.cu", "memd_diag.cu"]
CXX_SOURCES = ["memd_synth.cpp"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith((".h", ".hpp"))]
    return hs


def _nvcc() -> str:
    n = shutil.which("nvcc")
    if n:
        return n
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra_deps: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if _newer(obj, [src] + extra_deps):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVFLAGS + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-c", src, "-o", obj]
    subprocess.check_call(cmd)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _headers()
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CXX_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=max(2, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, deps), srcs))
    if not _newer(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.check_call(cmd)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
