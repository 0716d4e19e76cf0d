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
# the same library with the index checks of MEMD_CHECKED compiled in (tests)
LIB_CHECKED = os.path.join(LIBDIR, "libmemd_gb300_checked.so")
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


def _compile(src: str, extra_deps: list[str], checked: bool = False) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + (".checked.o" if checked else ".o"))
    if _newer(obj, [src] + extra_deps):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVFLAGS + (["-DMEMD_CHECKED"] if checked else []) + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-c", src, "-o", obj]
    subprocess.check_call(cmd)
    return obj


EXAMPLES = ["sample_synthetic_signal", "memd_cli", "memd_sweep"]
BINDIR = os.path.join(PKG, "bin")
MEX_STUB_DIR = os.path.join(REPO, "tests", "mex_stub")
MEX_STUB_LIB = os.path.join(LIBDIR, "libmemd_mex_stub.so")


def _cuda_lib_dir() -> str:
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return "/usr/local/cuda/lib64"


def _link_host(out: str, srcs: list[str], extra_inc: list[str], shared: bool) -> None:
    deps = srcs + _headers() + [LIB]
    for d in extra_inc:
        for root, _, files in os.walk(d):
            deps += [os.path.join(root, f) for f in files if f.endswith(".h")]
    if _newer(out, deps):
        return
    cmd = ["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", "-I/usr/local/cuda/include"]
    cmd += [f"-I{d}" for d in extra_inc]
    if shared:
        cmd += ["-fPIC", "-shared"]
    cmd += ["-o", out] + srcs + [f"-L{LIBDIR}", "-lmemd_gb300", f"-L{_cuda_lib_dir()}", "-lcudart",
                                 f"-Wl,-rpath,{LIBDIR}", f"-Wl,-rpath,{_cuda_lib_dir()}"]
    subprocess.check_call(cmd)


def build_host_tools() -> None:
    """The reference-style example driver, the .bin CLI and (for the tests)
    the MEX entry linked against the stub of the mex/mxGPU API."""
    os.makedirs(BINDIR, exist_ok=True)
    for name in EXAMPLES:
        _link_host(os.path.join(BINDIR, name), [os.path.join(PKG, "examples", name + ".cpp")], [], False)
    _link_host(MEX_STUB_LIB, [os.path.join(PKG, "mex", "memd_mex.cpp"), os.path.join(MEX_STUB_DIR, "mex_stub.cpp")],
               [MEX_STUB_DIR], True)


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _headers()
    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES + CXX_SOURCES]
    api = os.path.join(CSRC, "memd_api.cu")
    jobs = [(s_, False) for s_ in srcs] + [(api, True)]
    with cf.ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        built = list(ex.map(lambda j: _compile(j[0], deps, j[1]), jobs))
    objs, api_checked = built[:-1], built[-1]
    if not _newer(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.check_call(cmd)
    objs_checked = [api_checked if o.endswith("memd_api.cu.o") else o for o in objs]
    if not _newer(LIB_CHECKED, objs_checked):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB_CHECKED] + objs_checked + ["-lcudart"]
        subprocess.check_call(cmd)
    build_host_tools()
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
