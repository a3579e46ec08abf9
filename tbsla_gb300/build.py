"""Build recipe of the native library (no CMake): every CUDA translation unit
compiled for sm_103a with nvcc, the host C++ with g++, in parallel, linked
into ``tbsla_gb300/libtbsla_gb300.so`` (the C ABI of ``include/tbsla_gb300.h``)
and ``tbsla_gb300/libtbsla.so`` (the C++ drop-in classes ``tbsla::cpp::Matrix*``
on top of it).  Objects go to ``tbsla_gb300/_build/``.  Rebuilds only what
changed.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtbsla_gb300.so")
CPPLIB = os.path.join(PKG, "libtbsla.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tbsla_gb300")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "**", "*.h*"), recursive=True) +
            glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True) +
            glob.glob(os.path.join(ROOT, "include", "*.h")) +
            glob.glob(os.path.join(PKG, "cpp", "include", "**", "*.hpp"), recursive=True))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, hdr: list[str], verbose: bool) -> str:
    rel = os.path.relpath(src, PKG).replace(os.sep, "_")
    obj = os.path.join(BUILD, rel + ".o")
    if not _stale(obj, [src, os.path.abspath(__file__)] + hdr):
        return obj
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC,
           "-I", os.path.join(PKG, "cpp", "include")]
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--extended-lambda",
               "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", *inc, "-c", src, "-o", obj]
        if os.environ.get("TBSLA_PTXAS_VERBOSE"):
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
               "-I", os.path.join(_cuda_home(), "include"), *inc, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{res.stdout}\n{res.stderr}")
    if res.stderr.strip() and verbose:
        print(res.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    core = sorted(glob.glob(os.path.join(CSRC, "**", "*.cu"), recursive=True) +
                  glob.glob(os.path.join(CSRC, "**", "*.cpp"), recursive=True))
    cpp = sorted(glob.glob(os.path.join(PKG, "cpp", "src", "*.cpp")))
    hdr = _headers()
    jobs = min(len(core) + len(cpp), max(2, os.cpu_count() or 2))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        core_objs = list(ex.map(lambda s: _compile(s, hdr, verbose), core))
        cpp_objs = list(ex.map(lambda s: _compile(s, hdr, verbose), cpp))
    if _stale(LIB, core_objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *core_objs, "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    if cpp_objs and _stale(CPPLIB, cpp_objs + [LIB]):
        cmd = ["g++", "-shared", "-o", CPPLIB, *cpp_objs, "-L", PKG, "-ltbsla_gb300",
               "-Wl,-rpath,$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
