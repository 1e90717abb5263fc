"""Build recipes for the native parts of the package.

Compiles, in parallel and in-tree:
  * the CUDA library ``_lib/libbruno_gb300.so`` (sm_103a, ``nvcc`` only, no CMake);
  * the host-only synthetic-read generator ``_lib/libbruno_synth.so``;
  * the C++ driver ``_lib/compact_dbg_gb300`` (same flags and outputs as the reference's
    compact_dbg_freq_construct_clean).
Portable flags only, so the same recipe builds on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "_lib")
REPO = os.path.dirname(PKG)
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
CUDA_SOURCES = ["build.cu", "chain.cu", "capi.cu", "pool.cu"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build_library(force: bool = False) -> str:
    """Compiles the CUDA library; returns the path of the shared object."""
    os.makedirs(os.path.join(LIB, "obj"), exist_ok=True)
    out = os.path.join(LIB, "libbruno_gb300.so")
    headers = [os.path.join(CSRC, h) for h in ("kmer.cuh", "internal.cuh", "piece_cuts.h", "pool_admission.h")] + [os.path.join(INCLUDE, "bruno_gb300.h")]
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES]
    if not force and _newer(out, srcs + headers):
        return out
    nvcc = _nvcc()
    objs = [os.path.join(LIB, "obj", os.path.splitext(s)[0] + ".o") for s in CUDA_SOURCES]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        list(ex.map(_run, [[nvcc, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o] for s, o in zip(srcs, objs)]))
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", out, *objs])
    return out


def build_synth(force: bool = False) -> str:
    out = os.path.join(LIB, "libbruno_synth.so")
    src = os.path.join(CSRC, "synth.cpp")
    os.makedirs(LIB, exist_ok=True)
    if force or not _newer(out, [src]):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-o", out, src, "-lpthread"])
    return out


def build_driver(force: bool = False) -> str:
    out = os.path.join(LIB, "compact_dbg_gb300")
    src = os.path.join(CSRC, "compact_dbg_main.cpp")
    hdrs = [os.path.join(INCLUDE, "bruno_gb300.h"), os.path.join(INCLUDE, "bruno_gb300.hpp")]
    lib = os.path.join(LIB, "libbruno_gb300.so")
    if not os.path.exists(src):
        return ""
    if force or not _newer(out, [src, lib, *hdrs]):
        _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, "-o", out, src, "-L", LIB, "-lbruno_gb300",
              f"-Wl,-rpath,{LIB}", "-Wl,-rpath,$ORIGIN"])
    return out


def build_all(force: bool = False) -> None:
    build_library(force)
    build_synth(force)
    build_driver(force)


if __name__ == "__main__":
    build_all(force=True)
    print("built", LIB)
