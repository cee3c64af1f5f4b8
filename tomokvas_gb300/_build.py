"""In-tree build of the GB300 CUDA library (libtk_fdk.so) with nvcc.

Every translation unit is compiled for sm_103a only, in parallel, then
linked into one shared library next to the package.  No cmake, no
torch extension machinery: the library has a plain C ABI (include/tk_fdk.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libtk_fdk.so")
SOURCES = ["tk_capi.cu", "tk_filter.cu", "tk_bp.cu", "tk_batch.cu", "tk_phantom.cu", "tk_noalloc.cu", "tk_rebin.cu", "tk_diag.cu", "tk_toeplitz.cu", "tk_refine.cu"]
HEADERS = ["tk_common.cuh", "tk_internal.h", "tk_bp_core.cuh", "tk_filter_core.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CLI_SRC = os.path.join(PKG, "cli", "tk_para_tc.cpp")
CLI = os.path.join(LIB_DIR, "tk_para_tc")


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtk_fdk.so")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                   "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")] + list(extra)


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "tk_fdk.h")]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + _flags(extra_flags) + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode != 0:
                print(" ".join(cmd))
                print(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print(" ".join(cmd))
            print(r.stdout + r.stderr)
            raise RuntimeError("linking libtk_fdk.so failed")
        os.replace(tmp, LIB)
    build_cli(force)
    return LIB


def build_cli(force: bool = False) -> str:
    """The para_TC-equivalent driver (host C++ over libtk_fdk.so): lib/tk_para_tc."""
    deps = [CLI_SRC, LIB] + [os.path.join(ROOT, "include", h) for h in ("tk_fdk.h", "tk_fdk.hpp", "tk_io.hpp")]
    if not (force or _stale(CLI, deps)):
        return CLI
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "include")
    tmp = CLI + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, CLI_SRC,
           "-o", tmp, "-L", LIB_DIR, "-ltk_fdk", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print(" ".join(cmd))
        print(r.stdout + r.stderr)
        raise RuntimeError("building tk_para_tc failed")
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
