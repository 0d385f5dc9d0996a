"""Build libwenofd.so (CUDA kernels + C ABI) and the `wenofd` driver for sm_103a.

    python fd-weno-eulerequation_gb300/build.py [--force] [--verbose-ptxas] [--bounds-check]

Compiles every translation unit in parallel, skipping objects newer than
their sources, into fd-weno-eulerequation_gb300/_build/.  --bounds-check
builds the debug library instead, with -DWENOFD_BOUNDS_CHECK (every kernel's
index guards on, csrc/guard.cuh), into fd-weno-eulerequation_gb300/_build_check/.  The FP64 parity
units are compiled with -fmad=false; host C++ with -ffp-contract=off so the
initial conditions round like the reference's.  The FP32-arithmetic units
(FP32 and learned forms, not bitwise by design) take the hardware square-root
approximation (-prec-sqrt=false), the indicator also approximate division.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
OUT_CHECK = os.path.join(PKG, "_build_check")
ROOT = os.path.dirname(PKG)
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + os.path.join(CUDA_HOME, "include"),
             "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

# translation unit -> extra flags
CUDA_UNITS = {
    "stage_fp64.cu": ["-fmad=false"],
    "stage_fp32.cu": ["-prec-sqrt=false"],
    "aux_kernels.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "learned_data.cu": ["-fmad=false"],
    "learned.cu": ["-prec-sqrt=false", "-prec-div=false"],
    "batch_fp64.cu": ["-fmad=false"],
    "batch_fp32.cu": ["-prec-sqrt=false"],
    "batch_learned.cu": ["-prec-sqrt=false"],
}
CXX_UNITS = ["capi.cpp", "cases.cpp", "batch.cpp"]

LIB = os.path.join(OUT, "libwenofd.so")
LIB_CHECK = os.path.join(OUT_CHECK, "libwenofd.so")
EXE = os.path.join(OUT, "wenofd")
TRAIN_EXE = os.path.join(OUT, "wenofd_train")


def _deps() -> list[str]:
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "wenofd.h"), os.path.abspath(__file__)]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + _deps())


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def build_pipe_peaks() -> str:
    """Opt-in measurement tool (not part of the library): FP64/FP32 pipe and
    host-link peaks, fd-weno-eulerequation_gb300/_build/pipe_peaks."""
    os.makedirs(OUT, exist_ok=True)
    probe = os.path.join(OUT, "pipe_peaks")
    _run([NVCC] + ARCH + ["-O3", "-std=c++17", os.path.join(PKG, "tools", "pipe_peaks.cu"), "-o", probe])
    return probe


def _build_lib(out_dir: str, lib: str, defines: list[str], force: bool, verbose_ptxas: bool) -> str:
    os.makedirs(out_dir, exist_ok=True)
    jobs = []
    objs = []
    for unit, extra in CUDA_UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(out_dir, unit + ".o")
        objs.append(obj)
        if force or verbose_ptxas or _stale(obj, src):
            cmd = [NVCC] + ARCH + NVCC_FLAGS + defines + extra + ["-c", src, "-o", obj]
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    cxx = shutil.which(os.environ.get("CXX", "g++")) or "g++"
    for unit in CXX_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(out_dir, unit + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            jobs.append([cxx] + CXX_FLAGS + defines + ["-c", src, "-o", obj])
    log = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            log.append(out)
    if jobs or not os.path.exists(lib):
        lib_dir = os.path.join(CUDA_HOME, "lib64")
        _run([NVCC] + ARCH + ["-shared", "-cudart", "shared", "-Xlinker", "-rpath," + lib_dir] + objs + ["-o", lib])
    return "".join(log)


def build_checked(force: bool = False) -> str:
    """The bounds-checked debug library (index guards on), _build_check/libwenofd.so."""
    _build_lib(OUT_CHECK, LIB_CHECK, ["-DWENOFD_BOUNDS_CHECK"], force, False)
    return LIB_CHECK


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    log = [_build_lib(OUT, LIB, [], force, verbose_ptxas)]
    cxx = shutil.which(os.environ.get("CXX", "g++")) or "g++"
    host_srcs = [os.path.join(HOST, f) for f in ("WENOFD.cpp", "main.cpp")]
    if all(os.path.exists(p) for p in host_srcs) and (force or not os.path.exists(EXE) or any(
            os.path.getmtime(p) > os.path.getmtime(EXE) for p in host_srcs + [LIB, os.path.join(HOST, "WENOFD.hpp")])):
        _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-I" + os.path.join(ROOT, "include"),
              "-I" + HOST] + host_srcs + ["-L" + OUT, "-lwenofd", "-Wl,-rpath,$ORIGIN", "-o", EXE])
    # the indicator's C-ABI training driver (no Python involved)
    train_src = os.path.join(HOST, "train_indicator.cpp")
    if force or not os.path.exists(TRAIN_EXE) or any(
            os.path.getmtime(p) > os.path.getmtime(TRAIN_EXE) for p in (train_src, LIB)):
        lib_dir = os.path.join(CUDA_HOME, "lib64")
        _run([cxx, "-O2", "-std=c++17", "-Wall", "-I" + os.path.join(ROOT, "include"),
              "-I" + os.path.join(CUDA_HOME, "include"), train_src, "-L" + OUT, "-lwenofd", "-L" + lib_dir,
              "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + lib_dir, "-o", TRAIN_EXE])
    return "".join(log)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    ap.add_argument("--pipe-peaks", action="store_true", help="also build the pipe/link peak measurement tool")
    ap.add_argument("--bounds-check", action="store_true", help="build the index-guarded debug library instead")
    a = ap.parse_args()
    if a.pipe_peaks:
        print(build_pipe_peaks())
    if a.bounds_check:
        print(build_checked(a.force))
        sys.exit(0)
    out = build(a.force, a.verbose_ptxas)
    if out.strip():
        sys.stdout.write(out)
    print(LIB)
