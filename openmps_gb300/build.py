"""In-tree build of ``libopenmps_gb300.so`` for sm_103a (GB300).

Each CUDA translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo`` and linked into
``openmps_gb300/libopenmps_gb300.so``.  The per-particle stage kernels
(``grid.cu``, ``stages.cu``, ``dim3.cu``) are compiled with ``-fmad=false`` so that every
floating-point operation rounds like the reference's FP64 CPU path; the solver
(``cg.cu``) uses fused multiply-adds.  Host code never contracts either
(``-ffp-contract=off``), so x86 and Arm hosts compute the same constants.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libopenmps_gb300.so")
DRIVER_SRC = os.path.join(HERE, "driver", "main.cpp")
DRIVER = os.path.join(HERE, "openmps_gb300_main")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-Xcompiler", "-Wall", "-I", INCLUDE]
UNITS = {
    "grid.cu": ["-fmad=false"],
    "stages.cu": ["-fmad=false"],
    "dim3.cu": ["-fmad=false"],
    "cg.cu": [],
    "mg.cu": [],
    "learned.cu": [],
    "batch.cu": [],
    "scan.cu": [],
    "noalloc.cu": [],
    "mps_abi.cu": [],
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libopenmps_gb300.so")
    return path


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    return files + [os.path.join(INCLUDE, "mps.h")]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str, extra: list[str], verbose_ptxas: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    if not _stale(obj, _deps()):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj + ".tmp"]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), res.stderr))
    if verbose_ptxas and res.stderr:
        sys.stderr.write(res.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose_ptxas: bool = False, force: bool = False) -> str:
    """Compiles and links the library if any source changed; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, u, flags, verbose_ptxas) for u, flags in UNITS.items()]
        objs = [f.result() for f in futs]
    if _stale(LIB, objs) or force:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
        os.replace(tmp, LIB)
    build_driver(force)
    return LIB


def build_driver(force: bool = False) -> str:
    """The command-line driver (reference XML/CSV in, CSV out) linked to the library."""
    deps = [DRIVER_SRC, LIB, os.path.join(INCLUDE, "mps.h"), os.path.join(INCLUDE, "openmps_gb300.hpp")]
    if not force and not _stale(DRIVER, deps):
        return DRIVER
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the driver")
    tmp = DRIVER + ".tmp%d" % os.getpid()
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-ffp-contract=off", "-I", INCLUDE, DRIVER_SRC, "-o", tmp,
           "-L", HERE, "-lopenmps_gb300", "-Wl,-rpath,$ORIGIN"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("driver build failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv))
