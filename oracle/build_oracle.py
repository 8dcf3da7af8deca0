"""Build recipe of the CPU oracle (test infrastructure only).

Compiles ``oracle/mps_oracle.cpp`` (2D) and ``oracle/mps_oracle3.cpp`` (3D) twice into
``oracle/_build/``:

* ``libmps_oracle.so``      serial, ``-O2 -ffp-contract=off``: the parity oracle;
* ``libmps_oracle_omp.so``  ``-O3 -fopenmp -ffp-contract=off``: the timed CPU baseline.

The reference itself (OpenMps, header-only C++) cannot be compiled here: it needs
Boost (uBLAS, multi_array, property_tree, format) and the ViennaCL submodule,
which are absent, so there is no ``oracle/_ref`` build.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRCS = [os.path.join(HERE, "mps_oracle.cpp"), os.path.join(HERE, "mps_oracle3.cpp")]

VARIANTS = {
    "libmps_oracle.so": ["-O2", "-ffp-contract=off"],
    "libmps_oracle_omp.so": ["-O3", "-ffp-contract=off", "-fopenmp"],
}


def _needs_build(out: str) -> bool:
    if not os.path.exists(out):
        return True
    mtime = os.path.getmtime(out)
    deps = [*SRCS, os.path.join(HERE, "mps_oracle.h"), os.path.join(HERE, "..", "include", "mps.h")]
    return any(os.path.getmtime(d) > mtime for d in deps)


def _compile(name: str, flags: list[str]) -> str:
    out = os.path.join(BUILD, name)
    if not _needs_build(out):
        return out
    tmp = out + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++17", "-shared", "-fPIC", "-Wall", "-Wextra", *flags, *SRCS, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


def build(verbose: bool = False) -> dict[str, str]:
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(VARIANTS)) as ex:
        futs = {name: ex.submit(_compile, name, flags) for name, flags in VARIANTS.items()}
        outs = {name: f.result() for name, f in futs.items()}
    if verbose:
        for k, v in outs.items():
            print("built", k, "->", v)
    return outs


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
