"""Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

FP32 bit-exactness needs the reference's operation order without fused multiply-adds, hence
-ffp-contract=off and no fast-math. OpenMP threads the timed FP32 baseline.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-fexcess-precision=standard", "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "glsl.hpp")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["g++"] + FLAGS + [srcs[0], "-o", tmp]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
