"""Build libmlgi.so (CUDA kernels for sm_103a + C ABI + host scene fixture) in-tree.

The library lands in many-lights-gi_gb300/_build/libmlgi.so. Translation units compile in
parallel; the VPL/ISM/pull-push unit is built with -fmad=false so its FP32 arithmetic matches
the reference shaders word for word. build(checked=True) builds the bounds-checked variant
(-DMLGI_CHECKS, csrc/checks.cuh) as _build_checked/libmlgi_checked.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmlgi.so")
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(BUILD_CHECKED, "libmlgi_checked.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
               f"-I{INCLUDE}", f"-I{os.path.join(HERE, 'csrc')}"]
CUDA_UNITS = [
    ("csrc/ism_kernels.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    ("csrc/fg_kernels.cu", []),
    ("csrc/mlgi_api.cu", []),
    ("csrc/ism_static.cu", []),
    ("csrc/scene_kernels.cu", []),
    ("csrc/post_kernels.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    ("csrc/cluster_kernels.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    ("host/serve.cpp", []),
    ("host/autotune.cpp", []),
]
# The scene fixture must be identical on x86 and Arm hosts: no FMA contraction in its double math.
HOST_UNITS = [("host/scene.cpp", ["-O3", "-fopenmp", "-fPIC", "-std=c++17", "-ffp-contract=off", f"-I{INCLUDE}"])]
DEPS = ["csrc/gi_device.cuh", "csrc/kernels.h", "csrc/batch_items.cuh", "csrc/pyramid.cuh", "csrc/checks.cuh",
        "host/room.h"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _sources():
    return list(CUDA_UNITS)


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    paths = [os.path.join(HERE, u) for u, _ in _sources() + HOST_UNITS] + [os.path.join(HERE, d) for d in DEPS]
    paths += [os.path.join(INCLUDE, "mlgi.h"), os.path.abspath(__file__)]
    return any(os.path.exists(p) and os.path.getmtime(p) > t for p in paths)


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    """Compile and link libmlgi.so (checked: libmlgi_checked.so) if any source changed; return its path."""
    lib, bdir = (LIB_CHECKED, BUILD_CHECKED) if checked else (LIB, BUILD)
    if not force and not _stale(lib):
        return lib
    os.makedirs(bdir, exist_ok=True)
    jobs = []
    for unit, flags in _sources():
        src = os.path.join(HERE, unit)
        obj = os.path.join(bdir, os.path.basename(unit) + ".o")
        if checked:
            flags = flags + ["-DMLGI_CHECKS"]
        if unit.endswith(".cu"):
            cmd = [nvcc()] + ARCH + NVCC_COMMON + flags + ["-c", src, "-o", obj]
        else:  # host-side C++ that also holds small kernels: compiled as CUDA
            cmd = [nvcc()] + NVCC_COMMON + flags + ["-x", "cu", "-c", src, "-o", obj] + ARCH
        jobs.append((cmd, obj))
    for unit, flags in HOST_UNITS:
        src = os.path.join(HERE, unit)
        obj = os.path.join(bdir, os.path.basename(unit) + ".o")
        jobs.append((["g++"] + flags + ["-c", src, "-o", obj], obj))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        outs = list(ex.map(lambda j: _run(j[0]), jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    objs = [o for _, o in jobs]
    tmp = lib + ".tmp"
    _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp", "-lpthread"])
    os.replace(tmp, lib)
    return lib


def build_all(force: bool = False) -> tuple[str, str]:
    """Both libraries, built side by side."""
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        normal = ex.submit(build, force)
        checked = ex.submit(build, force, False, True)
        return normal.result(), checked.result()


if __name__ == "__main__":
    if "--all" in sys.argv:
        print(*build_all(force="--force" in sys.argv), sep="\n")
    else:
        print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
