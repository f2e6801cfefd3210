"""Build the engine's shared library in-tree: ``avalancheflume3d_gb300/libaf3d.so``.

CUDA translation units are compiled for sm_103a only.  The step kernels are compiled with
``-fmad=false`` so that no multiply-add is contracted and every force, torque and
acceleration is bit-identical to the reference's FP64 arithmetic; the host I/O unit is
compiled with ``-ffp-contract=off`` for the same reason.  The CUDA runtime is linked
statically, so the library loads without a CUDA toolkit on the library path.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libaf3d.so")
PROGRAM = os.path.join(PKG, "af3d_avalanche")
OBJ = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
# Extra nvcc flags for tuning sweeps (e.g. AF3D_NVCC_FLAGS="-DAF3D_FORCES_MINB=4").
COMMON += os.environ.get("AF3D_NVCC_FLAGS", "").split()

# (source, object name, extra flags).  The step kernels are built twice: exact (no contraction,
# the reference's operation order) and the fast FP64 mode (-DAF3D_FAST, contracted multiply-adds).
UNITS = [
    ("af3d_kernels.cu", "af3d_kernels", ["-fmad=false", "-Xptxas", "-v"]),
    ("af3d_kernels.cu", "af3d_kernels_fast", ["-fmad=true", "-DAF3D_FAST", "-Xptxas", "-v"]),
    ("af3d_adjoint.cu", "af3d_adjoint", ["-fmad=false"]),
    ("af3d_adjoint_rot.cu", "af3d_adjoint_rot", ["-fmad=true"]),
    ("af3d_cells.cu", "af3d_cells", []),
    ("af3d_capi.cu", "af3d_capi", []),
    ("af3d_peaks.cu", "af3d_peaks", []),
]
HOST_UNITS = [("af3d_hostio.cpp", "af3d_hostio", ["-O2", "-ffp-contract=off"])]

HEADERS = ["af3d_internal.h", "af3d_physics.cuh", "af3d_cellwalk.cuh", "af3d_adjoint.cuh"]


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "af3d.h"), __file__]
    jobs = []
    for src, obj, extra in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, obj + ".o")
        if force or _stale(o, [s] + hdrs):
            jobs.append([NVCC, "-c"] + ARCH + COMMON + extra + ["-o", o, s])
    for src, obj, extra in HOST_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, obj + ".o")
        if force or _stale(o, [s] + hdrs):
            jobs.append(["g++", "-c", "-std=c++17", "-fPIC", "-I", INCLUDE] + extra + ["-o", o, s])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 2))) as ex:
            logs = list(ex.map(_run, jobs))
    objs = [os.path.join(OBJ, obj + ".o") for _, obj, _ in UNITS + HOST_UNITS]
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([NVCC, "-shared"] + ARCH + ["-o", tmp] + objs)
        os.replace(tmp, LIB)
    # the reference's simulation program over the C ABI, linked against the library beside it
    src = os.path.join(CSRC, "af3d_avalanche.cpp")
    if force or _stale(PROGRAM, [src, LIB, os.path.join(INCLUDE, "af3d.h")]):
        tmp = PROGRAM + ".tmp%d" % os.getpid()
        _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, "-o", tmp, src, "-L" + PKG, "-laf3d",
              "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, PROGRAM)
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
