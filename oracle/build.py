"""Build recipe for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Three libraries:

* ``oracle/liboracle_af3d.so``: the plain-C restatement of the reference's
  host step routines (``af3d_oracle.c``).  Built everywhere, including the GPU
  box, because the GPU parity tests and the CPU baseline use it.
* ``oracle/liboracle_tangent.so``: the FP64 tangent-linear model
  (``af3d_tangent.cpp``: the same source compiled as C++ over a dual-number
  type), the forward-mode reference for the engine's adjoint.  Built everywhere.
* ``oracle/_ref/libaf3d_ref.so``: the reference's OWN routines, compiled from
  the unmodified sources where they lie in the read-only reference tree with
  the reference Makefile's flags (``nvcc -c -O2``, MakeAvalancheHst.mk:45-103)
  plus ``-fPIC`` and ``-ffp-contract=off``, linked with ``ref_shim.cu``.  Built
  only where the reference tree exists; used to pin the restatement and to
  generate ``tests/golden/``.  Nothing is copied out of the reference tree.
* ``oracle/_ref/dev/*.cubin``: the reference's OWN device kernels (the ``*_dev``
  twins the reference's GPU driver ``avalanche_dev.cu:636-693`` launches), one
  module per source file, compiled from the same unmodified sources with the
  Makefile's ``-O2`` (MakeAvalancheDev.mk) for sm_103a.  Built only where the
  reference tree exists; the modules travel to the GPU machine, where
  ``oracle/ref_dev.py`` loads them through the CUDA driver and runs the
  reference's device step sequence (a GPU baseline and a parity check of the
  engine against the reference's own kernels).

Run ``python oracle/build.py`` or call :func:`build`.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: AF3D_REFERENCE_DIR, else a directory named "reference" beside this
# repository's root.  Where neither holds the reference's sources, oracle/_ref is not built and
# the tests that need it are skipped.
REFERENCE_DIR = os.environ.get("AF3D_REFERENCE_DIR") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
ORACLE_SO = os.path.join(HERE, "liboracle_af3d.so")
TANGENT_SO = os.path.join(HERE, "liboracle_tangent.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libaf3d_ref.so")

# Reference translation units holding the routines the oracle checks (everything but the two
# drivers avalanche_hst.cu / avalanche_dev.cu and the never-called force_dep.cu).
REF_UNITS = [
    "calculate_particle_parameters", "cells", "cell_dim", "clear_forces", "error_check",
    "finish_Verlet", "force_flume", "force_funnel", "force_hop", "force_part", "force_walls",
    "generate_particles", "get_accel", "init_Verlet", "place_particles", "rannew64",
    "rotate_vectors", "set_initial_velocity",
]


# Reference translation units holding the device kernels of avalanche_dev.cu's step loop.
REF_DEV_UNITS = [
    "init_Verlet", "rotate_vectors", "clear_forces", "cells", "force_hop", "force_funnel", "force_walls",
    "force_part", "force_flume", "get_accel", "finish_Verlet",
]
REF_DEV_DIR = os.path.join(REF_DIR, "dev")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "af3d_oracle.c")
    hdr = os.path.join(HERE, "af3d_oracle.h")
    if force or not _newer(ORACLE_SO, [src, hdr, __file__]):
        tmp = ORACLE_SO + ".tmp%d" % os.getpid()
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp",
              "-o", tmp, src, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_tangent(force: bool = False) -> str:
    src = os.path.join(HERE, "af3d_tangent.cpp")
    deps = [src, os.path.join(HERE, "af3d_oracle.c"), os.path.join(HERE, "af3d_oracle.h"), __file__]
    if force or not _newer(TANGENT_SO, deps):
        tmp = TANGENT_SO + ".tmp%d" % os.getpid()
        _run(["g++", "-O2", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-fvisibility=hidden",
              "-fopenmp", "-o", tmp, src, "-lm"])
        os.replace(tmp, TANGENT_SO)
    return TANGENT_SO


def reference_available() -> bool:
    return all(os.path.exists(os.path.join(REFERENCE_DIR, u + ".cu")) for u in REF_UNITS)


def build_ref(force: bool = False) -> str | None:
    if not reference_available():
        return None
    obj_dir = os.path.join(REF_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    srcs = [os.path.join(REFERENCE_DIR, u + ".cu") for u in REF_UNITS]
    shim = os.path.join(HERE, "ref_shim.cu")
    hdr = os.path.join(REFERENCE_DIR, "cabecera.hu")
    if not force and _newer(REF_SO, srcs + [shim, hdr, __file__]):
        return REF_SO
    flags = ["-O2", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", REFERENCE_DIR]
    jobs = []
    for s in srcs + [shim]:
        o = os.path.join(obj_dir, os.path.splitext(os.path.basename(s))[0] + ".o")
        jobs.append((s, o))
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(lambda so: _run(["nvcc", "-c"] + flags + ["-o", so[1], so[0]]), jobs))
    tmp = REF_SO + ".tmp%d" % os.getpid()
    _run(["nvcc", "-shared", "-o", tmp] + [o for _, o in jobs])
    os.replace(tmp, REF_SO)
    return REF_SO


def build_ref_dev(force: bool = False) -> str | None:
    """The reference's device kernels as cubins (MakeAvalancheDev.mk's ``nvcc -c -O2``, here
    ``-cubin`` for sm_103a), one per source file, into oracle/_ref/dev/."""
    if not reference_available():
        return None
    os.makedirs(REF_DEV_DIR, exist_ok=True)
    hdr = os.path.join(REFERENCE_DIR, "cabecera.hu")
    jobs = []
    for u in REF_DEV_UNITS:
        src = os.path.join(REFERENCE_DIR, u + ".cu")
        out = os.path.join(REF_DEV_DIR, u + ".cubin")
        if force or not _newer(out, [src, hdr, __file__]):
            jobs.append(["nvcc", "-cubin", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", "-I", REFERENCE_DIR,
                         "-o", out, src])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, jobs))
    return REF_DEV_DIR


def build(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        jobs = [ex.submit(build_oracle, force), ex.submit(build_tangent, force)]
        for j in jobs:
            j.result()
    build_ref(force)
    build_ref_dev(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(ORACLE_SO)
    print(TANGENT_SO)
    print(REF_SO if os.path.exists(REF_SO) else "(reference tree absent: _ref not built)")
