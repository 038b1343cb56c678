"""In-tree build of the native libraries.

* ``robast_gb300/_build/librobast_gb.so`` -- the product: scene flattener,
  ray sources, CUDA kernels for sm_103a and the C ABI of include/robast_gb.h.
* ``oracle/_build/liboracle.so`` -- the CPU FP64 oracle used by the tests
  and by bench.py's CPU baseline (test infrastructure, not the product).

Translation units compile in parallel; nvcc cross-compiles without a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "robast_gb300")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["trace_fp64.cu", "trace_mixed_all.cu", "trace_mixed_facets.cu", "trace_mixed_coated.cu",
              "trace_mixed_cones.cu", "trace_mixed_csg.cu", "capi.cu", "trace_mixed.cu", "adjoint.cu", "noalloc.cu",
              "corsika_rays.cu", "ray_order.cu", "tmm.cu", "psf.cu", "fma_peak.cu", "shoot.cu", "trace_count.cu"]
CPP_SOURCES = ["scene.cpp", "shoot.cpp", "corsika.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    out = os.path.join(BUILD, "librobast_gb.so")
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES]
    if not force and not _stale(out, srcs + _headers()):
        return out
    common = ["-I", INCLUDE, "-I", CSRC]
    jobs = []
    for f in CU_SOURCES:
        obj = os.path.join(BUILD, f + ".o")
        cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-c",
               os.path.join(CSRC, f), "-o", obj, *common]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        jobs.append((obj, cmd))
    for f in CPP_SOURCES:
        obj = os.path.join(BUILD, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", os.path.join(CSRC, f), "-o", obj, *common]
        jobs.append((obj, cmd))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(2, min(16, os.cpu_count() or 2))) as ex:
        for log in ex.map(lambda j: _run(j[1]), jobs):
            logs.append(log)
    tmp = out + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *[j[0] for j in jobs]])
    os.replace(tmp, out)
    if verbose:
        sys.stdout.write("".join(logs))
    return out


def build_oracle(force: bool = False) -> str:
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    out = os.path.join(ORACLE_BUILD, "liboracle.so")
    src = os.path.join(ORACLE, "oracle.c")
    if not force and not _stale(out, [src, os.path.join(ORACLE, "oracle.h")] + _headers()):
        return out
    tmp = out + ".tmp"
    # -ffp-contract=off: the same rounding on x86-64 and aarch64 hosts
    _run(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-ffp-contract=off", "-I", INCLUDE, src,
          "-o", tmp, "-lm", "-lpthread"])
    os.replace(tmp, out)
    return out


def build_all(verbose: bool = False) -> None:
    build_library(verbose=verbose)
    build_oracle()


if __name__ == "__main__":
    build_library(verbose="-v" in sys.argv, force="-f" in sys.argv)
    build_oracle(force="-f" in sys.argv)
    print("built")
