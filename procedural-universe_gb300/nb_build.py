"""Builds libnbody_gb300.so in-tree with nvcc for sm_103a.

Each translation unit under csrc/ is compiled in parallel into _build/, then
linked into a shared library next to this file.  No torch, no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnbody_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    # host code: no contraction into fused multiply-adds, so that host results
    # (seeders, file re-centring) are the same on x86-64 and AArch64
    cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-Xcompiler", "-ffp-contract=off",
           "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
    if verbose_ptxas and src.endswith(".cu"):
        cmd[1:1] = ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    if not force and not verbose_ptxas and up_to_date():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    srcs = _sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = LIB + ".tmp.%d" % os.getpid()
    cmd = [NVCC, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


DRIVER_SRC = os.path.join(HERE, "driver", "nbody_driver.cpp")
DRIVER = os.path.join(HERE, "nbody_driver")


def build_driver(force: bool = False) -> str:
    """Builds the headless precompute driver against libnbody_gb300.so."""
    build()
    deps = [DRIVER_SRC, LIB, os.path.join(INCLUDE, "cuda_nbody_sim.hpp"), os.path.join(INCLUDE, "nbody_gb300.h")]
    if not force and os.path.exists(DRIVER) and all(os.path.getmtime(d) <= os.path.getmtime(DRIVER) for d in deps):
        return DRIVER
    tmp = DRIVER + ".tmp.%d" % os.getpid()
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I", INCLUDE, DRIVER_SRC, "-o", tmp,
           "-L", HERE, "-lnbody_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
    print(build_driver(force="--force" in sys.argv))
