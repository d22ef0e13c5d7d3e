"""Builds libbs2e.so (the C-ABI CUDA library) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel into _build/, then linked
into libbs2e.so next to this file.  Also builds the CPU oracle (a test
fixture) when asked.  Usage: python build.py [--oracle]
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbs2e.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
SOURCES = ["bs2e_capi.cu", "bs2e_radial.cu", "bs2e_assembly.cu", "bs2e_dipole.cu",
           "bs2e_noalloc.cu", "bs2e_angular.cpp", "bs2e_basis.cpp", "bs2e_fortio.cpp",
           "bs2e_spmv.cu", "bs2e_batch.cu", "bs2e_blockcsr.cu", "bs2e_bands.cpp"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-Xcompiler", "-fvisibility=hidden", "-I" + os.path.join(HERE, "..", "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    cmd = [_nvcc(), ARCH, "-lineinfo", *COMMON, "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [_nvcc(), *COMMON, "-x", "c++", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    hdr = os.path.join(HERE, "..", "include", "bs2e.h")
    return os.path.getmtime(hdr) > t


def build(force=False):
    """Compiles libbs2e.so if any source is newer than it; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


DRIVER_SRC = os.path.join(HERE, "..", "tests", "capi_driver.c")
DRIVER = os.path.join(HERE, "..", "tests", "_build", "capi_driver")


def build_driver():
    """Compiles the plain-C caller of include/bs2e.h (tests/capi_driver.c)
    with the host C compiler, strict C11 with warnings as errors, linked
    against libbs2e.so: the header's declarations meet a C compiler and every
    entry point it calls must resolve in the library."""
    os.makedirs(os.path.dirname(DRIVER), exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-O1",
           "-I" + os.path.join(HERE, "..", "include"), DRIVER_SRC, "-L" + HERE, "-lbs2e",
           "-Wl,-rpath," + HERE, "-o", DRIVER]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("C driver build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return DRIVER


def build_oracle():
    """Builds the CPU oracle shared library (test infrastructure) with make."""
    odir = os.path.join(HERE, "..", "oracle")
    r = subprocess.run(["make", "-C", odir], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return os.path.join(odir, "liboracle.so")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    if "--oracle" in sys.argv:
        print(build_oracle())
