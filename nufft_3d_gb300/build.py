"""Builds libnufft3d.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked with the static
CUDA runtime so the library has no run-time dependency beyond the driver.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnufft3d.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
HARNESS_SRC = os.path.join(HERE, "c_harness", "nufft3d_harness.c")
HARNESS = os.path.join(HERE, "c_harness", "nufft3d_harness")
SOURCES = ["plan.cu", "api.cu", "fft.cu", "interp.cu", "tables.cu", "solver.cu", "noalloc.cu", "batch.cu", "tune.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unused-function"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose_ptxas=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "--cudart=static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    if verbose_ptxas:
        for src, (_, log) in zip(SOURCES, results):
            sys.stdout.write("== %s\n%s" % (src, log))
    return LIB


def build_harness(out=HARNESS):
    """Compiles the plain C host (nufft3d_harness.c) against libnufft3d.so."""
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    cmd = [cc, "-std=c99", "-O2", "-Wall", "-Wextra", "-D_DEFAULT_SOURCE", "-I", INCLUDE, HARNESS_SRC, "-o", out,
           "-L", HERE, "-lnufft3d", "-lm", "-Wl,-rpath," + HERE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("harness build failed:\n%s\n%s" % (r.stdout, r.stderr))
    return out


if __name__ == "__main__":
    build(verbose_ptxas="-v" in sys.argv)
    build_harness()
    print(LIB)
